// relax_host.cu -- launch planning (shared-memory layout, workspace sizing)
// and dispatch of the node-relaxation kernels over the objective / LMO kinds.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "relax.cuh"

namespace gbx {

template <int OK, int LK>
int launch_one(const Params& p, cudaStream_t st, std::string* err);
template <int LK>
int probe_one(const gbx_lmo& l, const Layout& L, int cases, int mode, const double* dir, const double* x,
              const double* lb, const double* ub, double* out, double* out_step, cudaStream_t st,
              std::string* err);
template <int LK>
int feas_one(const gbx_lmo& l, const Layout& L, int cases, const double* lb, const double* ub,
             const uint8_t* flags, uint8_t* out, cudaStream_t st, std::string* err);

namespace {
int next_pow2(int v) { int r = 1; while (r < v) r <<= 1; return r; }
constexpr size_t kSmemBudget = 220 * 1024;
constexpr size_t kSmemPerSm = 228 * 1024;        // shared memory of an SM
constexpr size_t kSmemPerCtaReserve = 2 * 1024;  // per-CTA reserve and the kernels' static shared memory
}

int make_layout(const gbx_objective& o, const gbx_lmo& l, const gbx_algorithm& a,
                int n_nodes, Layout* out, std::string* err, const Variant* var) {
    (void)n_nodes;
    const Variant v = var ? *var : tuned_variant(o, l, a);
    Layout L{};
    L.persistent = v.persistent == 1 ? 1 : 0;
    const int n = o.n;
    for (int& v : L.off) v = -1;
    const bool dicg = a.kind == GBX_ALG_DICG;
    const bool secant = a.line_search == GBX_LS_SECANT;
    const bool mixed = a.precision == GBX_PRECISION_MIXED;
    if (mixed) {
        if (o.kind != GBX_OBJ_GRAPH_MATCHING || l.kind != GBX_LMO_BIRKHOFF) {
            *err = "mixed precision covers the graph-matching objective over the Birkhoff polytope";
            return GBX_ERR_UNSUPPORTED;
        }
        if (secant) {
            *err = "the secant line search is not available in mixed precision";
            return GBX_ERR_UNSUPPORTED;
        }
    }
    // which node vectors exist
    bool need[B_COUNT] = {};
    need[B_X] = need[B_G] = need[B_V] = need[B_LB] = need[B_UB] = true;
    need[B_AW] = dicg && !mixed;
    need[B_TX] = need[B_TG] = secant;
    need[B_R] = o.kind == GBX_OBJ_GRAPH_MATCHING;
    need[B_CAND] = !secant;  // with the secant search the candidate reuses the trial point
    int cnt = 0;
    for (int b = 0; b < B_COUNT; ++b) cnt += need[b];
    L.nvec = cnt;

    size_t fixed_bytes = 0;
    if (l.kind == GBX_LMO_SIMPLEX || l.kind == GBX_LMO_EQUALITY_SIMPLEX) {
        if (n > 8192) { *err = "simplex LMO supports n <= 8192"; return GBX_ERR_UNSUPPORTED; }
        L.sort_size = next_pow2(n);
        fixed_bytes += align16((size_t)L.sort_size * 8) * 2 + align16((size_t)L.sort_size * 4)
                       + align16((size_t)n);
    }
    if (l.kind == GBX_LMO_CARDINALITY) {
        if (n % 2 || n > 8192) { *err = "cardinality LMO needs n = 2 * assets <= 8192"; return GBX_ERR_UNSUPPORTED; }
        // ranks (in the key array), sorted order and prefix sums of the free z-costs
        L.sort_size = next_pow2(n / 2 + 1);
        fixed_bytes += align16((size_t)L.sort_size * 8) * 2 + align16((size_t)L.sort_size * 4)
                       + align16((size_t)n);
    }
    if (l.kind == GBX_LMO_LINKED_CARDINALITY) {
        if (n % 2 || l.order < 0 || l.order > n / 2) {
            *err = "linked cardinality LMO needs n = 2 * (padded) assets and 0 <= order <= n / 2";
            return GBX_ERR_UNSUPPORTED;
        }
    }
    if (l.kind == GBX_LMO_BIRKHOFF) {
        if (l.order <= 0 || l.order > 1024) { *err = "Birkhoff order out of range"; return GBX_ERR_UNSUPPORTED; }
        L.hung_order = l.order;
        L.hung_warps = 2;
        L.hung_bytes = hung_ws_bytes(l.order);
        fixed_bytes += 2 * L.hung_bytes;
    }
    L.mixed = mixed ? 1 : 0;
    size_t mx_bytes = 0, cost_bytes = 0, code_bytes = 0;
    if (mixed) {
        if (l.order > 512) {
            *err = "mixed precision supports Birkhoff orders up to 512";
            return GBX_ERR_UNSUPPORTED;
        }
        mx_bytes = mixed_array_bytes(n);
        // forward and in-face integer costs
        cost_bytes = align16(2 * (size_t)n * sizeof(int));
        // the FP32 SIMT gradient keeps its arrays in shared memory up to order ~90
        // (above, in the workspace, over the nonzero lists of sparse graphs); the
        // tensor-core gradient pads any order up to 128
        const bool tc_ok = l.order > 16 && l.order <= 128;
        L.tc = tc_ok && (v.tc == 1 || (v.tc < 0 && l.order > 64)) ? 1 : 0;
        if (L.tc) cost_bytes = std::max(cost_bytes, kTcOperandBytes);
        const size_t staged = std::max(cost_bytes, align16((size_t)n * sizeof(double)));  // + certificate costs
        code_bytes = align16((size_t)n);   // edge codes and the iterate's face bits
        L.ihw_bytes = ihw_bytes(l.order);
        // large orders: the oracle costs and edge codes move to the node's workspace
        // (every order above 128: the large-order kernel then holds the only
        // 8- and 16-column integer Hungarians)
        L.cost_global = !L.tc && (l.order > 128 || fixed_bytes + staged + code_bytes + 2 * L.ihw_bytes > kSmemBudget)
                            ? 1 : 0;
        // The SIMT kernel holds up to two nodes per SM (its register limit). Of
        // the cost-region layouts -- both oracles' costs with the certificate's
        // gradient staged beside them, without staging, the in-face costs
        // derived from the forward ones (staged or not) -- take the first that
        // reaches the most nodes per SM (order 120: derived, not staged).
        L.cert_stage = 1;
        L.derive_inface = 0;
        if (!L.tc && !L.cost_global && l.order > 64) {
            auto per_sm = [&](size_t bytes) {
                return std::min<int>(2, (int)(kSmemPerSm / (bytes + kSmemPerCtaReserve)));
            };
            const size_t base = fixed_bytes + code_bytes + 2 * L.ihw_bytes;
            const size_t one = align16((size_t)n * sizeof(int)), dbl = align16((size_t)n * sizeof(double));
            const size_t opts[4][3] = {{std::max(cost_bytes, dbl), 1, 0}, {cost_bytes, 0, 0},
                                       {std::max(one, dbl), 1, 1}, {one, 0, 1}};
            // the FP32 arrays join shared memory whenever they fit (placement below)
            auto total = [&](size_t costs) {
                return base + costs + (mx_bytes + base + costs > kSmemBudget ? 0 : mx_bytes);
            };
            int best = 0;
            for (int q = 0; q < 4; ++q) best = std::max(best, per_sm(total(opts[q][0])));
            for (int q = 0; q < 4; ++q)
                if (per_sm(total(opts[q][0])) == best) {
                    cost_bytes = opts[q][0];
                    L.cert_stage = (int)opts[q][1];
                    L.derive_inface = (int)opts[q][2];
                    break;
                }
        } else {
            cost_bytes = staged;
        }
        fixed_bytes += (L.cost_global ? 0 : cost_bytes + code_bytes) + 2 * L.ihw_bytes;
        if (L.cost_global) {
            // large orders: only the certificate's forward oracle runs in FP64
            // (one workspace), and the integer oracles' column state moves to
            // shared memory (below) -- two nodes per SM
            L.hung_warps = 1;
            fixed_bytes -= L.hung_bytes;
        }
    }
    size_t obj_doubles = o.kind == GBX_OBJ_GRAPH_MATCHING ? 2 * (size_t)o.order * o.order
                                                          : (size_t)n * n;
    const size_t obj_bytes = align16(obj_doubles * sizeof(double));
    L.obj_doubles = obj_doubles;
    if (fixed_bytes > kSmemBudget) { *err = "LMO workspace exceeds shared memory"; return GBX_ERR_UNSUPPORTED; }
    // Placement. The mixed loop touches only x and the bounds among the FP64
    // vectors, so those stay in shared memory and the certificate's vectors and
    // the FP64 objective matrices go to the workspace (two nodes per SM fit).
    // The FP64 path keeps everything in shared memory when it fits.
    bool smem[B_COUNT] = {};
    const size_t vec_all = align16((size_t)cnt * n * sizeof(double));
    if (mixed) {
        // the FP32 arrays go to the workspace when they do not fit beside
        // the oracle costs (orders above ~90); x and the bounds follow them
        L.obj_smem = 0;
        L.mx_global = (L.tc || L.cost_global || mx_bytes + fixed_bytes > kSmemBudget) ? 1 : 0;
        if (!L.mx_global) fixed_bytes += mx_bytes;
        const bool xs = align16(3 * (size_t)n * sizeof(double)) + fixed_bytes <= kSmemBudget;
        smem[B_X] = smem[B_LB] = smem[B_UB] = xs;
    } else if (vec_all + obj_bytes + fixed_bytes <= kSmemBudget) {
        for (int b = 0; b < B_COUNT; ++b) smem[b] = need[b];
        L.obj_smem = 1;
    } else if (vec_all + fixed_bytes <= kSmemBudget) {
        for (int b = 0; b < B_COUNT; ++b) smem[b] = need[b];
        L.obj_smem = 0;
    } else {
        L.obj_smem = obj_bytes + fixed_bytes <= kSmemBudget ? 1 : 0;
    }
    int sc = 0, gc = 0;
    L.vec_smem = 1;
    for (int b = 0; b < B_COUNT; ++b) {
        L.off[b] = -1;
        L.in_smem[b] = 0;
        if (!need[b]) continue;
        if (smem[b]) { L.in_smem[b] = 1; L.off[b] = sc++ * n; }
        else { L.off[b] = gc++ * n; L.vec_smem = 0; }
    }
    if (secant) { L.off[B_CAND] = L.off[B_TX]; L.in_smem[B_CAND] = L.in_smem[B_TX]; }
    L.node_stride = (size_t)gc * n;
    size_t p = 0;
    L.sm_vec = p; p += align16((size_t)sc * n * sizeof(double));
    L.sm_obj = p; if (L.obj_smem) p += obj_bytes;
    L.sm_keys = p; L.sm_prefix = p; L.sm_idx = p; L.sm_fixed = p;
    if (L.sort_size) {
        L.sm_keys = p; p += align16((size_t)L.sort_size * 8);
        L.sm_prefix = p; p += align16((size_t)L.sort_size * 8);
        L.sm_idx = p; p += align16((size_t)L.sort_size * 4);
        L.sm_fixed = p; p += align16((size_t)n);
    }
    L.sm_hung = p; p += (size_t)L.hung_warps * L.hung_bytes;
    L.sm_mx = p; if (mixed && !L.mx_global) p += mx_bytes;
    L.sm_cost = p; if (!L.cost_global) p += cost_bytes;
    L.sm_code = p; if (!L.cost_global) p += code_bytes;
    L.sm_ihw = p; p += mixed ? 2 * L.ihw_bytes : 0;
    L.cs_bytes = mixed && L.cost_global ? colstate_bytes(l.order <= 256 ? 8 : 16) : 0;
    L.sm_cs = p; p += 2 * L.cs_bytes;
    L.sm_total = p;
    // FP64 kernels: two nodes per SM (a 128-register cap) wherever two fit in
    // shared memory, unless pinned
    if (v.per_sm != -1 && v.per_sm != 1 && v.per_sm != 2) {
        *err = "nodes per SM: 1 or 2";
        return GBX_ERR_INVALID;
    }
    if (v.per_sm == 2 && mixed) {
        *err = "nodes per SM applies to the FP64 kernels (mixed precision picks its own)";
        return GBX_ERR_UNSUPPORTED;
    }
    L.per_sm2 = !mixed && (v.per_sm == 2 || (v.per_sm == -1 && 2 * (L.sm_total + kSmemPerCtaReserve) <= kSmemPerSm))
                    ? 1 : 0;
    // a pair of CTAs per node: the dense quadratic objective's products split
    // between them; every node vector must sit in shared memory (each CTA keeps
    // its own copy of the node)
    L.pair = 0;
    L.sm_xch = 0;
    if (v.persistent == 3) {
        if (mixed || o.kind != GBX_OBJ_DENSE_QUADRATIC || !L.vec_smem) {
            *err = "a pair of CTAs per node covers the FP64 dense quadratic objective with the node in shared memory";
            return GBX_ERR_UNSUPPORTED;
        }
        L.pair = 1;
        L.persistent = 0;
        L.sm_xch = align16(L.sm_total);
        L.sm_total = L.sm_xch + align16((size_t)kThreads * sizeof(double));
    }
    // large orders: each integer oracle on four warps unless pinned to one
    L.oracle_group = (L.cs_bytes && v.oracle_warps != 1) ? 1 : 0;
    if (v.oracle_warps != -1 && v.oracle_warps != 1 && v.oracle_warps != 4) {
        *err = "oracle warps: 1 or 4";
        return GBX_ERR_INVALID;
    }
    if (v.oracle_warps == 4 && !L.cs_bytes) {
        *err = "four warps per oracle cover mixed-precision Birkhoff orders 129..512";
        return GBX_ERR_UNSUPPORTED;
    }
    if (v.persistent == 2) {
        // a cluster of kClCtas CTAs per node (large orders, mixed precision):
        // each CTA holds a slice of the packed oracle costs; the leader's FP64
        // workspace (feasibility, certificate) shares the slice's memory, used
        // only while no oracle runs
        if (!mixed || !L.cost_global || L.tc || o.kind != GBX_OBJ_GRAPH_MATCHING || l.kind != GBX_LMO_BIRKHOFF) {
            *err = "a cluster per node covers mixed-precision graph matching over the Birkhoff polytope above order 128";
            return GBX_ERR_UNSUPPORTED;
        }
        const int S = (l.order + kClCtas - 1) / kClCtas;
        const size_t slice = align16((size_t)l.order * S * sizeof(int));
        const size_t chw = align16(chw_bytes(l.order));
        const size_t lpi = align16(4 * (size_t)l.order * sizeof(int));
        const size_t total = slice + 2 * chw + lpi + align16(sizeof(ClCtl));
        if (S > 32 * kClCpl || total > kSmemBudget || L.hung_bytes > slice) {
            *err = "a cluster per node: the cost slices of this order do not fit in shared memory (orders 129..404)";
            return GBX_ERR_UNSUPPORTED;
        }
        L.cluster = kClCtas;
        L.oracle_group = 0;
        L.cl_cols = S;
        L.chw_bytes = chw;
        L.persistent = 0;
        L.sm_slice = 0;
        L.sm_hung = 0;
        L.sm_chw = slice;
        L.sm_lpi = slice + 2 * chw;
        L.sm_cl = L.sm_lpi + lpi;
        L.sm_total = L.sm_cl + align16(sizeof(ClCtl));
    }
    L.mixed_node_bytes = L.mx_global ? (mx_bytes + 255) / 256 * 256 : 0;
    if (L.tc) L.mixed_node_bytes += kTcImageBytes;
    L.mx_cost_off = L.mx_code_off = 0;
    if (L.cost_global) {
        L.mx_cost_off = L.mixed_node_bytes;
        L.mixed_node_bytes += (cost_bytes + 255) / 256 * 256;
        L.mx_code_off = L.mixed_node_bytes;
        L.mixed_node_bytes += (code_bytes + 255) / 256 * 256;
    }
    L.sparse_cap = 0;
    L.sparse_bytes = 0;
    if (o.kind == GBX_OBJ_GRAPH_MATCHING && o.order >= 16) {
        // zero-skipping products pay off below a quarter density
        const int m = o.order;
        L.sparse_cap = m * m / 4;
        L.sparse_bytes = 16 + 4 * sparse_list_bytes(m, L.sparse_cap);
    }
    *out = L;
    return GBX_OK;
}

size_t mixed_region_offset(const Layout& L, int n_nodes) {
    return (L.node_stride * sizeof(double) * (size_t)n_nodes + 255) / 256 * 256;
}

// ---- autotuned launch shapes, per problem shape, process-wide
namespace {
struct Key {
    int ok, lk, n, order, prec, alg, ls;
    bool operator<(const Key& o) const {
        return std::tie(ok, lk, n, order, prec, alg, ls) < std::tie(o.ok, o.lk, o.n, o.order, o.prec, o.alg, o.ls);
    }
};
std::mutex g_tune_mutex;
std::map<Key, Variant> g_tuned;
Key key_of(const gbx_objective& o, const gbx_lmo& l, const gbx_algorithm& a) {
    return {o.kind, l.kind, o.n, l.order, a.precision, a.kind, a.line_search};
}
}  // namespace

Variant tuned_variant(const gbx_objective& o, const gbx_lmo& l, const gbx_algorithm& a) {
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    auto it = g_tuned.find(key_of(o, l, a));
    return it == g_tuned.end() ? Variant{} : it->second;
}

void store_variant(const gbx_objective& o, const gbx_lmo& l, const gbx_algorithm& a, const Variant& v) {
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    g_tuned[key_of(o, l, a)] = v;
}

std::vector<Variant> candidate_variants(const gbx_objective& o, const gbx_lmo& l, const gbx_algorithm& a) {
    std::vector<Variant> out;
    std::vector<int> tcs = {-1};
    if (a.precision == GBX_PRECISION_MIXED && o.kind == GBX_OBJ_GRAPH_MATCHING && l.kind == GBX_LMO_BIRKHOFF
            && l.order > 16 && l.order <= 128)
        tcs = {l.order > 64 ? 1 : 0, l.order > 64 ? 0 : 1};
    // large-order mixed Birkhoff: one or four warps per integer oracle
    std::vector<int> ows = {-1};
    if (a.precision == GBX_PRECISION_MIXED && o.kind == GBX_OBJ_GRAPH_MATCHING && l.kind == GBX_LMO_BIRKHOFF
            && l.order > 128 && l.order <= 512)
        ows = {4, 1};
    // FP64 kernels: two nodes per SM (where they fit) or one
    std::vector<int> pss = {-1};
    if (a.precision != GBX_PRECISION_MIXED) {
        Variant two;
        two.per_sm = 2;
        Layout L2;
        std::string e2;
        if (make_layout(o, l, a, 1, &L2, &e2, &two) == GBX_OK
                && 2 * (L2.sm_total + kSmemPerCtaReserve) <= kSmemPerSm)
            pss = {2, 1};
    }
    for (int tc : tcs)
        for (int ow : ows)
            for (int ps : pss)
                for (int pers : {0, 1}) {
                    Variant v;
                    v.tc = tc;
                    v.persistent = pers;
                    v.oracle_warps = ow;
                    v.per_sm = ps;
                    out.push_back(v);
                }
    // a cluster of CTAs per node where it applies (large-order mixed graph matching)
    Variant cl;
    cl.persistent = 2;
    Layout L;
    std::string err;
    if (make_layout(o, l, a, 1, &L, &err, &cl) == GBX_OK) out.push_back(cl);
    // a pair of CTAs per node where it applies (FP64 dense quadratic, node in shared memory)
    Variant pr;
    pr.persistent = 3;
    if (make_layout(o, l, a, 1, &L, &err, &pr) == GBX_OK) out.push_back(pr);
    return out;
}

size_t sparse_region_offset(const Layout& L, int n_nodes) {
    return (mixed_region_offset(L, n_nodes) + L.mixed_node_bytes * (size_t)n_nodes + 255) / 256 * 256;
}

size_t workspace_bytes(const Layout& L, int n_nodes) {
    return sparse_region_offset(L, n_nodes) + L.sparse_bytes + 256;
}

size_t queue_offset(const Layout& L, int n_nodes) {
    return (sparse_region_offset(L, n_nodes) + L.sparse_bytes + 15) / 16 * 16;
}

size_t workspace_bytes_any_variant(const gbx_objective& o, const gbx_lmo& l, const gbx_algorithm& a, int n_nodes) {
    size_t best = 0;
    for (const Variant& v : candidate_variants(o, l, a)) {
        Layout L;
        std::string err;
        if (make_layout(o, l, a, n_nodes, &L, &err, &v) == GBX_OK) best = std::max(best, workspace_bytes(L, n_nodes));
    }
    return best;
}

int launch_relax(const Params& p, void* stream, std::string* err) {
    if (p.b.n_nodes == 0) return GBX_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int ok = p.obj.kind, lk = p.lmo.kind;
#define GBX_CASE(O, LMOK) if (ok == O && lk == LMOK) return launch_one<O, LMOK>(p, st, err);
    GBX_CASE(GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_BOX)
    GBX_CASE(GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_SIMPLEX)
    GBX_CASE(GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_EQUALITY_SIMPLEX)
    GBX_CASE(GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_BIRKHOFF)
    GBX_CASE(GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_CARDINALITY)
    GBX_CASE(GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_LINKED_CARDINALITY)
    GBX_CASE(GBX_OBJ_GRAPH_MATCHING, GBX_LMO_BIRKHOFF)
    GBX_CASE(GBX_OBJ_GRAPH_MATCHING, GBX_LMO_BOX)
#undef GBX_CASE
    *err = "unsupported objective/LMO combination";
    return GBX_ERR_UNSUPPORTED;
}

static int probe_layout(const gbx_lmo& l, Layout* L, std::string* err) {
    gbx_objective o{};
    o.kind = GBX_OBJ_DENSE_QUADRATIC;
    o.n = l.n;
    gbx_algorithm a{};
    a.kind = GBX_ALG_DICG;
    const int rc = make_layout(o, l, a, 1, L, err);
    if (rc) return rc;
    // probes only need the LMO scratch: rebuild offsets without node vectors
    size_t p = 0;
    Layout& M = *L;
    M.sm_keys = M.sm_prefix = M.sm_idx = M.sm_fixed = 0;
    if (M.sort_size) {
        M.sm_keys = p; p += align16((size_t)M.sort_size * 8);
        M.sm_prefix = p; p += align16((size_t)M.sort_size * 8);
        M.sm_idx = p; p += align16((size_t)M.sort_size * 4);
        M.sm_fixed = p; p += align16((size_t)l.n);
    }
    M.sm_hung = p; p += 2 * M.hung_bytes;
    M.sm_total = p;
    return GBX_OK;
}

int launch_lmo_batch(const gbx_lmo& l, int cases, int mode, const double* dir,
                     const double* x, const double* lb, const double* ub, double* out,
                     double* out_step, void* stream, std::string* err) {
    if (cases == 0) return GBX_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the box oracles are element-wise: one stream over the whole batch; the
    // DICG maximum step (a per-case reduction) stays with the per-case kernel
    if (l.kind == GBX_LMO_BOX && !out_step)
        return launch_box_lmo_stream(mode, (size_t)cases * l.n, dir, x, lb, ub, out, st, err);
    Layout L;
    int rc = probe_layout(l, &L, err);
    if (rc) return rc;
    switch (l.kind) {
    case GBX_LMO_BOX: return probe_one<GBX_LMO_BOX>(l, L, cases, mode, dir, x, lb, ub, out, out_step, st, err);
    case GBX_LMO_SIMPLEX: return probe_one<GBX_LMO_SIMPLEX>(l, L, cases, mode, dir, x, lb, ub, out, out_step, st, err);
    case GBX_LMO_EQUALITY_SIMPLEX: return probe_one<GBX_LMO_EQUALITY_SIMPLEX>(l, L, cases, mode, dir, x, lb, ub, out, out_step, st, err);
    case GBX_LMO_BIRKHOFF: return probe_one<GBX_LMO_BIRKHOFF>(l, L, cases, mode, dir, x, lb, ub, out, out_step, st, err);
    case GBX_LMO_CARDINALITY:
        if (mode != 0) { *err = "the cardinality LMO has no in-face oracle (Frank-Wolfe only)"; return GBX_ERR_UNSUPPORTED; }
        return probe_one<GBX_LMO_CARDINALITY>(l, L, cases, mode, dir, x, lb, ub, out, out_step, st, err);
    case GBX_LMO_LINKED_CARDINALITY:
        return probe_one<GBX_LMO_LINKED_CARDINALITY>(l, L, cases, mode, dir, x, lb, ub, out, out_step, st, err);
    default: *err = "lmo kind"; return GBX_ERR_UNSUPPORTED;
    }
}

int launch_node_feasible(const gbx_lmo& l, int cases, const double* lb, const double* ub,
                         const uint8_t* flags, uint8_t* out, void* stream, std::string* err) {
    if (cases == 0) return GBX_OK;
    Layout L;
    int rc = probe_layout(l, &L, err);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    switch (l.kind) {
    case GBX_LMO_BOX: return feas_one<GBX_LMO_BOX>(l, L, cases, lb, ub, flags, out, st, err);
    case GBX_LMO_SIMPLEX: return feas_one<GBX_LMO_SIMPLEX>(l, L, cases, lb, ub, flags, out, st, err);
    case GBX_LMO_EQUALITY_SIMPLEX: return feas_one<GBX_LMO_EQUALITY_SIMPLEX>(l, L, cases, lb, ub, flags, out, st, err);
    case GBX_LMO_BIRKHOFF: return feas_one<GBX_LMO_BIRKHOFF>(l, L, cases, lb, ub, flags, out, st, err);
    case GBX_LMO_CARDINALITY: return feas_one<GBX_LMO_CARDINALITY>(l, L, cases, lb, ub, flags, out, st, err);
    case GBX_LMO_LINKED_CARDINALITY:
        return feas_one<GBX_LMO_LINKED_CARDINALITY>(l, L, cases, lb, ub, flags, out, st, err);
    default: *err = "lmo kind"; return GBX_ERR_UNSUPPORTED;
    }
}

}  // namespace gbx
