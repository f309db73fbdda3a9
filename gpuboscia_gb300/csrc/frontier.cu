// frontier.cu -- branch and bound with the frontier in device memory.
//
// The host engine (device_resident_solver.h; reference loop
// device_resident_solver.cuh:1570-2067) copies every batch of node vectors
// host -> device and every result back, and branches on the host. Here the
// open nodes live in HBM and a round of the search is a fixed sequence of
// kernels on one stream:
//
//   select   pop the best min(B, live) nodes (the frontier is kept sorted by
//            (bound, id), so this is its head)
//   gather   copy their bounds / start points into the relaxation batch
//   relax    the node-relaxation kernel, batch size read from device memory
//   vars     branch_pow2's variables per node: the k most fractional
//            (branching.h:24-65), ties to the lowest variable index
//   decide   in batch order: incumbent (prefix minimum of the candidates'
//            values, strict improvement as AtomicIncumbent::try_update),
//            certified bound, pruning, continuation of unconverged integral
//            nodes, child ids and sorted frontier keys
//            (process_completed_batch, device_resident_solver.cuh:1865-2007)
//   expand   write the children (2^k' per branched node: bit b of the child
//            index sets lb = ceil(x) or ub = floor(x), branching.h:80-118)
//   merge    merge the sorted children into the rest of the frontier, drop
//            what the incumbent prunes and recycle its pool slots
//   status   live bound, termination (frontier empty, or the certified gap
//            within tolerance, gap_utils.h:44-52)
//
// The sequence is captured once into a CUDA graph of R rounds and replayed;
// the host reads a small control block after every replay (time limit,
// completion). Kernels of a finished search return at once. Nothing waits on
// another CTA: every round is ordered by streams and events alone.
//
// Pool layout. A binary problem (every integer variable's root bounds in
// {0, 1}) stores an open node's bounds as one byte per variable (bit 0: lb = 1,
// bit 1: ub = 1; continuous variables keep the root's bounds), 16x less than
// two FP64 vectors: at order 400 a node takes 160 KB instead of 2.56 MB, so a
// search that opens 10^5 nodes fits in HBM. The iterate of a continued node
// (an unconverged integral node requeued with its x) goes to a small separate
// pool. Other problems keep FP64 bounds and an iterate slot per node.
//
// Two batch slots (default): round r pops slot r % 2 and relaxes it on that
// slot's stream while the control stream branches, decides and merges the
// other slot, so the GPU is not idle behind a batch's slowest node. The
// frontier keeps a head pointer for the popped-but-unmerged entries; the live
// bound includes the slot still relaxing; each slot's cutoff is the incumbent
// at its pop, so results do not depend on timing.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <limits>
#include <string>
#include <vector>

#include "../../include/gpuboscia/gap_utils.h"
#include "../../include/gpuboscia/nvtx.h"
#include "features.h"
#include "relax.cuh"
#include "scorer_mlp.cuh"

namespace gbx {
namespace {

constexpr int kMaxBatch = 1024;    // nodes per round: one decide CTA
constexpr int kMaxK = 8;           // branch_pow2 variables per node on this path
constexpr int kEpsDepths = 4096;   // node tolerance by depth (deeper nodes use the last)
// rounds per graph replay: the host checks the time limit between replays,
// so problems whose rounds are long (large node vectors) replay two at a time
constexpr int kRoundsPerReplay = 4;
constexpr int kRoundsPerReplayLarge = 2;
constexpr long long kLargeRoundDoubles = 1ll << 24;   // batch * n above which a round counts as long

enum Why { RUNNING = 0, EXHAUSTED = 1, TOLERANCE = 2, CAPACITY = 3, NODE_LIMIT = 4 };

// device control block (read by the host after every replay). Two batch
// slots can be in flight: one relaxing while the other is decided and merged.
struct FState {
    double incumbent;
    double bound;          // live bound after the last round
    long long nodes_done;
    int done;
    int why;
    int cur;               // frontier buffer holding the live entries
    int n_front;           // entries of that buffer; [head, n_front) are open
    int head;              // entries before head were popped into a slot
    int free_top;          // free pool slots on the stack
    int next_id;
    int inc_src;           // batch index whose best vertex is the new incumbent (-1)
    int has_inc;
    int rounds;
    int batches;           // rounds whose slot held at least one node
    int xfree_top;         // free continuation-iterate slots (compact pool)
    long long round_nodes[4];   // nodes_done after each of the last four rounds
    int n_batch[2];        // nodes popped into each slot
    int n_new[2];          // entries each slot pushes
    int pop_at[2];         // frontier position the slot's nodes were popped from
    int pop_base[2];       // free-stack position their pool slots went to
    double slot_bound[2];  // smallest bound among a slot's nodes (+inf: empty)
    double slot_cut[2];    // the incumbent when the slot was popped (its relaxation cutoff)
};

// one relaxation batch and the entries it pushes
struct Slot {
    double* x;             // [B * n]
    double* lb;
    double* ub;
    double* best;
    double* eps;           // [B]
    double* gap;
    double* value;
    double* bvv;
    int* it;
    unsigned char* st;
    double* bbound;
    int* bdepth;
    int* bid;
    int* bvars;            // [B * kMaxK]
    int* bnv;              // [B]
    // entries pushed by the slot's decision, sorted by (bound, id) [B << k]
    double* ekey;
    int* eid;
    int* eslot;
    int* esrc;
    int* emask;            // child index, -1: continuation of the node itself
};

struct Tree {
    int n, cap, B, k, n_int, id_stride;
    long long node_limit;  // processed nodes that end the search (0: none)
    double abs_tol, rel_tol, int_tol;
    // pool of open nodes and their records [cap]. Compact pool: pcode
    // [cap * n] bound codes, px [xcap * n] continuation iterates addressed by
    // mxslot, free x slots on xfree. Otherwise plb / pub / px [cap * n].
    int compact;
    int xcap;
    unsigned char* pcode;
    const double* root_lb;  // [n]
    const double* root_ub;
    const unsigned char* isint;  // [n]
    int* mxslot;
    int* xfree;
    double* plb;
    double* pub;
    double* px;
    double* mbound;
    int* mdepth;
    int* mid;
    int* miters;
    unsigned char* mhasx;
    // frontier, sorted by (bound, id), double-buffered for the merge
    double* fkey[2];
    int* fid[2];
    int* fslot[2];
    int* free_stack;       // [cap]
    Slot sl[2];
    const int* int_vars;   // [n_int]
    const double* eps_tab; // [kEpsDepths]
    double* inc_x;         // [n]
    FState* S;
};

__device__ inline bool key_less(double ka, int ia, double kb, int ib) {
    return ka < kb || (ka == kb && ia < ib);
}

// number of entries of the sorted (key, id) list strictly before (k, i)
__device__ inline int count_before(const double* key, const int* id, int len, double k, int i) {
    int lo = 0, hi = len;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (key_less(key[mid], id[mid], k, i)) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// first index whose key is >= v
__device__ inline int first_at_least(const double* key, int len, double v) {
    int lo = 0, hi = len;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (key[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__device__ inline double certified_lower(double inherited, double value, double gap) {
    if (!isfinite(value) || !isfinite(gap) || gap < 0.0) return inherited;
    return fmax(inherited, value - gap);
}

__device__ inline bool within_tolerance(double bound, double inc, double abs_tol, double rel_tol) {
    if (!isfinite(bound) || !isfinite(inc)) return false;
    const double a = fabs(inc - bound);
    if (a <= abs_tol) return true;
    const double scale = fmin(fabs(bound), fabs(inc));
    if (scale == 0.0) return false;
    return (inc - bound) / scale <= rel_tol;
}

// pop the best min(B, open) nodes into slot s; their pool slots are reserved
// on the free stack (gather writes them there once their data is copied)
__global__ void select_kernel(Tree T, int s) {
    FState* S = T.S;
    const int N = S->done ? 0 : min(T.B, S->n_front - S->head);
    S->n_new[s] = 0;
    S->n_batch[s] = N;
    S->pop_at[s] = S->head;
    S->pop_base[s] = S->free_top;
    S->slot_bound[s] = N > 0 ? T.fkey[S->cur][S->head] : __longlong_as_double(0x7ff0000000000000ll);
    S->slot_cut[s] = S->incumbent;   // fixed for the slot's relaxation: the result is timing-independent
    S->head += N;
    S->free_top += N;
    if (N > 0) S->batches += 1;
}

// one CTA per batch node
__global__ void __launch_bounds__(256) gather_kernel(Tree T, int s) {
    FState* S = T.S;
    const Slot& B = T.sl[s];
    const int i = blockIdx.x;
    if (i >= S->n_batch[s]) return;
    const int slot = T.fslot[S->cur][S->pop_at[s] + i];
    const size_t n = T.n, src = (size_t)slot * n, dst = (size_t)i * n;
    const bool hx = T.mhasx[slot] != 0;
    if (T.compact) {
        const int xs = hx ? T.mxslot[slot] : -1;
        const double* xsrc = T.px + (size_t)(xs < 0 ? 0 : xs) * n;
        for (size_t j = threadIdx.x; j < n; j += blockDim.x) {
            const unsigned char c = T.pcode[src + j];
            const bool in = T.isint[j] != 0;
            const double l = in ? ((c & 1) ? 1.0 : 0.0) : T.root_lb[j];
            B.lb[dst + j] = l;
            B.ub[dst + j] = in ? ((c & 2) ? 1.0 : 0.0) : T.root_ub[j];
            B.x[dst + j] = xs >= 0 ? xsrc[j] : l;
        }
        // the iterate now lives in the batch: its x slot goes back to the free stack
        if (threadIdx.x == 0 && xs >= 0) T.xfree[atomicAdd(&S->xfree_top, 1)] = xs;
    } else {
        for (size_t j = threadIdx.x; j < n; j += blockDim.x) {
            const double l = T.plb[src + j];
            B.lb[dst + j] = l;
            B.ub[dst + j] = T.pub[src + j];
            B.x[dst + j] = hx ? T.px[src + j] : l;
        }
    }
    if (threadIdx.x == 0) {
        const int d = T.mdepth[slot];
        B.eps[i] = T.eps_tab[min(d, kEpsDepths - 1)];
        B.it[i] = T.miters[slot];
        B.st[i] = hx ? GBX_NODE_INITIAL_POINT_SUPPLIED : 0;
        B.bbound[i] = T.mbound[slot];
        B.bdepth[i] = d;
        B.bid[i] = T.mid[slot];
        // the node now lives in the batch; its pool slot goes back to the stack
        T.free_stack[S->pop_base[s] + i] = slot;
    }
}

// branch_pow2's variables of batch node i: up to k integer variables with
// fractional distance above the tolerance, most fractional first, ties to the
// lower index (top_k_infeasible). Called by all threads of the CTA.
__device__ void pick_most_fractional(const Tree& T, const Slot& B, int i, const double* x) {
    __shared__ double s_d[8];
    __shared__ int s_j[8];
    __shared__ int s_pick[kMaxK];
    __shared__ int s_count;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) s_count = 0;
    __syncthreads();
    for (int r = 0; r < T.k; ++r) {
        double bd = -1.0;
        int bj = INT_MAX;
        for (int q = tid; q < T.n_int; q += blockDim.x) {
            const int j = T.int_vars[q];
            bool taken = false;
            for (int t = 0; t < r; ++t) taken = taken || s_pick[t] == j;
            if (taken) continue;
            const double v = x[j];
            const double fr = v - floor(v);
            const double d = fmin(fr, 1.0 - fr);
            if (!(d > T.int_tol)) continue;
            if (d > bd || (d == bd && j < bj)) { bd = d; bj = j; }
        }
        for (int o = 16; o; o >>= 1) {
            const double od = __shfl_xor_sync(0xffffffffu, bd, o);
            const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
            if (od > bd || (od == bd && oj < bj)) { bd = od; bj = oj; }
        }
        if (lane == 0) { s_d[w] = bd; s_j[w] = bj; }
        __syncthreads();
        if (tid == 0) {
            double d = s_d[0];
            int j = s_j[0];
            for (int q = 1; q < (int)(blockDim.x >> 5); ++q)
                if (s_d[q] > d || (s_d[q] == d && s_j[q] < j)) { d = s_d[q]; j = s_j[q]; }
            if (j != INT_MAX && d > T.int_tol) s_pick[s_count++] = j;
        }
        __syncthreads();
        if (s_count <= r) break;   // no further fractional variable
    }
    if (tid < s_count) B.bvars[i * kMaxK + tid] = s_pick[tid];
    if (tid == 0) B.bnv[i] = s_count;
}

__global__ void __launch_bounds__(256) vars_kernel(Tree T, int s) {
    const FState* S = T.S;
    const Slot& B = T.sl[s];
    const int i = blockIdx.x;
    if (i >= S->n_batch[s]) return;
    if (B.st[i] >= GBX_NODE_INTEGRAL_UNCONVERGED) {
        if (threadIdx.x == 0) B.bnv[i] = 0;
        return;
    }
    pick_most_fractional(T, B, i, B.x + (size_t)i * T.n);
}

// Learned branching (the host's LearnedBrancher): every fractional candidate
// of the node is scored by the MLP (BF16 weights widened to FP32 when a BF16
// copy exists, as gbx_scorer_forward); branch_pow2 splits on the k highest
// scores, ties to the earlier candidate. A non-finite score sends the node
// to the most-fractional rule. Shared memory: the parameters, then the
// permutation row / column statistics of a Birkhoff iterate.
template <int H>
__global__ void __launch_bounds__(256) learned_vars_kernel(Tree T, int s, gbx_scorer sc, int order) {
    extern __shared__ __align__(16) unsigned char dyn[];
    __shared__ float s_z[8];
    __shared__ int s_q[8];
    __shared__ int s_win;
    const FState* S = T.S;
    const Slot& B = T.sl[s];
    const int i = blockIdx.x;
    if (i >= S->n_batch[s]) return;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (B.st[i] >= GBX_NODE_INTEGRAL_UNCONVERGED) {
        if (tid == 0) B.bnv[i] = 0;
        return;
    }
    const int cnt = mlp::param_count(mlp::kF, H);
    float* prm = reinterpret_cast<float*>(dyn);
    const bool perm = order > 0 && order * order == T.n;
    const int m = perm ? order : 0;
    double* rmax = reinterpret_cast<double*>(dyn + align16((size_t)cnt * sizeof(float)));
    double* cmax = rmax + m;
    int* rfrac = reinterpret_cast<int*>(cmax + m);
    int* cfrac = rfrac + m;
    int* rfree = cfrac + m;
    for (int q = tid; q < cnt; q += blockDim.x)
        prm[q] = sc.params_bf16 ? mlp::bf16_to_f(sc.params_bf16[q]) : sc.params[q];
    const size_t base = (size_t)i * T.n;
    const double* x = B.x + base;
    const double* lb = B.lb + base;
    const double* ub = B.ub + base;
    for (int r = tid; r < m; r += blockDim.x) {
        double rm = 0.0, cm = 0.0;
        int rf = 0, cf = 0, rfr = 0;
        for (int j = 0; j < m; ++j) {
            const int e = r * m + j;
            const double v = x[e];
            rm = (rm < v) ? v : rm;
            const double fr = v - floor(v);
            if (((1.0 - fr) < fr ? 1.0 - fr : fr) > 1e-6) ++rf;
            if (lb[e] < 0.5 && ub[e] >= 0.5) ++rfr;
            const double u = x[j * m + r];
            cm = (cm < u) ? u : cm;
            const double fu = u - floor(u);
            if (((1.0 - fu) < fu ? 1.0 - fu : fu) > 1e-6) ++cf;
        }
        rmax[r] = rm;
        cmax[r] = cm;
        rfrac[r] = rf;
        cfrac[r] = cf;
        rfree[r] = rfr;
    }
    __syncthreads();
    const double rel = feature_rel_gap(B.gap[i], B.value[i]);
    const int depth = B.bdepth[i];
    const mlp::Off o = mlp::offsets(mlp::kF, H);
    // this thread's k best candidates, score descending (earlier first on ties)
    float ks[kMaxK];
    int kq[kMaxK];
    int kc = 0;
    bool bad = false;
    for (int q = tid; q < T.n_int; q += blockDim.x) {
        const int v = T.int_vars[q];
        const double xv = x[v];
        if (!isfinite(xv)) continue;
        const double fr = xv - floor(xv);
        if (!(((1.0 - fr) < fr ? 1.0 - fr : fr) > T.int_tol)) continue;
        PermStats p{};
        if (perm) {
            const int r = v / m, c = v - (v / m) * m;
            p.rfrac = rfrac[r];
            p.cfrac = cfrac[c];
            p.rfree = rfree[r];
            p.rmax = rmax[r];
            p.cmax = cmax[c];
        }
        float f[mlp::kF], a1[H], a2[H];
        candidate_features(xv, depth, rel, perm, m, p, f);
        const float z = mlp::forward_row<H>(prm, o, f, a1, a2);
        if (!isfinite(z)) { bad = true; continue; }
        int pos = kc;
        while (pos > 0 && ks[pos - 1] < z) --pos;
        if (pos >= T.k) continue;
        const int last = kc < T.k ? kc : T.k - 1;
        for (int t = last; t > pos; --t) { ks[t] = ks[t - 1]; kq[t] = kq[t - 1]; }
        ks[pos] = z;
        kq[pos] = q;
        if (kc < T.k) ++kc;
    }
    if (__syncthreads_or(bad)) {
        pick_most_fractional(T, B, i, x);
        return;
    }
    // k rounds over the threads' heads: highest score, then earliest candidate
    int h = 0, picked = 0;
    for (int r = 0; r < T.k; ++r) {
        float bz = 0.f;
        int bq = INT_MAX;
        if (h < kc) { bz = ks[h]; bq = kq[h]; }
        for (int off = 16; off; off >>= 1) {
            const float oz = __shfl_xor_sync(0xffffffffu, bz, off);
            const int oq = __shfl_xor_sync(0xffffffffu, bq, off);
            if (oq != INT_MAX && (bq == INT_MAX || oz > bz || (oz == bz && oq < bq))) { bz = oz; bq = oq; }
        }
        if (lane == 0) { s_z[w] = bz; s_q[w] = bq; }
        __syncthreads();
        if (tid == 0) {
            float z = s_z[0];
            int q = s_q[0];
            for (int t = 1; t < (int)(blockDim.x >> 5); ++t)
                if (s_q[t] != INT_MAX && (q == INT_MAX || s_z[t] > z || (s_z[t] == z && s_q[t] < q))) {
                    z = s_z[t];
                    q = s_q[t];
                }
            s_win = q;
            if (q != INT_MAX) B.bvars[i * kMaxK + r] = T.int_vars[q];
        }
        __syncthreads();
        const int win = s_win;
        __syncthreads();
        if (win == INT_MAX) break;
        if (h < kc && kq[h] == win) ++h;
        ++picked;
    }
    if (tid == 0) B.bnv[i] = picked;
}

size_t learned_smem_bytes(int H, int order) {
    return align16((size_t)mlp::param_count(mlp::kF, H) * sizeof(float))
           + (size_t)std::max(order, 0) * (2 * sizeof(double) + 3 * sizeof(int));
}

// block-wide inclusive scans over kMaxBatch threads
__device__ double block_scan_min(double v, double* wbuf) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const double u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v = fmin(v, u);
    }
    if (lane == 31) wbuf[w] = v;
    __syncthreads();
    if (w == 0) {
        double t = wbuf[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const double u = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t = fmin(t, u);
        }
        wbuf[lane] = t;
    }
    __syncthreads();
    if (w > 0) v = fmin(v, wbuf[w - 1]);
    __syncthreads();
    return v;
}

__device__ int block_scan_sum(int v, int* wbuf, int* total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    if (lane == 31) wbuf[w] = v;
    __syncthreads();
    if (w == 0) {
        int t = wbuf[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += u;
        }
        wbuf[lane] = t;
    }
    __syncthreads();
    if (w > 0) v += wbuf[w - 1];
    *total = wbuf[31];
    __syncthreads();
    return v;   // inclusive
}

// one CTA of kMaxBatch threads; thread i owns batch node i
__global__ void __launch_bounds__(kMaxBatch) decide_kernel(Tree T, int s) {
    FState* S = T.S;
    const Slot& B = T.sl[s];
    const int N = S->n_batch[s];
    if (N == 0) return;
    __shared__ double s_key[kMaxBatch];
    __shared__ int s_first[kMaxBatch];
    __shared__ int s_node[kMaxBatch];
    __shared__ int s_cnt[kMaxBatch];
    __shared__ double s_lower[kMaxBatch];
    __shared__ double wd[32];
    __shared__ int wi[32];
    __shared__ int s_src;
    const int i = threadIdx.x;
    const bool real = i < N;
    const double inc0 = S->incumbent;
    const double kInfD = __longlong_as_double(0x7ff0000000000000ll);

    // incumbent after node i (AtomicIncumbent::try_update in batch order)
    double cand = kInfD;
    if (real) {
        const double v = B.bvv[i];
        if (v < 1e299 && isfinite(v)) cand = v;
    }
    const double inc_i = fmin(inc0, block_scan_min(cand, wd));
    if (i == kMaxBatch - 1) wd[0] = inc_i;   // reuse: final incumbent
    if (i == 0) s_src = INT_MAX;
    __syncthreads();
    const double inc_final = wd[0];
    if (real && inc_final < inc0 && cand == inc_final) atomicMin(&s_src, i);

    // per-node decision
    int cnt = 0, branched = 0, first = INT_MAX;
    double lower = kInfD;
    int status = 0, nv = 0;
    bool cont = false;
    if (real) {
        status = B.st[i];
        const double gap = B.gap[i];
        if (status != GBX_NODE_INFEASIBLE) {
            lower = certified_lower(B.bbound[i], B.value[i], gap);
            const bool certified = isfinite(gap) && gap >= 0.0 && gap < B.eps[i];
            if (lower < inc_i) {
                if (status >= GBX_NODE_INTEGRAL_UNCONVERGED) {
                    cont = !certified;
                } else {
                    nv = B.bnv[i];
                }
            }
        }
        cnt = cont ? 1 : (nv > 0 ? 1 << nv : 0);
        branched = nv > 0 ? 1 : 0;
    }
    int n_branched = 0;
    const int b_incl = block_scan_sum(branched, wi, &n_branched);
    const int id_base = S->next_id + (b_incl - branched) * T.id_stride;
    int n_cont = 0;
    block_scan_sum(cont ? 1 : 0, wi, &n_cont);
    if (real) first = cont ? B.bid[i] : id_base;
    // groups sorted by (bound, first id); a group's ids are consecutive, so the
    // concatenation is sorted by (bound, id)
    s_key[i] = cnt ? lower : kInfD;
    s_first[i] = cnt ? first : INT_MAX;
    s_node[i] = i;
    s_cnt[i] = cnt;
    s_lower[i] = lower;
    __syncthreads();
    for (int size = 2; size <= kMaxBatch; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            const int j = i ^ stride;
            if (j > i) {
                const bool up = (i & size) == 0;
                const bool gt = key_less(s_key[j], s_first[j], s_key[i], s_first[i]);
                if (gt == up) {
                    const double tk = s_key[i]; s_key[i] = s_key[j]; s_key[j] = tk;
                    const int tf = s_first[i]; s_first[i] = s_first[j]; s_first[j] = tf;
                    const int tn = s_node[i]; s_node[i] = s_node[j]; s_node[j] = tn;
                }
            }
            __syncthreads();
        }
    }
    const int node = s_node[i];
    const int gcnt = (node < N) ? s_cnt[node] : 0;
    const int gcont = (gcnt > 0 && B.st[node] >= GBX_NODE_INTEGRAL_UNCONVERGED) ? 1 : 0;
    // free-stack tops, read before the scans' barriers: thread 0 rewrites them
    // below (the batch's pool slots were returned by gather)
    const int top = S->free_top;
    const int xtop = S->xfree_top;
    int E = 0, ncont = 0;
    const int off = block_scan_sum(gcnt, wi, &E) - gcnt;
    const int crank = block_scan_sum(gcont, wi, &ncont) - gcont;   // continuation rank, sorted order
    if (E > top || (T.compact && ncont > xtop)) {
        if (i == 0) { S->done = 1; S->why = CAPACITY; }
        return;
    }
    if (gcnt) {
        const int g = node;
        const bool gc = B.st[g] >= GBX_NODE_INTEGRAL_UNCONVERGED;   // continuation
        const double lo = s_lower[g];
        const int depth = B.bdepth[g];
        for (int c = 0; c < gcnt; ++c) {
            const int p = off + c;
            const int slot = T.free_stack[top - 1 - p];
            const int id = s_first[i] + (gc ? 0 : c);
            B.ekey[p] = lo;
            B.eid[p] = id;
            B.eslot[p] = slot;
            B.esrc[p] = g;
            B.emask[p] = gc ? -1 : c;
            T.mbound[slot] = lo;
            T.mdepth[slot] = gc ? depth : depth + 1;
            T.mid[slot] = id;
            T.miters[slot] = gc ? B.it[g] : 0;
            T.mhasx[slot] = gc ? 1 : 0;
            if (T.compact) T.mxslot[slot] = gc ? T.xfree[xtop - 1 - crank] : -1;
        }
    }
    if (i == 0) {
        S->free_top = top - E;
        if (T.compact) S->xfree_top = xtop - ncont;
        S->n_new[s] = E;
        S->next_id += n_branched * T.id_stride;
        S->nodes_done += N - n_cont;
        if (s_src != INT_MAX) {
            S->incumbent = inc_final;
            S->inc_src = s_src;
            S->has_inc = 1;
        } else {
            S->inc_src = -1;
        }
    }
}

// children / continuations into their pool slots, and the incumbent's x
__global__ void __launch_bounds__(256) expand_kernel(Tree T, int s) {
    const FState* S = T.S;
    if (S->done) return;
    const Slot& B = T.sl[s];
    const int E = S->n_new[s];
    const size_t n = T.n;
    __shared__ int s_vars[kMaxK];
    for (int p = blockIdx.x; p <= E; p += gridDim.x) {
        if (p == E) {
            const int src = S->inc_src;
            if (src < 0) break;
            for (size_t j = threadIdx.x; j < n; j += blockDim.x) T.inc_x[j] = B.best[(size_t)src * n + j];
            break;
        }
        const int slot = B.eslot[p], g = B.esrc[p], mask = B.emask[p];
        const int nv = mask < 0 ? 0 : B.bnv[g];
        __syncthreads();
        if ((int)threadIdx.x < nv) s_vars[threadIdx.x] = B.bvars[g * kMaxK + threadIdx.x];
        __syncthreads();
        const size_t src = (size_t)g * n, dst = (size_t)slot * n;
        double* xdst = T.px + (T.compact ? (size_t)(mask < 0 ? T.mxslot[slot] : 0) * n : dst);
        for (size_t j = threadIdx.x; j < n; j += blockDim.x) {
            double l = B.lb[src + j], u = B.ub[src + j];
            for (int b = 0; b < nv; ++b) {
                if (s_vars[b] == (int)j) {
                    const double xv = B.x[src + j];
                    if (mask >> b & 1) l = ceil(xv);
                    else u = floor(xv);
                }
            }
            if (T.compact) {
                // integer variables of a binary problem: l, u in {0, 1}
                T.pcode[dst + j] = (unsigned char)((l >= 0.5 ? 1 : 0) | (u >= 0.5 ? 2 : 0));
            } else {
                T.plb[dst + j] = l;
                T.pub[dst + j] = u;
            }
            if (mask < 0) xdst[j] = B.x[src + j];
        }
    }
}

// merge the open part of the frontier with slot s's sorted new entries into
// the other buffer; entries the incumbent prunes form the tail and free their slots
__global__ void __launch_bounds__(256) merge_kernel(Tree T, int s) {
    FState* S = T.S;
    if (S->done) return;
    const Slot& B = T.sl[s];
    const int cur = S->cur, h = S->head, E = S->n_new[s];
    const int R = S->n_front - h;
    const double inc = S->incumbent;
    const double* rk = T.fkey[cur] + h;
    const int* ri = T.fid[cur] + h;
    const int* rs = T.fslot[cur] + h;
    double* ok = T.fkey[cur ^ 1];
    int* oi = T.fid[cur ^ 1];
    int* os = T.fslot[cur ^ 1];
    const int total = R + E;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        double k;
        int id, slot, pos;
        if (t < R) {
            k = rk[t]; id = ri[t]; slot = rs[t];
            pos = t + count_before(B.ekey, B.eid, E, k, id);
        } else {
            const int e = t - R;
            k = B.ekey[e]; id = B.eid[e]; slot = B.eslot[e];
            pos = e + count_before(rk, ri, R, k, id);
        }
        if (k < inc) {
            ok[pos] = k; oi[pos] = id; os[pos] = slot;
        } else {
            T.free_stack[atomicAdd(&S->free_top, 1)] = slot;
        }
    }
}

// after slot s's merge: the open frontier, the live bound (the frontier's head,
// the other slot's nodes still relaxing, the incumbent) and termination
__global__ void status_kernel(Tree T, int s) {
    FState* S = T.S;
    if (S->done) return;
    const Slot& B = T.sl[s];
    const int cur = S->cur, h = S->head, E = S->n_new[s];
    const int R = S->n_front - h;
    const double inc = S->incumbent;
    const int live = first_at_least(T.fkey[cur] + h, R, inc) + first_at_least(B.ekey, E, inc);
    S->cur = cur ^ 1;
    S->n_front = live;
    S->head = 0;
    S->round_nodes[S->rounds & 3] = S->nodes_done;
    S->rounds += 1;
    S->inc_src = -1;
    S->n_batch[s] = 0;
    S->n_new[s] = 0;
    S->slot_bound[s] = __longlong_as_double(0x7ff0000000000000ll);
    const bool other = S->n_batch[s ^ 1] > 0;
    double bound = live > 0 ? fmin(T.fkey[cur ^ 1][0], inc) : inc;
    if (other) bound = fmin(bound, S->slot_bound[s ^ 1]);
    S->bound = bound;
    if (live == 0 && !other) { S->done = 1; S->why = EXHAUSTED; }
    else if (within_tolerance(bound, inc, T.abs_tol, T.rel_tol)) { S->done = 1; S->why = TOLERANCE; }
    else if (T.node_limit > 0 && S->nodes_done >= T.node_limit) { S->done = 1; S->why = NODE_LIMIT; }
}

struct DeviceBuffers {
    std::vector<void*> ptrs;
    ~DeviceBuffers() { for (void* p : ptrs) cudaFree(p); }
    template <class T>
    T* get(size_t count, cudaError_t* e) {
        void* p = nullptr;
        if (*e == cudaSuccess) *e = cudaMalloc(&p, std::max<size_t>(count * sizeof(T), 16));
        if (*e != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
};

}  // namespace

size_t frontier_slot_bytes(int n, int compact) {
    const size_t vectors = compact ? (size_t)n + sizeof(int)        // bound codes, x-pool index
                                   : 3 * (size_t)n * sizeof(double); // lb, ub, iterate
    return vectors + sizeof(double) + 3 * sizeof(int) + 1              // pool records
           + 2 * (sizeof(double) + 2 * sizeof(int)) + sizeof(int);     // frontier, free stack
}

// Binary problem: every integer variable's root bounds are 0 or 1, so every
// node's bounds are too and fit the one-byte codes of the compact pool.
static bool frontier_compact(const gbx_problem& pr) {
    for (int q = 0; q < pr.n_int; ++q) {
        const double l = pr.lb[pr.int_vars[q]], u = pr.ub[pr.int_vars[q]];
        if (!((l == 0.0 || l == 1.0) && (u == 0.0 || u == 1.0))) return false;
    }
    return true;
}

int solve_device_frontier(const gbx_problem& pr, const gbx_objective& obj, const gbx_lmo& lmo,
                          const gbx_settings& s, const double* root_x, gbx_result* res, std::string* err) {
    const int n = pr.n_vars, B = s.gpu_batch_size, k = s.branch_k;
    if (B < 1 || B > kMaxBatch) { *err = "device frontier: gpu_batch_size must be in [1, 1024]"; return GBX_ERR_INVALID; }
    if (k < 1 || k > kMaxK) { *err = "device frontier: branch_k must be in [1, 8]"; return GBX_ERR_INVALID; }
    if (s.frontier_slots != 1 && s.frontier_slots != 2) {
        *err = "device frontier: frontier_slots must be 1 or 2";
        return GBX_ERR_INVALID;
    }
    if (s.scorer && (!s.scorer->params || s.scorer->n_features != GBX_SCORER_FEATURES
                     || (s.scorer->hidden != 16 && s.scorer->hidden != 32 && s.scorer->hidden != 64))) {
        *err = "scorer: invalid descriptor (hidden must be 16, 32 or 64)";
        return GBX_ERR_INVALID;
    }
    // the host engine's argument checks (its constructor)
    if (s.gpu_max_iters <= 0) { *err = "GPU iterations, batch size and streams must be positive"; return GBX_ERR_INVALID; }
    if (!std::isfinite(s.gpu_eps) || s.gpu_eps <= 0.0 || !std::isfinite(s.gpu_eps_min) || s.gpu_eps_min <= 0.0
            || !std::isfinite(s.gpu_eps_decay) || s.gpu_eps_decay <= 0.0 || s.gpu_eps_decay > 1.0
            || !std::isfinite(s.abs_gap_tol) || s.abs_gap_tol < 0.0 || !std::isfinite(s.rel_gap_tol)
            || s.rel_gap_tol < 0.0) {
        *err = "invalid tolerance configuration";
        return GBX_ERR_INVALID;
    }
    if (std::isnan(s.time_limit_seconds) || s.time_limit_seconds <= 0.0) {
        *err = "time limit must be positive";
        return GBX_ERR_INVALID;
    }
    for (int q = 0; q < pr.n_int; ++q)
        if (pr.int_vars[q] < 0 || pr.int_vars[q] >= n) { *err = "integer variable index out of range"; return GBX_ERR_INVALID; }
    if (gbx_relax_workspace_bytes(&obj, &lmo, &s.algorithm, B) == 0) {
        *err = gbx_last_error();
        return GBX_ERR_INVALID;
    }
    const auto t0 = std::chrono::steady_clock::now();
    cudaStream_t st = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } sg{st};

    // pool capacity: the caller's, else a quarter of free memory up to 2^18 nodes
    // (less the continuation iterates of a compact pool: two batches' worth)
    const int compact = frontier_compact(pr) ? 1 : 0;
    long long cap = s.frontier_capacity;
    const int E_max = B << k;
    if (cap <= 0) {
        size_t fr = 0, tot = 0;
        e = cudaMemGetInfo(&fr, &tot);
        if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
        const size_t xbytes = compact ? (size_t)2 * B * n * sizeof(double) : 0;
        const size_t room = fr / 4 > xbytes ? fr / 4 - xbytes : 0;
        cap = std::min<long long>(1 << 18, (long long)(room / frontier_slot_bytes(n, compact)));
        cap = std::max<long long>(cap, (long long)E_max + B + 1);
    }
    if (cap < (long long)E_max + 1 || cap > (1ll << 30)) {
        *err = "device frontier: frontier_capacity must hold at least one round's children (batch * 2^branch_k + 1)";
        return GBX_ERR_INVALID;
    }

    DeviceBuffers D;
    Tree T{};
    T.n = n; T.cap = (int)cap; T.B = B; T.k = k; T.n_int = pr.n_int;
    T.id_stride = std::max(8, 1 << k);
    T.abs_tol = s.abs_gap_tol; T.rel_tol = s.rel_gap_tol; T.int_tol = s.integer_tol;
    T.node_limit = s.node_limit;
    const size_t C = (size_t)cap, Nn = (size_t)n;
    T.compact = compact;
    T.xcap = compact ? (int)std::min<long long>(cap, 2ll * B) : 0;
    if (compact) {
        T.pcode = D.get<unsigned char>(C * Nn, &e);
        T.mxslot = D.get<int>(C, &e);
        T.xfree = D.get<int>((size_t)T.xcap, &e);
        T.px = D.get<double>((size_t)T.xcap * Nn, &e);
    } else {
        T.plb = D.get<double>(C * Nn, &e);
        T.pub = D.get<double>(C * Nn, &e);
        T.px = D.get<double>(C * Nn, &e);
    }
    T.mbound = D.get<double>(C, &e);
    T.mdepth = D.get<int>(C, &e);
    T.mid = D.get<int>(C, &e);
    T.miters = D.get<int>(C, &e);
    T.mhasx = D.get<unsigned char>(C, &e);
    for (int b = 0; b < 2; ++b) {
        T.fkey[b] = D.get<double>(C, &e);
        T.fid[b] = D.get<int>(C, &e);
        T.fslot[b] = D.get<int>(C, &e);
    }
    T.free_stack = D.get<int>(C, &e);
    const size_t BN = (size_t)B * Nn;
    const int NS = s.frontier_slots == 1 ? 1 : 2;
    for (int q = 0; q < NS; ++q) {
        Slot& L = T.sl[q];
        L.x = D.get<double>(BN, &e);
        L.lb = D.get<double>(BN, &e);
        L.ub = D.get<double>(BN, &e);
        L.best = D.get<double>(BN, &e);
        L.eps = D.get<double>(B, &e);
        L.gap = D.get<double>(B, &e);
        L.value = D.get<double>(B, &e);
        L.bvv = D.get<double>(B, &e);
        L.it = D.get<int>(B, &e);
        L.st = D.get<unsigned char>(B, &e);
        L.bbound = D.get<double>(B, &e);
        L.bdepth = D.get<int>(B, &e);
        L.bid = D.get<int>(B, &e);
        L.bvars = D.get<int>((size_t)B * kMaxK, &e);
        L.bnv = D.get<int>(B, &e);
        L.ekey = D.get<double>(E_max, &e);
        L.eid = D.get<int>(E_max, &e);
        L.eslot = D.get<int>(E_max, &e);
        L.esrc = D.get<int>(E_max, &e);
        L.emask = D.get<int>(E_max, &e);
    }
    if (NS == 1) T.sl[1] = T.sl[0];
    int* d_int_vars = D.get<int>(std::max(pr.n_int, 1), &e);
    double* d_eps = D.get<double>(kEpsDepths, &e);
    T.inc_x = D.get<double>(Nn, &e);
    T.S = D.get<FState>(1, &e);
    unsigned char* d_flags = D.get<unsigned char>(Nn, &e);
    double* d_root_lb = compact ? D.get<double>(Nn, &e) : nullptr;
    double* d_root_ub = compact ? D.get<double>(Nn, &e) : nullptr;
    T.root_lb = d_root_lb;
    T.root_ub = d_root_ub;
    T.isint = d_flags;
    if (e != cudaSuccess) { *err = std::string("device frontier allocation: ") + cudaGetErrorString(e); return GBX_ERR_CUDA; }
    T.int_vars = d_int_vars;
    T.eps_tab = d_eps;

    // host-side initial state: the root in slot 0, every other slot free
    std::vector<unsigned char> flags(n, 0);
    for (int q = 0; q < pr.n_int; ++q) flags[pr.int_vars[q]] = 1;
    std::vector<double> eps(kEpsDepths);
    for (int d = 0; d < kEpsDepths; ++d)
        eps[d] = gpuboscia::depth_dependent_tolerance(s.gpu_eps, s.gpu_eps_decay, s.gpu_eps_min, d);
    std::vector<int> stack(C - 1);
    for (size_t q = 0; q + 1 < C; ++q) stack[q] = (int)(C - 1 - q);   // slot 1 on top
    FState S0{};
    S0.incumbent = std::numeric_limits<double>::infinity();
    S0.bound = s.natural_lower_bound;
    S0.n_front = 1;
    S0.free_top = (int)C - 1;
    S0.next_id = 1;
    S0.inc_src = -1;
    S0.slot_bound[0] = S0.slot_bound[1] = std::numeric_limits<double>::infinity();
    // compact pool: the root's codes; its start point (if any) in x slot 0
    std::vector<unsigned char> root_code;
    std::vector<int> xstack;
    int root_xslot = -1;
    if (compact) {
        root_code.assign(Nn, 0);
        for (int q = 0; q < pr.n_int; ++q) {
            const int j = pr.int_vars[q];
            root_code[j] = (unsigned char)((pr.lb[j] == 1.0 ? 1 : 0) | (pr.ub[j] == 1.0 ? 2 : 0));
        }
        const int first = root_x ? 1 : 0;
        for (int q = T.xcap - 1; q >= first; --q) xstack.push_back(q);   // lowest free slot on top
        root_xslot = root_x ? 0 : -1;
        S0.xfree_top = (int)xstack.size();
    }
    const double root_bound = s.natural_lower_bound;
    const int zero = 0;
    const unsigned char hx = root_x ? 1 : 0;
    auto up = [&](void* dst, const void* src, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    };
    up(d_flags, flags.data(), Nn);
    up(d_int_vars, pr.int_vars, sizeof(int) * pr.n_int);
    up(d_eps, eps.data(), sizeof(double) * kEpsDepths);
    up(T.free_stack, stack.data(), sizeof(int) * stack.size());
    if (compact) {
        up(T.pcode, root_code.data(), Nn);
        up(T.mxslot, &root_xslot, sizeof(int));
        up(T.xfree, xstack.data(), sizeof(int) * xstack.size());
        up(d_root_lb, pr.lb, sizeof(double) * Nn);
        up(d_root_ub, pr.ub, sizeof(double) * Nn);
    } else {
        up(T.plb, pr.lb, sizeof(double) * Nn);
        up(T.pub, pr.ub, sizeof(double) * Nn);
    }
    if (root_x) up(T.px, root_x, sizeof(double) * Nn);
    up(T.mbound, &root_bound, sizeof(double));
    up(T.mdepth, &zero, sizeof(int));
    up(T.mid, &zero, sizeof(int));
    up(T.miters, &zero, sizeof(int));
    up(T.mhasx, &hx, 1);
    up(T.fkey[0], &root_bound, sizeof(double));
    up(T.fid[0], &zero, sizeof(int));
    up(T.fslot[0], &zero, sizeof(int));
    up(T.S, &S0, sizeof(FState));
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }

    // the relaxation launch of each slot over its batch buffers, with its own
    // workspace (nonzero lists, persistent-grid counter)
    Params P[2] = {};
    for (int q = 0; q < NS; ++q) {
        Params& p = P[q];
        const Slot& L = T.sl[q];
        p.obj = obj;
        p.lmo = lmo;
        p.alg = s.algorithm;
        p.b.n_nodes = B;
        p.b.max_iters = s.gpu_max_iters;
        p.b.candidate_tol = s.integer_tol;
        p.b.x = L.x; p.b.lb = L.lb; p.b.ub = L.ub; p.b.eps = L.eps;
        p.b.iterations = L.it; p.b.status = L.st; p.b.gap = L.gap; p.b.value = L.value;
        p.b.best_vertex = L.best; p.b.best_vertex_val = L.bvv; p.b.integer_flags = d_flags;
        p.b.cutoff = s.incumbent_cutoff ? &T.S->slot_cut[q] : nullptr;
        int rc = make_layout(obj, lmo, s.algorithm, B, &p.L, err);
        if (rc) return rc;
        const size_t wsb = workspace_bytes(p.L, B);
        unsigned char* ws = D.get<unsigned char>(wsb, &e);
        if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
        p.ws = reinterpret_cast<double*>(ws);
        p.queue = p.L.persistent ? reinterpret_cast<int*>(ws + queue_offset(p.L, B)) : nullptr;
        p.mixed = p.L.mixed_node_bytes ? ws + mixed_region_offset(p.L, B) : nullptr;
        p.sparse = nullptr;
        p.live_count = &T.S->n_batch[q];
        if (p.L.sparse_bytes) {
            p.sparse = ws + sparse_region_offset(p.L, B);
            rc = launch_sparse_build(obj, p.L, p.sparse, st, err);
            if (rc) return rc;
        }
    }
    // one stream per slot for its relaxation; the frontier work stays on `st`
    cudaStream_t rs[2] = {nullptr, nullptr};
    cudaEvent_t ev_fork[2] = {nullptr, nullptr}, ev_join[2] = {nullptr, nullptr};
    struct SlotStreams {
        cudaStream_t* s; cudaEvent_t* a; cudaEvent_t* b;
        ~SlotStreams() {
            for (int q = 0; q < 2; ++q) {
                if (s[q]) cudaStreamDestroy(s[q]);
                if (a[q]) cudaEventDestroy(a[q]);
                if (b[q]) cudaEventDestroy(b[q]);
            }
        }
    } ssg{rs, ev_fork, ev_join};
    if (NS == 2)
        for (int q = 0; q < 2; ++q) {
            if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&rs[q], cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_fork[q], cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_join[q], cudaEventDisableTiming);
        }
    // per-round timing (gbx_settings.trace): an event at the start of every
    // replay and one after each of its rounds, all on the frontier's stream
    // (recorded as external events, so that a captured replay records them too)
    const bool tracing = s.trace && s.trace->capacity > 0 && s.trace->ms && s.trace->nodes;
    cudaEvent_t ev_round[kRoundsPerReplay + 1] = {};
    struct RoundEvents {
        cudaEvent_t* ev;
        ~RoundEvents() { for (int i = 0; i <= kRoundsPerReplay; ++i) if (ev[i]) cudaEventDestroy(ev[i]); }
    } reg{ev_round};
    if (tracing)
        for (int i = 0; i <= kRoundsPerReplay && e == cudaSuccess; ++i) e = cudaEventCreate(&ev_round[i]);
    if (s.trace) s.trace->count = 0;
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    int rc = GBX_OK;

    int dev = 0, sms = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    // branching kernel: most fractional, or the learned scorer
    const gbx_scorer sc = s.scorer ? *s.scorer : gbx_scorer{};
    const int sc_order = lmo.kind == GBX_LMO_BIRKHOFF ? lmo.order : 0;
    const size_t sc_smem = s.scorer ? learned_smem_bytes(sc.hidden, sc_order) : 0;
    if (s.scorer) {
        auto kfn = sc.hidden == 16 ? learned_vars_kernel<16> : sc.hidden == 32 ? learned_vars_kernel<32>
                                                                                 : learned_vars_kernel<64>;
        e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sc_smem);
        if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    }
    const int expand_grid = std::min(E_max + 1, 4 * sms);
    const int merge_grid = 4 * sms;
    // the other half of a round: branch, decide, expand, merge, status of slot q
    auto finish = [&](int q) {
        if (!s.scorer) vars_kernel<<<B, 256, 0, st>>>(T, q);
        else if (sc.hidden == 16) learned_vars_kernel<16><<<B, 256, sc_smem, st>>>(T, q, sc, sc_order);
        else if (sc.hidden == 32) learned_vars_kernel<32><<<B, 256, sc_smem, st>>>(T, q, sc, sc_order);
        else learned_vars_kernel<64><<<B, 256, sc_smem, st>>>(T, q, sc, sc_order);
        decide_kernel<<<1, kMaxBatch, 0, st>>>(T, q);
        expand_kernel<<<expand_grid, 256, 0, st>>>(T, q);
        merge_kernel<<<merge_grid, 256, 0, st>>>(T, q);
        status_kernel<<<1, 1, 0, st>>>(T, q);
    };
    // Round r pops into slot r % 2 and relaxes it on that slot's stream, then
    // finishes the other slot, whose relaxation the previous round started.
    // A replay holds an even number of rounds and ends by joining its last
    // relaxation, so the next replay's first round finishes it in stream order.
    // With one slot a round is pop, relax, finish on one stream.
    const int rpr = (long long)B * n > kLargeRoundDoubles ? kRoundsPerReplayLarge : kRoundsPerReplay;
    auto round = [&](int r) -> int {
        const int q = NS == 1 ? 0 : (r & 1);
        if (tracing && r % rpr == 0) {
            const cudaError_t ee = cudaEventRecordWithFlags(ev_round[0], st, cudaEventRecordExternal);
            if (ee != cudaSuccess) { *err = cudaGetErrorString(ee); return GBX_ERR_CUDA; }
        }
        select_kernel<<<1, 1, 0, st>>>(T, q);
        gather_kernel<<<B, 256, 0, st>>>(T, q);
        if (NS == 1) {
            int rr = launch_relax(P[0], st, err);
            if (rr) return rr;
            finish(0);
        } else {
            cudaError_t ee = cudaEventRecord(ev_fork[q], st);
            if (ee == cudaSuccess) ee = cudaStreamWaitEvent(rs[q], ev_fork[q], 0);
            if (ee != cudaSuccess) { *err = cudaGetErrorString(ee); return GBX_ERR_CUDA; }
            int rr = launch_relax(P[q], rs[q], err);
            if (rr) return rr;
            ee = cudaEventRecord(ev_join[q], rs[q]);
            if (ee == cudaSuccess && r % rpr != 0) ee = cudaStreamWaitEvent(st, ev_join[q ^ 1], 0);
            if (ee != cudaSuccess) { *err = cudaGetErrorString(ee); return GBX_ERR_CUDA; }
            finish(q ^ 1);
            if (r % rpr == rpr - 1) {   // join the last relaxation of the replay
                ee = cudaStreamWaitEvent(st, ev_join[q], 0);
                if (ee != cudaSuccess) { *err = cudaGetErrorString(ee); return GBX_ERR_CUDA; }
            }
        }
        if (tracing) {
            const cudaError_t ee = cudaEventRecordWithFlags(ev_round[r % rpr + 1], st, cudaEventRecordExternal);
            if (ee != cudaSuccess) { *err = cudaGetErrorString(ee); return GBX_ERR_CUDA; }
        }
        const cudaError_t le = cudaGetLastError();
        if (le != cudaSuccess) { *err = cudaGetErrorString(le); return GBX_ERR_CUDA; }
        return GBX_OK;
    };

    cudaGraphExec_t exec = nullptr;
    struct ExecGuard { cudaGraphExec_t* g; ~ExecGuard() { if (*g) cudaGraphExecDestroy(*g); } } eg{&exec};
    if (s.use_cuda_graph) {
        cudaGraph_t g = nullptr;
        e = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed);
        int crc = e == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
        for (int r = 0; r < rpr && crc == GBX_OK; ++r) crc = round(r);
        const cudaError_t ee = cudaStreamEndCapture(st, &g);
        if (crc == GBX_OK && ee == cudaSuccess && g) {
            if (cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) exec = nullptr;
        }
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();   // a failed capture falls back to direct launches
        if (!exec) err->clear();
    }

    FState* hS = nullptr;
    e = cudaMallocHost(&hS, sizeof(FState));
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    struct HostGuard { FState* p; ~HostGuard() { cudaFreeHost(p); } } hg{hS};
    bool timed_out = false;
    int rounds_seen = 0;
    long long nodes_seen = 0;
    const auto t_search = std::chrono::steady_clock::now();   // the time limit counts from here
    for (;;) {
        gpuboscia::detail::NvtxRange replay_range("gbx.frontier_rounds");
        if (exec) {
            e = cudaGraphLaunch(exec, st);
            if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
        } else {
            for (int r = 0; r < rpr; ++r) {
                rc = round(r);
                if (rc) return rc;
            }
        }
        e = cudaMemcpyAsync(hS, T.S, sizeof(FState), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
        if (tracing) {
            // the rounds this replay completed (a finished search skips the rest)
            const int nr = std::min(hS->rounds - rounds_seen, rpr);
            float prev = 0.f;
            for (int i = 0; i < nr; ++i) {
                float t = 0.f;
                e = cudaEventElapsedTime(&t, ev_round[0], ev_round[i + 1]);
                if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
                const long long after = hS->round_nodes[(rounds_seen + i) & 3];
                gbx_round_trace* tr = s.trace;
                if (tr->count < tr->capacity) {
                    tr->ms[tr->count] = t - prev;
                    tr->nodes[tr->count] = (int)(after - nodes_seen);
                    tr->count += 1;
                }
                prev = t;
                nodes_seen = after;
            }
            rounds_seen = hS->rounds;
        }
        if (hS->done) break;
        const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_search).count();
        if (std::isfinite(s.time_limit_seconds) && el >= s.time_limit_seconds) { timed_out = true; break; }
    }
    if (hS->why == CAPACITY) {
        *err = "device frontier: pool capacity exceeded (raise frontier_capacity)";
        return GBX_ERR_WORKSPACE;
    }
    res->objective = hS->incumbent;
    res->dual_bound = hS->why == EXHAUSTED ? hS->incumbent : hS->bound;
    res->nodes_processed = (int)hS->nodes_done;
    res->reached_tolerance = hS->why == TOLERANCE ? 1 : 0;
    res->reached_time_limit = timed_out ? 1 : 0;
    res->reached_node_limit = hS->why == NODE_LIMIT ? 1 : 0;
    res->batches = hS->batches;
    res->has_incumbent = hS->has_inc;
    if (res->x && hS->has_inc) {
        e = cudaMemcpy(res->x, T.inc_x, sizeof(double) * Nn, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    }
    res->elapsed_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return GBX_OK;
}

}  // namespace gbx
