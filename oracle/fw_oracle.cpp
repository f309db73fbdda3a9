// fw_oracle.cpp -- TEST INFRASTRUCTURE, not product code.
//
// FP64 CPU restatement of GPUBoscia's node-relaxation path, used only as the
// checker by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg.
// Nothing in gpuboscia_gb300/ links or calls it.
//
// What it restates (file:line in the reference project):
//   drs_fw_relax_node              include/gpuboscia/device_resident_solver.cuh:337-629
//   drs_node_feasible / scoring    device_resident_solver.cuh:206-335
//   SecantLS::search               include/gpuboscia/algorithms.cuh:121-258
//   QuadraticExactLS::search       algorithms.cuh:277-295, line_search_options.h:53-63
//   open-loop / scaled schedules   algorithms.cuh:57-89, device_resident_solver.cuh:562-580
//   BoxLMO                         include/gpuboscia/lmo.cuh:212-321
//   UnitSimplexLMO (GPU oracle)    lmo.cuh:373-397, 517-618, 787-906
//   BirkhoffLMO Hungarian          lmo.cuh:1063-1171 (CPU), 1239-1417 (block)
//   dense quadratic objective      include/gpuboscia/dense_quadratic_objectives.cuh:43-111
//   graph-matching objective       examples/main.cu:131-181 (generalised)
//   RoundingHeuristic              include/gpuboscia/heuristics.h:23-35
//   host B&B worker (one slot)     device_resident_solver.cuh:1570-2086
//   queue / incumbent / branching  concurrent_queue.h:10-90, atomic_incumbent.h,
//                                  branching.h:24-118, gap_utils.h:14-62,
//                                  gpuboscia.cuh:56-170, tree.h:100-149
//
// Arithmetic order. Every block reduction is restated with 256 lanes: lane l
// accumulates elements j = l, l+256, ... in increasing j, each warp of 32 lanes
// folds with the shuffle-down tree (16, 8, 4, 2, 1) and warp 0 folds the 8
// warp partials the same way with zero padding. Products that the GPU fuses
// are written as std::fma here; everything else is one IEEE operation at a
// time (built with -ffp-contract=off). The FP64 GPU path follows the same
// order, so its iterates can be compared bit for bit.
//
// Parity pins: the LMOs are checked against the reference's own CPU functions
// (compute_v_cpu, compute_inface_v_cpu, lmo_dicg.h) compiled from the
// reference sources into oracle/_ref, and the solver against the known
// answers held by the reference tests (tests/test_pipeline.cu, test_cpu.cpp,
// examples/minimal.cu); see tests/test_oracle_*.py.

#include "../include/gpuboscia_gb300.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <queue>
#include <set>
#include <string>
#include <thread>
#include <vector>

namespace {

constexpr int kLanes = 256;
constexpr int kWarps = kLanes / 32;
constexpr double kNone = 1e300;
constexpr double kInf = std::numeric_limits<double>::infinity();

thread_local std::string g_error;

// ---------------------------------------------------------------- reductions
double fold32_sum(double* p) {
    for (int off = 16; off > 0; off >>= 1)
        for (int l = 0; l < off; ++l) p[l] = p[l] + p[l + off];
    return p[0];
}
double fold32_min(double* p) {
    for (int off = 16; off > 0; off >>= 1)
        for (int l = 0; l < off; ++l) p[l] = std::fmin(p[l], p[l + off]);
    return p[0];
}

struct Lanes {
    double v[kLanes];
    void fill(double x) { for (double& e : v) e = x; }
};

// drs_block_reduce / lmo_block_sum / feasibility_block_sum (256 threads).
double reduce_sum(const Lanes& in) {
    double w[32];
    for (int k = 0; k < kWarps; ++k) {
        double t[32];
        std::memcpy(t, in.v + 32 * k, sizeof(t));
        w[k] = fold32_sum(t);
    }
    for (int k = kWarps; k < 32; ++k) w[k] = 0.0;
    return fold32_sum(w);
}
// drs_block_min: lanes beyond the warp count read 1.0.
double reduce_min(const Lanes& in) {
    double w[32];
    for (int k = 0; k < kWarps; ++k) {
        double t[32];
        std::memcpy(t, in.v + 32 * k, sizeof(t));
        w[k] = fold32_min(t);
    }
    for (int k = kWarps; k < 32; ++k) w[k] = 1.0;
    return fold32_min(w);
}

// ---------------------------------------------------------------- objective
struct Objective {
    const gbx_objective* o;
    int n;
    // residual scratch for graph matching (n doubles)
    mutable std::vector<double> R;

    explicit Objective(const gbx_objective* obj) : o(obj), n(obj->n), R(obj->n) {}

    bool graph() const { return o->kind == GBX_OBJ_GRAPH_MATCHING; }

    void residual(const double* X, double* out) const {
        const int m = o->order;
        const double* A = o->A;
        const double* B = o->B;
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < m; ++j) {
                double r = 0.0;
                for (int k = 0; k < m; ++k) {
                    r = std::fma(A[i * m + k], X[k * m + j], r);
                    r = std::fma(-X[i * m + k], B[k * m + j], r);
                }
                out[i * m + j] = r;
            }
    }

    // gradient; for graph matching R holds the residual of x afterwards.
    void grad(const double* x, double* g) const {
        if (graph()) {
            const int m = o->order;
            residual(x, R.data());
            const double two_s = 2.0 * o->scale;
            for (int p = 0; p < m; ++p)
                for (int q = 0; q < m; ++q) {
                    double acc = 0.0;
                    for (int r = 0; r < m; ++r)
                        acc = std::fma(o->A[r * m + p], R[r * m + q], acc);
                    for (int c = 0; c < m; ++c)
                        acc = std::fma(-R[p * m + c], o->B[q * m + c], acc);
                    g[p * m + q] = two_s * acc;
                }
            return;
        }
        for (int j = 0; j < n; ++j) {
            double acc = 0.0;
            for (int k = 0; k < n; ++k)
                acc = std::fma(o->Q[(size_t)k * n + j], x[k], acc);
            const double lin = o->c ? o->linear_scale * o->c[j] : 0.0;
            g[j] = o->scale * (acc + lin);
        }
    }

    double value_from_residual() const {
        Lanes L;
        for (int l = 0; l < kLanes; ++l) {
            double loc = 0.0;
            for (int e = l; e < n; e += kLanes) loc = std::fma(R[e], R[e], loc);
            L.v[l] = loc;
        }
        return o->scale * reduce_sum(L);
    }

    double value(const double* x) const {
        if (graph()) {
            residual(x, R.data());
            return value_from_residual();
        }
        const double a = 0.5 * o->scale;
        const double b = o->scale * o->linear_scale;
        Lanes L;
        for (int l = 0; l < kLanes; ++l) {
            double quad = 0.0, lin = 0.0;
            for (int j = l; j < n; j += kLanes) {
                double qx = 0.0;
                for (int k = 0; k < n; ++k)
                    qx = std::fma(o->Q[(size_t)k * n + j], x[k], qx);
                quad = std::fma(x[j], qx, quad);
                if (o->c) lin = std::fma(o->c[j], x[j], lin);
            }
            double val = a * quad + b * lin;
            if (l == 0) val += o->constant;
            L.v[l] = val;
        }
        return reduce_sum(L);
    }

    // f(x) from the gradient g just evaluated at x, for the incumbent cutoff
    // (the kernel's value_at_grad: graph matching from the residual, dense
    // quadratic as x'g/2 + s l c'x/2 + k, lane order of the reductions)
    double value_at_grad(const double* x, const double* g) const {
        if (graph()) return value_from_residual();
        const double hb = 0.5 * o->scale * o->linear_scale;
        Lanes L;
        for (int l = 0; l < kLanes; ++l) {
            double loc = 0.0;
            for (int j = l; j < n; j += kLanes) {
                loc = std::fma(0.5 * x[j], g[j], loc);
                if (o->c) loc = std::fma(hb * o->c[j], x[j], loc);
            }
            L.v[l] = loc;
        }
        return reduce_sum(L) + o->constant;
    }

    // value at the point whose gradient was just evaluated
    double value_after_grad(const double* x) const {
        return graph() ? value_from_residual() : value(x);
    }

    double curvature(const double* d) const {
        Lanes L;
        if (graph()) {
            residual(d, R.data());
            for (int l = 0; l < kLanes; ++l) {
                double loc = 0.0;
                for (int e = l; e < n; e += kLanes) loc = std::fma(R[e], R[e], loc);
                L.v[l] = loc;
            }
            return (2.0 * o->scale) * reduce_sum(L);
        }
        for (int l = 0; l < kLanes; ++l) {
            double curv = 0.0;
            for (int j = l; j < n; j += kLanes) {
                double prod = 0.0;
                for (int k = 0; k < n; ++k)
                    prod = std::fma(o->Q[(size_t)k * n + j], d[k], prod);
                curv = std::fma(o->scale * d[j], prod, curv);
            }
            L.v[l] = curv;
        }
        return reduce_sum(L);
    }
};

// ---------------------------------------------------------------- LMOs
int next_pow2(int v) { int r = 1; while (r < v) r <<= 1; return r; }

struct LMO {
    const gbx_lmo* l;
    int n;
    explicit LMO(const gbx_lmo* lmo) : l(lmo), n(lmo->n) {}
    bool eq() const { return l->kind == GBX_LMO_EQUALITY_SIMPLEX; }
    bool simplex() const {
        return l->kind == GBX_LMO_SIMPLEX || l->kind == GBX_LMO_EQUALITY_SIMPLEX;
    }
    bool isint(int j) const { return l->is_int && l->is_int[j]; }

    // parallel_greedy_allocate_cooperative (lmo.cuh:529-618), run sequentially.
    void greedy(const double* g, const double* ub, double* out,
                const unsigned char* fixed, double remaining, bool force_full,
                bool floor_int) const {
        const int S = next_pow2(n);
        std::vector<double> key(S), prefix(S);
        std::vector<int> idx(S);
        for (int pos = 0; pos < S; ++pos) {
            const bool el = pos < n && (!fixed || !fixed[pos])
                && (force_full || g[pos] <= 0.0);
            key[pos] = el ? g[pos] : kInf;
            idx[pos] = el ? pos : -1;
        }
        for (int width = 2; width <= S; width <<= 1)
            for (int stride = width >> 1; stride > 0; stride >>= 1)
                for (int left = 0; left < S; ++left) {
                    const int right = left ^ stride;
                    if (right <= left) continue;
                    const double lk = key[left], rk = key[right];
                    const int li = idx[left], ri = idx[right];
                    const bool after = rk < lk || (rk == lk && ri >= 0 && (li < 0 || ri < li));
                    const bool asc = (left & width) == 0;
                    if (after == asc) {
                        key[left] = rk; key[right] = lk;
                        idx[left] = ri; idx[right] = li;
                    }
                }
        for (int pos = 0; pos < S; ++pos) {
            const int j = idx[pos];
            prefix[pos] = j < 0 ? 0.0 : (isint(j) ? std::fmax(ub[j] - out[j], 0.0) : remaining);
        }
        for (int off = 1; off < S; off <<= 1)
            for (int op = 0; op < S / (off << 1); ++op) {
                const int right = (op + 1) * (off << 1) - 1;
                prefix[right] += prefix[right - off];
            }
        prefix[S - 1] = 0.0;
        for (int off = S >> 1; off > 0; off >>= 1)
            for (int op = 0; op < S / (off << 1); ++op) {
                const int right = (op + 1) * (off << 1) - 1;
                const double ls = prefix[right - off];
                prefix[right - off] = prefix[right];
                prefix[right] += ls;
            }
        for (int pos = 0; pos < S; ++pos) {
            const int j = idx[pos];
            if (j < 0) continue;
            double add = std::fmax(remaining - prefix[pos], 0.0);
            const double cap = isint(j) ? std::fmax(ub[j] - out[j], 0.0) : remaining;
            add = std::fmin(add, cap);
            if (floor_int && isint(j)) add = std::floor(add + (eq() ? 1e-9 : 0.0));
            out[j] += add;
        }
    }

    // ---- Birkhoff: shortest-augmenting-path Hungarian (lmo.cuh:1239-1417)
    bool hungarian(const double* cost, const double* lb, const double* ub,
                   double* out, const double* face) const {
        const int m = l->order;
        std::vector<int> fcol(m, -1), frow(m, -1), rows(m), cols(m);
        bool valid = true;
        for (int r = 0; r < m && valid; ++r)
            for (int c = 0; c < m; ++c) {
                const int e = r * m + c;
                if (lb[e] > ub[e] + 1e-9) { valid = false; break; }
                const bool ff = face && face[e] >= 1.0 - 1e-9;
                if (lb[e] > 0.5 || ff) {
                    if (ub[e] < 0.5 || fcol[r] >= 0 || frow[c] >= 0) { valid = false; break; }
                    fcol[r] = c; frow[c] = r; out[e] = 1.0;
                }
            }
        if (!valid) return false;
        int k = 0, kc = 0;
        for (int i = 0; i < m; ++i) {
            if (fcol[i] < 0) rows[k++] = i;
            if (frow[i] < 0) cols[kc++] = i;
        }
        if (k != kc) return false;
        std::vector<double> u(k + 1, 0.0), v(k + 1, 0.0), minv(k + 1);
        std::vector<int> p(k + 1, 0), way(k + 1, 0);
        std::vector<unsigned char> used(k + 1);
        for (int i = 1; i <= k; ++i) {
            p[0] = i;
            int j0 = 0;
            std::fill(minv.begin(), minv.end(), kNone);
            std::fill(used.begin(), used.end(), 0);
            for (;;) {
                used[j0] = 1;
                const int i0 = p[j0];
                for (int j = 1; j <= k; ++j) {
                    if (used[j]) continue;
                    const int e = rows[i0 - 1] * m + cols[j - 1];
                    if (ub[e] >= 0.5 && (!face || face[e] > 1e-9)) {
                        const double cur = cost[e] - u[i0] - v[j];
                        if (cur < minv[j]) { minv[j] = cur; way[j] = j0; }
                    }
                }
                double delta = kNone;
                int j1 = -1;
                for (int j = 1; j <= k; ++j) {
                    if (used[j] || !(minv[j] < kNone)) continue;
                    if (j1 < 0 || minv[j] < delta) { delta = minv[j]; j1 = j; }
                }
                if (j1 < 0 || !std::isfinite(delta)) return false;
                for (int j = 0; j <= k; ++j) {
                    if (used[j]) { u[p[j]] += delta; v[j] -= delta; }
                    else minv[j] -= delta;
                }
                j0 = j1;
                if (p[j0] == 0) break;
            }
            do { const int j1 = way[j0]; p[j0] = p[j1]; j0 = j1; } while (j0 != 0);
        }
        for (int j = 1; j <= k; ++j) out[rows[p[j] - 1] * m + cols[j - 1]] = 1.0;
        return true;
    }

    // ---- cardinality-linked simplex (the portfolio set; no reference counterpart):
    // x = (w, z), sum w = 1, 0 <= w <= z, sum z <= K. Vertex = w on one asset a
    // plus z on the forced assets and on the most negative free z-costs while
    // slots remain; values summed in the kernel's order (base over forced
    // assets by index, prefix sums over the sorted free negatives).
    bool card_forward(const double* g, const double* lb, const double* ub, double* v) const {
        const int N = n / 2;
        const int K = (int)std::floor(l->right_side + 1e-9);
        for (int j = 0; j < n; ++j) v[j] = 0.0;
        std::vector<int> ord, pos(N, -1);
        int nf = 0;
        double base = 0.0;
        for (int j = 0; j < N; ++j) {
            if (lb[N + j] > 0.5) { ++nf; base = base + g[N + j]; }
            else if (!(ub[N + j] < 0.5) && g[N + j] < 0.0) ord.push_back(j);
        }
        std::sort(ord.begin(), ord.end(), [&](int a, int b) {
            return g[N + a] < g[N + b] || (g[N + a] == g[N + b] && a < b);
        });
        const int nl = (int)ord.size();
        for (int t = 0; t < nl; ++t) pos[ord[t]] = t;
        std::vector<double> P(nl + 1, 0.0);
        for (int t = 0; t < nl; ++t) P[t + 1] = P[t] + g[N + ord[t]];
        if (nf > K) return false;
        const int r0 = K - nf, r1 = K - nf - 1;
        auto value = [&](int a) -> double {
            if (ub[N + a] < 0.5) return kInf;
            const double head = g[a] + base;
            double val;
            if (lb[N + a] > 0.5) val = head + P[std::min(r0, nl)];
            else if (r1 < 0) return kInf;
            else if (pos[a] >= 0 && pos[a] < r1) val = head + P[std::min(r1 + 1, nl)];
            else val = head + (g[N + a] + P[std::min(r1, nl)]);
            return val < kInf ? val : kInf;
        };
        double vmin = kInf;
        int a = -1;
        for (int i = 0; i < N; ++i) {
            const double val = value(i);
            if (val < vmin) { vmin = val; a = i; }
        }
        if (a < 0) return false;
        int limit;
        if (lb[N + a] > 0.5) limit = std::min(r0, nl);
        else if (pos[a] >= 0 && pos[a] < r1) limit = std::min(r1 + 1, nl);
        else limit = std::min(r1, nl);
        for (int j = 0; j < N; ++j)
            if (lb[N + j] > 0.5 || (pos[j] >= 0 && pos[j] < limit) || j == a) v[N + j] = 1.0;
        v[a] = 1.0;
        return true;
    }

    // ---- linked cardinality (LinkedCardinalityLMO, examples/sparse_sharpe.cu:266-546):
    // x = (v, y), y at n/2, the first `order` assets active, 0 <= v <= U y, sum y <= m
    bool linked() const { return l->kind == GBX_LMO_LINKED_CARDINALITY; }
    int lhalf() const { return n / 2; }
    int lassets() const { return l->order > 0 ? std::min(l->order, n / 2) : n / 2; }
    int lm() const { return (int)std::floor(l->right_side + 1e-9); }

    // compute_v: mandatory y, then the cheapest negative joint costs
    // g_y + min(0, U g_v) by (cost, asset) while slots remain
    void linked_forward(const double* g, const double* lb, const double* ub, double* v) const {
        const int h = lhalf(), A = lassets(), m = lm();
        for (int j = 0; j < n; ++j) v[j] = 0.0;
        int mand = 0;
        for (int i = 0; i < A; ++i) mand += lb[h + i] > 0.5 ? 1 : 0;
        if (mand > m) return;
        std::vector<std::pair<double, int>> opt;
        for (int i = 0; i < A; ++i) {
            const double ci = g[h + i] + std::fmin(0.0, l->upper[i] * g[i]);
            if (ci < 0.0 && lb[h + i] <= 0.5 && ub[h + i] > 0.5) opt.push_back({ci, i});
        }
        std::sort(opt.begin(), opt.end());
        for (int i = 0; i < A; ++i)
            if (lb[h + i] > 0.5) { v[h + i] = 1.0; v[i] = g[i] < 0.0 ? l->upper[i] : 0.0; }
        for (int r = 0; r < (int)opt.size() && r < m - mand; ++r) {
            const int i = opt[r].second;
            v[h + i] = 1.0;
            v[i] = g[i] < 0.0 ? l->upper[i] : 0.0;
        }
    }

    // compute_inface_v on the direction gd (the away step passes -g)
    void linked_inface(const double* gd, const double* x, const double* lb, const double* ub, double* a) const {
        const double atol = 1e-6, rtol = 1e-4;
        const int h = lhalf(), A = lassets(), m = lm();
        const double* U = l->upper;
        for (int j = 0; j < n; ++j) a[j] = 0.0;
        std::vector<unsigned char> yf(A), vz(A), la(A);
        int fixed_sel = 0;
        Lanes SY;
        for (int t = 0; t < kLanes; ++t) {
            double sy = 0.0;
            for (int i = t; i < A; i += kLanes) sy += x[h + i];
            SY.v[t] = sy;
        }
        for (int i = 0; i < A; ++i) {
            const double vi = x[i], yi = x[h + i];
            const bool lo = std::fabs(yi - lb[h + i]) <= atol + rtol * std::fmax(std::fabs(yi), std::fabs(lb[h + i]));
            const bool up = std::fabs(yi - ub[h + i]) <= atol + rtol * std::fmax(std::fabs(yi), std::fabs(ub[h + i]));
            yf[i] = lo || up;
            vz[i] = std::fabs(vi) <= atol + rtol * std::fabs(vi);
            la[i] = std::fabs(vi - U[i] * yi) <= atol + rtol * std::fmax(std::fabs(vi), std::fabs(U[i] * yi));
            if (yf[i]) {
                const double fy = lo ? lb[h + i] : ub[h + i];
                a[h + i] = fy;
                if (fy > 0.5) ++fixed_sel;
                if (!vz[i]) a[i] = la[i] ? U[i] * fy : (gd[i] < 0.0 ? U[i] * fy : 0.0);
            }
        }
        const double sum_y = reduce_sum(SY);
        const bool full = std::fabs(sum_y - m) <= atol + rtol * std::fmax(std::fabs(sum_y), (double)m);
        std::vector<std::pair<double, int>> opt;
        for (int i = 0; i < A; ++i) {
            if (yf[i]) continue;
            double ci = gd[h + i];
            if (la[i]) ci += U[i] * gd[i];
            else if (!vz[i]) ci += std::fmin(0.0, U[i] * gd[i]);
            if (full || ci < 0.0) opt.push_back({ci, i});
        }
        std::sort(opt.begin(), opt.end());
        for (int r = 0; r < (int)opt.size() && r < m - fixed_sel; ++r) {
            const int i = opt[r].second;
            a[h + i] = 1.0;
            a[i] = la[i] ? U[i] : (!vz[i] ? (gd[i] < 0.0 ? U[i] : 0.0) : 0.0);
        }
    }

    void forward(const double* g, const double* lb, const double* ub, double* v) const {
        if (linked()) {
            linked_forward(g, lb, ub, v);
        } else if (l->kind == GBX_LMO_CARDINALITY) {
            card_forward(g, lb, ub, v);
        } else if (l->kind == GBX_LMO_BOX) {
            for (int j = 0; j < n; ++j) v[j] = g[j] > 0.0 ? lb[j] : ub[j];
        } else if (simplex()) {
            Lanes L;
            for (int t = 0; t < kLanes; ++t) {
                double loc = 0.0;
                for (int j = t; j < n; j += kLanes) {
                    if (isint(j)) { v[j] = lb[j]; loc += v[j]; }
                    else v[j] = 0.0;
                }
                L.v[t] = loc;
            }
            const double mass = reduce_sum(L);
            const double remaining = l->right_side - mass;
            greedy(g, ub, v, nullptr, remaining, eq(), eq());
        } else {
            for (int j = 0; j < n; ++j) v[j] = 0.0;
            if (n != l->order * l->order) return;
            hungarian(g, lb, ub, v, nullptr);
        }
    }

    void inface(const double* g, const double* x, const double* lb,
                const double* ub, double* a) const {
        const double atol = 1e-6, rtol = 1e-4;
        if (linked()) {
            linked_inface(g, x, lb, ub, a);
        } else if (l->kind == GBX_LMO_BOX) {
            for (int j = 0; j < n; ++j) {
                const double ut = atol + rtol * std::fabs(ub[j]);
                const double lt = atol + rtol * std::fabs(lb[j]);
                if (std::fabs(x[j] - ub[j]) <= ut) a[j] = ub[j];
                else if (std::fabs(x[j] - lb[j]) <= lt) a[j] = lb[j];
                else a[j] = g[j] > 0.0 ? lb[j] : ub[j];
            }
        } else if (simplex()) {
            std::vector<unsigned char> fixed(n, 0);
            Lanes LM, LX;
            for (int t = 0; t < kLanes; ++t) {
                double lm = 0.0, lx = 0.0;
                for (int j = t; j < n; j += kLanes) {
                    fixed[j] = 0;
                    a[j] = isint(j) ? lb[j] : 0.0;
                    const double lower = isint(j) ? lb[j] : 0.0;
                    const double ltol = atol + rtol * std::fmax(std::fabs(x[j]), std::fabs(lower));
                    if (std::fabs(x[j] - lower) <= ltol) {
                        fixed[j] = 1; a[j] = lower;
                    } else if (isint(j)) {
                        const double utol = atol + rtol * std::fmax(std::fabs(x[j]), std::fabs(ub[j]));
                        if (std::fabs(x[j] - ub[j]) <= utol) { fixed[j] = 1; a[j] = ub[j]; }
                    }
                    lm += a[j];
                    lx += x[j];
                }
                LM.v[t] = lm; LX.v[t] = lx;
            }
            const double mass = reduce_sum(LM);
            const double xmass = reduce_sum(LX);
            const double remaining = l->right_side - mass;
            const bool force = eq() || std::fabs(xmass - l->right_side)
                <= atol + rtol * std::fmax(std::fabs(xmass), std::fabs(l->right_side));
            greedy(g, ub, a, fixed.data(), remaining, force, true);
        } else {
            for (int j = 0; j < n; ++j) a[j] = 0.0;
            if (n != l->order * l->order) return;
            hungarian(g, lb, ub, a, x);
        }
    }

    // min over coordinates of the feasible step for x - gamma*d, folded with
    // the aggregate constraint, clipped at 0 (device_resident_solver.cuh:533-545)
    double max_step(const double* d, const double* x, const double* lb,
                    const double* ub) const {
        if (linked()) {
            // dicg_maximum_step_local and dicg_sum_maximum_step
            const int h = lhalf(), A = lassets(), m = lm();
            const double tol = 1e-9;
            Lanes R, SX, SD;
            for (int t = 0; t < kLanes; ++t) {
                double res = 1.0, sx = 0.0, sd = 0.0;
                for (int i = t; i < A; i += kLanes) {
                    const double dv = d[i], dy = d[h + i], U = l->upper[i];
                    if (dv > tol) res = std::fmin(res, x[i] / dv);
                    const double link_d = dv - U * dy, link_x = x[i] - U * x[h + i];
                    if (link_d < -tol) res = std::fmin(res, link_x / link_d);
                    if (dy > tol) res = std::fmin(res, (x[h + i] - lb[h + i]) / dy);
                    else if (dy < -tol) res = std::fmin(res, (ub[h + i] - x[h + i]) / -dy);
                    sx += x[h + i];
                    sd += dy;
                }
                R.v[t] = res; SX.v[t] = sx; SD.v[t] = sd;
            }
            const double coord = reduce_min(R);
            const double sum_x = reduce_sum(SX), sum_d = reduce_sum(SD);
            const double agg = sum_d < -1e-9 ? std::fmax(0.0, std::fmin(1.0, (sum_x - m) / sum_d)) : 1.0;
            return std::fmax(0.0, std::fmin(coord, agg));
        }
        Lanes L;
        for (int t = 0; t < kLanes; ++t) {
            double res = 1.0;
            for (int j = t; j < n; j += kLanes) {
                const double dj = d[j];
                if (simplex()) {
                    const double tol = 1e-6;
                    if (dj > tol) res = std::fmin(res, (x[j] - (isint(j) ? lb[j] : 0.0)) / dj);
                    else if (dj < -tol)
                        res = std::fmin(res, ((isint(j) ? ub[j] : l->right_side) - x[j]) / -dj);
                } else if (l->kind == GBX_LMO_BOX) {
                    if (dj < 0.0) res = std::fmin(res, (ub[j] - x[j]) / -dj);
                    else if (dj > 0.0) res = std::fmin(res, (x[j] - lb[j]) / dj);
                } else {
                    if (dj > 0.0) res = std::fmin(res, (x[j] - lb[j]) / dj);
                    else if (dj < 0.0) res = std::fmin(res, (ub[j] - x[j]) / -dj);
                }
            }
            L.v[t] = res;
        }
        const double coord = reduce_min(L);
        double agg = 1.0;
        if (simplex()) {
            Lanes SX, SD;
            for (int t = 0; t < kLanes; ++t) {
                double sx = 0.0, sd = 0.0;
                for (int j = t; j < n; j += kLanes) { sx += x[j]; sd += d[j]; }
                SX.v[t] = sx; SD.v[t] = sd;
            }
            const double sum_x = reduce_sum(SX);
            const double sum_d = reduce_sum(SD);
            if (eq() && std::fabs(sum_d) > 1e-9) agg = 0.0;
            else agg = sum_d < 0.0 ? std::fmin(1.0, (sum_x - l->right_side) / sum_d) : 1.0;
        }
        return std::fmax(0.0, std::fmin(coord, agg));
    }

    bool check_feasible(const double* lb, const double* ub, const uint8_t* flags) const {
        if (l->kind == GBX_LMO_BOX) return true;
        if (linked()) {
            int mand = 0;
            for (int i = 0; i < lassets(); ++i) mand += lb[lhalf() + i] > 0.5 ? 1 : 0;
            return mand <= lm();
        }
        if (l->kind == GBX_LMO_CARDINALITY) {
            const int N = n / 2;
            const int K = (int)std::floor(l->right_side + 1e-9);
            int nf = 0;
            bool open = false;
            for (int j = 0; j < N; ++j) {
                nf += lb[N + j] > 0.5 ? 1 : 0;
                open = open || !(ub[N + j] < 0.5);
            }
            return nf <= K && (nf >= 1 || (K >= 1 && open));
        }
        if (simplex()) {
            bool valid = true, cont = false;
            Lanes LM, LC;
            for (int t = 0; t < kLanes; ++t) {
                double mand = 0.0, cap = 0.0;
                for (int j = t; j < n; j += kLanes) {
                    const bool integer = flags ? flags[j] != 0 : isint(j);
                    const double lo = integer ? std::ceil(std::fmax(0.0, lb[j])) : std::fmax(0.0, lb[j]);
                    const double hi = integer ? std::floor(ub[j]) : ub[j];
                    valid = valid && lo <= hi;
                    mand += lo; cap += hi;
                    cont = cont || !integer;
                }
                LM.v[t] = mand; LC.v[t] = cap;
            }
            const double ms = reduce_sum(LM);
            bool feas = valid && ms <= l->right_side + 1e-9;
            if (eq()) {
                const double cs = reduce_sum(LC);
                feas = feas && cs >= l->right_side - 1e-9
                    && (cont || std::fabs(l->right_side - std::round(l->right_side)) <= 1e-9);
            }
            return feas;
        }
        if (n != l->order * l->order) return false;
        std::vector<double> zero(n, 0.0), out(n, 0.0);
        return hungarian(zero.data(), lb, ub, out.data(), nullptr);
    }

    bool rounded_feasible(const double* x, double tol) const {
        if (l->kind == GBX_LMO_BOX) return true;
        if (linked()) {
            // candidate_feasible_device: 0 <= v <= U y, sum y <= m
            const int h = lhalf(), A = lassets();
            bool valid = true;
            Lanes SY;
            for (int t = 0; t < kLanes; ++t) {
                double sy = 0.0;
                for (int i = t; i < A; i += kLanes) {
                    valid = valid && x[i] >= -tol && x[i] <= l->upper[i] * x[h + i] + tol;
                    sy += x[h + i];
                }
                SY.v[t] = sy;
            }
            return valid && reduce_sum(SY) <= lm() + tol;
        }
        if (l->kind == GBX_LMO_CARDINALITY) {
            const int N = n / 2;
            bool valid = true;
            Lanes SW, SZ;
            for (int t = 0; t < kLanes; ++t) {
                double sw = 0.0, sz = 0.0;
                for (int j = t; j < N; j += kLanes) {
                    const double w = x[j], z = x[N + j];
                    valid = valid && w >= -tol && z >= -tol && z <= 1.0 + tol && w <= z + tol;
                    sw += w;
                    sz += z;
                }
                SW.v[t] = sw; SZ.v[t] = sz;
            }
            const double sum_w = reduce_sum(SW), sum_z = reduce_sum(SZ);
            return valid && std::fabs(sum_w - 1.0) <= tol && sum_z <= std::floor(l->right_side + 1e-9) + tol;
        }
        if (simplex()) {
            bool valid = true;
            Lanes L;
            for (int t = 0; t < kLanes; ++t) {
                double s = 0.0;
                for (int j = t; j < n; j += kLanes) { valid = valid && x[j] >= -tol; s += x[j]; }
                L.v[t] = s;
            }
            const double sum = reduce_sum(L);
            return valid && (eq() ? std::fabs(sum - l->right_side) <= tol
                                  : sum <= l->right_side + tol);
        }
        const int m = l->order;
        if (n != m * m) return false;
        bool valid = true;
        for (int i = 0; i < m; ++i) {
            double row = 0.0, col = 0.0;
            for (int j = 0; j < m; ++j) {
                if (x[i * m + j] < -tol) valid = false;
                row += x[i * m + j];
                col += x[j * m + i];
            }
            if (std::fabs(row - 1.0) > tol || std::fabs(col - 1.0) > tol) valid = false;
        }
        return valid;
    }
};

// ---------------------------------------------------------------- node relax
struct Relaxer {
    Objective obj;
    LMO lmo;
    const gbx_algorithm* alg;
    int n;
    std::vector<double> g, v, a, tx, tg, cand;

    Relaxer(const gbx_objective* o, const gbx_lmo* l, const gbx_algorithm* al)
        : obj(o), lmo(l), alg(al), n(o->n), g(n), v(n), a(n), tx(n), tg(n), cand(n) {}

    bool dicg() const { return alg->kind == GBX_ALG_DICG; }

    double dot_gap(const double* gr, const double* x, const double* vv) const {
        Lanes L;
        for (int t = 0; t < kLanes; ++t) {
            double loc = 0.0;
            for (int j = t; j < n; j += kLanes) loc = std::fma(gr[j], x[j] - vv[j], loc);
            L.v[t] = loc;
        }
        return reduce_sum(L);
    }

    // integer_candidate_device of the linked cardinality LMO: mandatory assets,
    // then the largest positive v of x up to m (or the asset of largest
    // mu = -ls c), scaled to the objective's minimum along the direction,
    // t = -ls c'd / d'Qd, capped by U_i / d_i; assets in order
    void linked_candidate(const double* x, const double* lb, const double* ub, double* cand) const {
        const int h = lmo.lhalf(), A = lmo.lassets(), m = lmo.lm();
        const gbx_objective* o = obj.o;
        const double* U = lmo.l->upper;
        for (int j = 0; j < n; ++j) cand[j] = 0.0;
        auto mu = [&](int i) { return o->c ? -o->linear_scale * o->c[i] : 0.0; };
        int selected = 0;
        for (int i = 0; i < A; ++i)
            if (lb[h + i] > 0.5) { cand[h + i] = 1.0; ++selected; }
        while (selected < m) {
            int best = -1;
            for (int i = 0; i < A; ++i)
                if (cand[h + i] == 0.0 && ub[h + i] > 0.5 && x[i] > 1e-12 && (best < 0 || x[i] > x[best])) best = i;
            if (best < 0) break;
            cand[h + best] = 1.0;
            ++selected;
        }
        bool direction = false;
        for (int i = 0; i < A; ++i)
            if (cand[h + i] == 1.0) {
                cand[i] = std::fmax(0.0, x[i]);
                direction = direction || cand[i] > 0.0;
            }
        if (!direction) {
            int best = -1;
            for (int i = 0; i < A; ++i)
                if ((cand[h + i] == 1.0 || (selected < m && ub[h + i] > 0.5)) && (best < 0 || mu(i) > mu(best)))
                    best = i;
            if (best >= 0 && mu(best) > 0.0) {
                cand[h + best] = 1.0;
                cand[best] = 1.0;
            }
        }
        double lin = 0.0, quad = 0.0, cap = kInf;
        for (int i = 0; i < A; ++i) {
            lin += mu(i) * cand[i];
            if (cand[i] > 0.0) cap = std::fmin(cap, U[i] / cand[i]);
            for (int j = 0; j < A; ++j) quad += cand[i] * o->Q[(size_t)i * n + j] * cand[j];
        }
        const double t = lin > 0.0 && quad > 0.0 ? std::fmin(lin / quad, cap) : 0.0;
        for (int i = 0; i < A; ++i) cand[i] *= t;
    }

    double integer_value(const double* x, const double* lb, const double* ub,
                         const uint8_t* flags, double tol) const {
        for (int j = 0; j < n; ++j)
            if (!std::isfinite(x[j]) || x[j] < lb[j] - tol || x[j] > ub[j] + tol
                    || (flags && flags[j] && x[j] != std::round(x[j])))
                return kNone;
        const double val = obj.value(x);
        return std::isfinite(val) ? val : kNone;
    }

    // SecantLS::search (algorithms.cuh:121-258)
    double secant(double gap, double maxg, const double* x, const double* dir) {
        const double tol = alg->secant_tol, deps = alg->secant_denom_eps;
        const double f_base = obj.value(x);
        double lo = 0.0, hi = maxg, best_f = f_base, best_gamma = 0.0;
        double phi_lo = -gap, phi_hi = 0.0, gamma = 0.0;
        bool done = phi_lo >= -tol;
        auto probe = [&](double gm, double& phi, double& f) {
            for (int j = 0; j < n; ++j) tx[j] = std::fma(gm, dir[j], x[j]);
            obj.grad(tx.data(), tg.data());
            Lanes L;
            for (int t = 0; t < kLanes; ++t) {
                double loc = 0.0;
                for (int j = t; j < n; j += kLanes) loc = std::fma(tg[j], dir[j], loc);
                L.v[t] = loc;
            }
            phi = reduce_sum(L);
            f = obj.value_after_grad(tx.data());
        };
        double f_hi;
        probe(maxg, phi_hi, f_hi);
        {
            const double f_abs = f_base >= 0.0 ? f_base : -f_base;
            const double allow = tol * (1.0 + f_abs);
            if (f_hi < best_f || (best_gamma == 0.0 && f_hi <= f_base + allow)) {
                best_f = f_hi; best_gamma = maxg;
            }
            if (!done && phi_hi <= tol && f_hi <= f_base + allow) { gamma = maxg; done = true; }
        }
        for (int it = 0; it < alg->secant_iters; ++it) {
            if (done) break;
            const double denom = phi_hi - phi_lo;
            double gm = (denom > deps || denom < -deps)
                ? hi - phi_hi * (hi - lo) / denom : 0.5 * (lo + hi);
            if (!(gm > lo && gm < hi)) gm = 0.5 * (lo + hi);
            gamma = gm;
            double phi, ft;
            probe(gamma, phi, ft);
            const double f_abs = f_base >= 0.0 ? f_base : -f_base;
            const double allow = tol * (1.0 + f_abs);
            if (ft < best_f || (best_gamma == 0.0 && ft <= f_base + allow)) {
                best_f = ft; best_gamma = gamma;
            }
            if (phi < 0.0) { lo = gamma; phi_lo = phi; }
            else { hi = gamma; phi_hi = phi; }
            if ((phi <= tol && phi >= -tol) || (hi - lo) <= tol) {
                gamma = 0.5 * (lo + hi); done = true;
            }
        }
        const double f_abs = f_base >= 0.0 ? f_base : -f_base;
        const double allow = tol * (1.0 + f_abs);
        if (best_gamma > 0.0 && best_f <= f_base + allow) gamma = best_gamma;
        else if (!done) gamma = 0.0;
        return gamma;
    }

    static double quad_step(double gap, double curv, double maximum) {
        if (maximum <= 0.0) return 0.0;
        if (curv > 0.0) {
            if (gap <= 0.0) return 0.0;
            const double s = gap / curv;
            return s < maximum ? s : maximum;
        }
        return -gap + 0.5 * curv * maximum < 0.0 ? maximum : 0.0;
    }

    bool uses_search() const {
        return alg->line_search == GBX_LS_SECANT || alg->line_search == GBX_LS_QUADRATIC_EXACT;
    }

    double search(double gap, double maxg, const double* x, const double* dir) {
        if (alg->line_search == GBX_LS_QUADRATIC_EXACT)
            return quad_step(gap, obj.curvature(dir), maxg);
        return secant(gap, maxg, x, dir);
    }

    // one node: drs_fw_relax_node
    void relax(int node, const gbx_node_batch* b) {
        const size_t off = (size_t)node * n;
        double* x = b->x + off;
        const double* lb = b->lb + off;
        const double* ub = b->ub + off;
        double* best = b->best_vertex + off;
        const uint8_t* flags = b->integer_flags;
        const double tol = b->candidate_tol;
        const double eps = b->eps[node];
        const int it0 = b->iterations[node];
        const bool supplied = (b->status[node] & GBX_NODE_INITIAL_POINT_SUPPLIED) != 0;
        double best_val = kNone;
        b->best_vertex_val[node] = kNone;
        b->iterations[node] = it0;

        // drs_node_feasible
        bool valid = true;
        for (int j = 0; j < n; ++j)
            if (std::isnan(lb[j]) || std::isnan(ub[j]) || lb[j] > ub[j]
                    || (flags && flags[j] && std::ceil(lb[j]) > std::floor(ub[j])))
                valid = false;
        if (!valid || !lmo.check_feasible(lb, ub, flags)) {
            b->status[node] = GBX_NODE_INFEASIBLE;
            b->value[node] = kInf;
            b->gap[node] = 0.0;
            return;
        }
        if (it0 == 0 && !supplied) {
            for (int j = 0; j < n; ++j) g[j] = -1.0 - static_cast<double>(j) / (n + 1.0);
            lmo.forward(g.data(), lb, ub, v.data());
            for (int j = 0; j < n; ++j) x[j] = v[j];
        }
        auto score = [&](const double* vert) {
            const double fv = integer_value(vert, lb, ub, flags, tol);
            if (fv < best_val) { best_val = fv; b->best_vertex_val[node] = fv; }
            if (fv < 1e299 && fv == best_val)
                for (int j = 0; j < n; ++j) best[j] = vert[j];
        };
        const int ls = alg->line_search;
        // incumbent cutoff (gbx_node_batch.cutoff): stop once the FW bound
        // f - gap clears it, after at least one step of this dispatch
        const double cutv = b->cutoff ? *b->cutoff : kInf;
        for (int iter = 0; iter < b->max_iters; ++iter) {
            b->iterations[node] = it0 + iter + 1;
            obj.grad(x, g.data());
            const double fcut = (cutv < kInf && iter > 0) ? obj.value_at_grad(x, g.data()) : 0.0;
            lmo.forward(g.data(), lb, ub, v.data());
            score(v.data());
            const double gap = dot_gap(g.data(), x, v.data());
            const bool done = gap >= 0.0 && gap < eps;
            b->gap[node] = gap;
            b->status[node] = done ? 1 : 0;
            if (done) break;
            if (cutv < kInf && iter > 0 && fcut - gap >= cutv) break;
            if (!dicg()) {
                if (uses_search()) {
                    for (int j = 0; j < n; ++j) v[j] -= x[j];
                    const double gm = search(gap, 1.0, x, v.data());
                    for (int j = 0; j < n; ++j) x[j] = std::fma(gm, v[j], x[j]);
                } else {
                    const double gm = 2.0 / (double)(it0 + iter + 2);
                    for (int j = 0; j < n; ++j) x[j] = std::fma(gm, v[j] - x[j], x[j]);
                }
                continue;
            }
            for (int j = 0; j < n; ++j) g[j] = -g[j];
            lmo.inface(g.data(), x, lb, ub, a.data());
            score(a.data());
            for (int j = 0; j < n; ++j) { g[j] = -g[j]; a[j] -= v[j]; }
            const double gmax = lmo.max_step(a.data(), x, lb, ub);
            if (uses_search()) {
                for (int j = 0; j < n; ++j) a[j] = -a[j];
                Lanes L;
                for (int t = 0; t < kLanes; ++t) {
                    double loc = 0.0;
                    for (int j = t; j < n; j += kLanes) loc = std::fma(-g[j], a[j], loc);
                    L.v[t] = loc;
                }
                const double pgap = reduce_sum(L);
                const double gm = search(pgap, gmax, x, a.data());
                for (int j = 0; j < n; ++j) x[j] = std::fma(gm, a[j], x[j]);
            } else {
                const double open = 2.0 / (double)(it0 + iter + 2);
                double gm;
                if (ls == GBX_LS_SAFEGUARDED_SCALED_OPEN_LOOP) gm = gmax <= open ? gmax : gmax * open;
                else if (ls == GBX_LS_SCALED_OPEN_LOOP) gm = gmax * open;
                else gm = std::fmin(gmax, open);
                for (int j = 0; j < n; ++j) x[j] = std::fma(-gm, a[j], x[j]);
            }
        }
        // final certificate at the returned iterate
        obj.grad(x, g.data());
        lmo.forward(g.data(), lb, ub, v.data());
        score(v.data());
        const double fgap = dot_gap(g.data(), x, v.data());
        const double fval = obj.value(x);
        b->value[node] = fval;
        b->gap[node] = fgap;
        uint8_t st = (fgap >= 0.0 && fgap < eps) ? 1 : 0;
        // rounding heuristic (the linked cardinality LMO's own candidate)
        if (flags) {
            if (lmo.linked()) linked_candidate(x, lb, ub, cand.data());
            else
                for (int j = 0; j < n; ++j) cand[j] = flags[j] ? std::round(x[j]) : x[j];
            if (lmo.rounded_feasible(cand.data(), tol)) {
                const double cv = integer_value(cand.data(), lb, ub, flags, tol);
                if (cv < b->best_vertex_val[node]) {
                    for (int j = 0; j < n; ++j) best[j] = cand[j];
                    b->best_vertex_val[node] = cv;
                }
            }
        }
        bool integral = true;
        for (int j = 0; j < n; ++j)
            if (!std::isfinite(x[j]) || (flags && flags[j] && std::fabs(x[j] - std::round(x[j])) > tol))
                integral = false;
        if (integral) st = st ? GBX_NODE_INTEGRAL_CONVERGED : GBX_NODE_INTEGRAL_UNCONVERGED;
        b->status[node] = st;
    }
};

int check_descs(const gbx_objective* o, const gbx_lmo* l, const gbx_algorithm* a) {
    if (!o || !l || !a) { g_error = "null descriptor"; return GBX_ERR_INVALID; }
    if (o->n <= 0 || l->n != o->n) { g_error = "objective/LMO size mismatch"; return GBX_ERR_INVALID; }
    if (o->kind == GBX_OBJ_GRAPH_MATCHING && o->order * o->order != o->n) {
        g_error = "graph matching order"; return GBX_ERR_INVALID;
    }
    if (o->kind != GBX_OBJ_GRAPH_MATCHING && o->kind != GBX_OBJ_DENSE_QUADRATIC) {
        g_error = "objective kind"; return GBX_ERR_UNSUPPORTED;
    }
    if (l->kind < GBX_LMO_BOX || l->kind > GBX_LMO_LINKED_CARDINALITY) { g_error = "lmo kind"; return GBX_ERR_UNSUPPORTED; }
    if (a->line_search < 0 || a->line_search > 4) { g_error = "line search"; return GBX_ERR_INVALID; }
    return GBX_OK;
}

// ---------------------------------------------------------------- B&B host
struct ONode {
    int id, parent_id, depth;
    std::vector<double> lb, ub, relaxation_x;
    int relaxation_iterations = 0;
    double dual_bound = -1e300;
};
struct MinHeap {
    bool operator()(const ONode& a, const ONode& b) const { return a.dual_bound > b.dual_bound; }
};

struct Queue {
    std::priority_queue<ONode, std::vector<ONode>, MinHeap> pq;
    void push(ONode nd) { pq.push(std::move(nd)); }
    std::vector<ONode> pop_batch(int n, double cutoff) {
        std::vector<ONode> out;
        while (!pq.empty() && (int)out.size() < n) {
            if (pq.top().dual_bound >= cutoff) { pq.pop(); continue; }
            out.push_back(pq.top()); pq.pop();
        }
        return out;
    }
    std::vector<ONode> pop_full_batch(int n, double cutoff) {
        while (!pq.empty() && pq.top().dual_bound >= cutoff) pq.pop();
        if ((int)pq.size() < n) return {};
        std::vector<ONode> out;
        for (int i = 0; i < n && !pq.empty(); ++i) {
            if (pq.top().dual_bound >= cutoff) { while (!pq.empty()) pq.pop(); break; }
            out.push_back(pq.top()); pq.pop();
        }
        if ((int)out.size() < n) { for (auto& nd : out) pq.push(std::move(nd)); return {}; }
        return out;
    }
    void discard_children(int parent) {
        decltype(pq) kept;
        while (!pq.empty()) { if (pq.top().parent_id != parent) kept.push(pq.top()); pq.pop(); }
        pq.swap(kept);
    }
    double best_bound(double cutoff) const {
        if (pq.empty()) return cutoff;
        const double b = pq.top().dual_bound;
        return b < cutoff ? b : cutoff;
    }
};

std::vector<int> top_k_infeasible(const std::vector<double>& x, const std::vector<int>& iv,
                                  int k, double tol) {
    struct C { int idx; double dist; };
    std::vector<C> c;
    for (int i : iv) {
        const double fr = x[i] - std::floor(x[i]);
        const double d = std::min(fr, 1.0 - fr);
        if (d > tol) c.push_back({i, d});
    }
    std::sort(c.begin(), c.end(), [](const C& a, const C& b) { return a.dist > b.dist; });
    const int m = std::min(k, (int)c.size());
    std::vector<int> r(m);
    for (int i = 0; i < m; ++i) r[i] = c[i].idx;
    return r;
}

std::vector<ONode> branch_pow2(const ONode& parent, int& next_id, const std::vector<double>& x,
                               const std::vector<int>& iv, int k, double tol) {
    auto vars = top_k_infeasible(x, iv, k, tol);
    if (vars.empty()) return {};
    const int ak = (int)vars.size();
    std::vector<ONode> ch;
    for (int mask = 0; mask < (1 << ak); ++mask) {
        ONode c = parent;
        c.id = next_id++;
        c.parent_id = parent.id;
        c.depth = parent.depth + 1;
        c.dual_bound = parent.dual_bound;
        c.relaxation_x.clear();
        c.relaxation_iterations = 0;
        for (int b = 0; b < ak; ++b) {
            const int vi = vars[b];
            if (mask & (1 << b)) c.lb[vi] = std::ceil(x[vi]);
            else c.ub[vi] = std::floor(x[vi]);
        }
        ch.push_back(std::move(c));
    }
    return ch;
}

double depth_tol(double root, double decay, double mn, int depth) {
    if (depth <= 0) return std::max(root, mn);
    return std::max(mn, root * std::pow(decay, depth));
}
double gap_abs(double b, double inc) { return (inc >= kInf || b <= -kInf) ? kInf : std::fabs(inc - b); }
double gap_rel(double b, double inc) {
    if (!std::isfinite(b) || !std::isfinite(inc)) return kInf;
    const double s = std::min(std::fabs(b), std::fabs(inc));
    if (s == 0.0) return kInf;
    return (inc - b) / s;
}
bool gap_ok(double b, double inc, double at, double rt) {
    if (!std::isfinite(b) || !std::isfinite(inc)) return false;
    return gap_abs(b, inc) <= at || gap_rel(b, inc) <= rt;
}
double certified_lb(double inherited, double primal, double gap) {
    if (!std::isfinite(primal) || !std::isfinite(gap) || gap < 0.0) return inherited;
    return std::max(inherited, primal - gap);
}

struct Batch {
    std::vector<ONode> nodes;
    std::vector<double> x, gap, value, best_vertex, best_vertex_val, lower_bound;
    std::vector<int> iterations;
    std::vector<uint8_t> status, branched_early;
    int generation = 0;
};

struct BnB {
    const gbx_problem* prob;
    const gbx_objective* obj;
    const gbx_lmo* lmo;
    const gbx_settings* s;
    int n;
    std::vector<int> int_vars;
    std::vector<uint8_t> flags;
    Queue queue;
    std::multiset<double> active_bounds;
    std::set<int> pruned_early_parents;
    double inc = kInf;
    std::vector<double> inc_x;
    int active = 0, next_id = 1, nodes_done = 0;
    bool done = false, reached_tol = false, reached_time = false, reached_nodes = false;
    double final_bound = -kInf;
    std::chrono::steady_clock::time_point started;
    // the single slot
    bool in_use = false;
    Batch slot;
    int generation = 0;

    double node_tol(const ONode& nd) const {
        return depth_tol(s->gpu_eps, s->gpu_eps_decay, s->gpu_eps_min, nd.depth);
    }
    bool should_prune(const ONode& nd) const { return nd.dual_bound >= inc; }
    double live_bound(double incumbent) const {
        const double q = queue.best_bound(incumbent);
        double a = incumbent;
        if (!active_bounds.empty()) { const double b = *active_bounds.begin(); a = b < incumbent ? b : incumbent; }
        return std::min(q, a);
    }
    void signal_done() { done = true; }
    bool time_up() {
        if (!std::isfinite(s->time_limit_seconds)) return false;
        const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - started).count();
        if (el < s->time_limit_seconds) return false;
        final_bound = live_bound(inc);
        reached_time = true;
        signal_done();
        return true;
    }
    // gbx_settings.node_limit (the library's extension, same rule as its engine:
    // checked where the time limit is, between batches)
    bool nodes_up() {
        if (s->node_limit <= 0 || nodes_done < s->node_limit) return false;
        final_bound = live_bound(inc);
        reached_nodes = true;
        signal_done();
        return true;
    }
    bool finish() {
        if (done) return true;
        if (queue.pq.empty() && active == 0) { final_bound = inc; signal_done(); return true; }
        const double b = live_bound(inc);
        if (gap_ok(b, inc, s->abs_gap_tol, s->rel_gap_tol)) {
            final_bound = b; reached_tol = true; signal_done(); return true;
        }
        return false;
    }
    void erase_bound(double b) { auto it = active_bounds.find(b); if (it != active_bounds.end()) active_bounds.erase(it); }

    void submit(std::vector<ONode> nodes) {
        const int N = (int)nodes.size();
        for (auto& nd : nodes) active_bounds.insert(nd.dual_bound);
        active += N;
        Batch bt;
        bt.generation = ++generation;
        bt.x.resize((size_t)N * n); bt.best_vertex.assign((size_t)N * n, 0.0);
        std::vector<double> lbv((size_t)N * n), ubv((size_t)N * n), eps(N);
        bt.gap.assign(N, 0.0); bt.value.assign(N, 0.0); bt.best_vertex_val.assign(N, kNone);
        bt.iterations.resize(N); bt.status.resize(N);
        for (int i = 0; i < N; ++i) {
            const ONode& nd = nodes[i];
            for (int j = 0; j < n; ++j) {
                bt.x[(size_t)i * n + j] = nd.relaxation_x.empty() ? nd.lb[j] : nd.relaxation_x[j];
                lbv[(size_t)i * n + j] = nd.lb[j];
                ubv[(size_t)i * n + j] = nd.ub[j];
            }
            eps[i] = node_tol(nd);
            bt.iterations[i] = nd.relaxation_iterations;
            bt.status[i] = nd.relaxation_x.empty() ? 0 : GBX_NODE_INITIAL_POINT_SUPPLIED;
        }
        gbx_node_batch b{};
        b.n_nodes = N; b.max_iters = s->gpu_max_iters; b.candidate_tol = s->integer_tol;
        b.x = bt.x.data(); b.lb = lbv.data(); b.ub = ubv.data(); b.eps = eps.data();
        b.iterations = bt.iterations.data(); b.status = bt.status.data();
        b.gap = bt.gap.data(); b.value = bt.value.data();
        b.best_vertex = bt.best_vertex.data(); b.best_vertex_val = bt.best_vertex_val.data();
        b.integer_flags = flags.data();
        const double cut = inc;   // the incumbent at dispatch
        b.cutoff = s->incumbent_cutoff ? &cut : nullptr;
        Relaxer r(obj, lmo, &s->algorithm);
        for (int i = 0; i < N; ++i) r.relax(i, &b);
        bt.nodes = std::move(nodes);
        slot = std::move(bt);
        in_use = true;
    }

    void fill(bool partial = false) {
        if (in_use) return;
        auto b = queue.pop_full_batch(s->gpu_batch_size, inc);
        if (b.empty() && partial) b = queue.pop_batch(s->gpu_batch_size, inc);
        if (b.empty()) return;
        submit(std::move(b));
    }

    Batch detach() {
        Batch b = std::move(slot);
        const int N = (int)b.nodes.size();
        b.branched_early.assign(N, 0);
        b.lower_bound.resize(N);
        for (int i = 0; i < N; ++i) {
            b.lower_bound[i] = certified_lb(b.nodes[i].dual_bound, b.value[i], b.gap[i]);
            if (b.status[i] == GBX_NODE_INFEASIBLE) b.lower_bound[i] = kInf;
        }
        in_use = false;
        return b;
    }

    bool try_update(double val, const std::vector<double>& x) {
        if (val < inc) { inc = val; inc_x = x; return true; }
        return false;
    }

    void branch_starved(std::vector<Batch>& batches) {
        struct Cd { size_t b; int i; double bound; };
        std::vector<Cd> cs;
        for (size_t b = 0; b < batches.size(); ++b)
            for (int i = 0; i < (int)batches[b].nodes.size(); ++i)
                cs.push_back({b, i, batches[b].lower_bound[i]});
        std::stable_sort(cs.begin(), cs.end(), [](const Cd& a, const Cd& b) { return a.bound < b.bound; });
        for (const auto& c : cs) {
            if (time_up() || in_use) return;
            Batch& bt = batches[c.b];
            ONode nd = bt.nodes[c.i];
            nd.dual_bound = c.bound;
            if (pruned_early_parents.count(nd.parent_id) || should_prune(nd)) continue;
            std::vector<double> x(bt.x.begin() + (size_t)c.i * n, bt.x.begin() + (size_t)(c.i + 1) * n);
            bool fin = true;
            for (double e : x) fin = fin && std::isfinite(e);
            if (!fin || bt.status[c.i] >= GBX_NODE_INTEGRAL_UNCONVERGED) continue;
            int nid = next_id; next_id += std::max(8, 1 << s->branch_k);
            auto ch = branch_pow2(nd, nid, x, int_vars, s->branch_k, s->integer_tol);
            bt.branched_early[c.i] = 1;
            for (auto& cn : ch) { cn.relaxation_x.clear(); cn.relaxation_iterations = 0; if (!should_prune(cn)) queue.push(cn); }
            if ((int)queue.pq.size() >= s->gpu_batch_size) { fill(true); return; }
        }
    }

    void process(Batch& b) {
        const int N = (int)b.nodes.size();
        for (int i = 0; i < N; ++i) {
            if (time_up()) return;
            ONode nd = b.nodes[i];
            const double ab = nd.dual_bound;
            if (b.status[i] == GBX_NODE_INFEASIBLE || pruned_early_parents.count(nd.parent_id)) {
                ++nodes_done; --active; erase_bound(ab); finish(); continue;
            }
            std::vector<double> xi(b.x.begin() + (size_t)i * n, b.x.begin() + (size_t)(i + 1) * n);
            const double gap = b.gap[i];
            nd.dual_bound = b.lower_bound[i];
            if (b.best_vertex_val[i] < 1e299 && std::isfinite(b.best_vertex_val[i])) {
                std::vector<double> bv(b.best_vertex.begin() + (size_t)i * n, b.best_vertex.begin() + (size_t)(i + 1) * n);
                try_update(b.best_vertex_val[i], bv);
            }
            const bool cert = std::isfinite(gap) && gap >= 0.0 && gap < node_tol(nd);
            if (should_prune(nd)) {
                if (b.branched_early[i]) { pruned_early_parents.insert(nd.id); queue.discard_children(nd.id); }
                ++nodes_done; --active; erase_bound(ab); finish(); continue;
            }
            if (b.status[i] >= GBX_NODE_INTEGRAL_UNCONVERGED && !cert) {
                nd.relaxation_x = std::move(xi);
                nd.relaxation_iterations = b.iterations[i];
                queue.push(nd);
                --active; erase_bound(ab);
                continue;
            }
            if (done) {
            } else if (b.status[i] >= GBX_NODE_INTEGRAL_UNCONVERGED) {
            } else if (!b.branched_early[i]) {
                int nid = next_id; next_id += std::max(8, 1 << s->branch_k);
                for (auto& c : branch_pow2(nd, nid, xi, int_vars, s->branch_k, s->integer_tol)) {
                    c.relaxation_x.clear(); c.relaxation_iterations = 0;
                    if (!should_prune(c)) queue.push(c);
                }
            }
            ++nodes_done; --active; erase_bound(ab); finish();
        }
        if (active == 0) finish();
    }

    void worker() {
        while (!done) {
            if (time_up() || nodes_up()) return;
            std::vector<Batch> completed;
            if (in_use) completed.push_back(detach());  // launch completed synchronously
            fill();
            if (queue.pq.empty() && !in_use) branch_starved(completed);
            for (auto& b : completed) process(b);
            if (active == 0 && finish()) return;
            fill();
            if (!in_use) { fill(true); if (in_use) continue; }
            if (!in_use && !queue.pq.empty()) fill(true);
            else if (!in_use) { if (active == 0 && finish()) return; }
        }
        if (in_use) { auto b = detach(); process(b); }
    }
};

}  // namespace

extern "C" {

const char* oracle_last_error(void) { return g_error.c_str(); }
int oracle_lanes(void) { return kLanes; }

int oracle_relax_batch(const gbx_objective* obj, const gbx_lmo* lmo,
                       const gbx_algorithm* alg, const gbx_node_batch* b,
                       int threads) {
    const int rc = check_descs(obj, lmo, alg);
    if (rc) return rc;
    if (!b || b->n_nodes < 0) { g_error = "batch"; return GBX_ERR_INVALID; }
    if (threads <= 1 || b->n_nodes <= 1) {
        Relaxer r(obj, lmo, alg);
        for (int i = 0; i < b->n_nodes; ++i) r.relax(i, b);
        return GBX_OK;
    }
    const int T = std::min(threads, b->n_nodes);
    std::vector<std::thread> pool;
    for (int t = 0; t < T; ++t)
        pool.emplace_back([=]() {
            Relaxer r(obj, lmo, alg);
            for (int i = t; i < b->n_nodes; i += T) r.relax(i, b);
        });
    for (auto& th : pool) th.join();
    return GBX_OK;
}

int oracle_lmo_batch(const gbx_lmo* lmo, int cases, int mode, const double* dir,
                     const double* x, const double* lb, const double* ub,
                     double* out, double* out_step) {
    if (!lmo || cases < 0 || (mode != 0 && mode != 1)) { g_error = "lmo args"; return GBX_ERR_INVALID; }
    LMO L(lmo);
    const int n = lmo->n;
    std::vector<double> neg(n), fwd(n), d(n);
    for (int c = 0; c < cases; ++c) {
        const size_t off = (size_t)c * n;
        if (mode == 0) { L.forward(dir + off, lb + off, ub + off, out + off); continue; }
        L.inface(dir + off, x + off, lb + off, ub + off, out + off);
        if (out_step) {
            for (int j = 0; j < n; ++j) neg[j] = -dir[off + j];
            L.forward(neg.data(), lb + off, ub + off, fwd.data());
            for (int j = 0; j < n; ++j) d[j] = out[off + j] - fwd[j];
            out_step[c] = L.max_step(d.data(), x + off, lb + off, ub + off);
        }
    }
    return GBX_OK;
}

int oracle_node_feasible_batch(const gbx_lmo* lmo, int cases, const double* lb,
                               const double* ub, const uint8_t* flags, uint8_t* out) {
    LMO L(lmo);
    const int n = lmo->n;
    for (int c = 0; c < cases; ++c) {
        const double* l = lb + (size_t)c * n;
        const double* u = ub + (size_t)c * n;
        bool valid = true;
        for (int j = 0; j < n; ++j)
            if (std::isnan(l[j]) || std::isnan(u[j]) || l[j] > u[j]
                    || (flags && flags[j] && std::ceil(l[j]) > std::floor(u[j])))
                valid = false;
        out[c] = (valid && L.check_feasible(l, u, flags)) ? 1 : 0;
    }
    return GBX_OK;
}

double oracle_objective_value(const gbx_objective* obj, const double* x) {
    Objective o(obj);
    return o.value(x);
}
void oracle_objective_grad(const gbx_objective* obj, const double* x, double* g) {
    Objective o(obj);
    o.grad(x, g);
}
double oracle_objective_curvature(const gbx_objective* obj, const double* d) {
    Objective o(obj);
    return o.curvature(d);
}

// Whole branch and bound with one slot, launches completing synchronously
// (gpuboscia::solve with num_streams = 1).
int oracle_solve(const gbx_problem* prob, const gbx_objective* obj, const gbx_lmo* lmo,
                 const gbx_settings* s, gbx_result* res) {
    int rc = check_descs(obj, lmo, &s->algorithm);
    if (rc) return rc;
    if (!prob || prob->n_vars != obj->n) { g_error = "problem size"; return GBX_ERR_INVALID; }
    if (s->algorithm.kind == GBX_ALG_FRANK_WOLFE
            && (s->algorithm.line_search == GBX_LS_SCALED_OPEN_LOOP
                || s->algorithm.line_search == GBX_LS_SAFEGUARDED_SCALED_OPEN_LOOP)) {
        g_error = "scaled open-loop is available only for DICG"; return GBX_ERR_INVALID;
    }
    BnB bb;
    bb.prob = prob; bb.obj = obj; bb.lmo = lmo; bb.s = s; bb.n = prob->n_vars;
    bb.int_vars.assign(prob->int_vars, prob->int_vars + prob->n_int);
    bb.flags.assign(bb.n, 0);
    for (int j : bb.int_vars) bb.flags[j] = 1;
    ONode root;
    root.id = 0; root.parent_id = -1; root.depth = 0;
    root.lb.assign(prob->lb, prob->lb + bb.n);
    root.ub.assign(prob->ub, prob->ub + bb.n);
    root.dual_bound = s->natural_lower_bound;
    if (s->root_initial_point) root.relaxation_x.assign(s->root_initial_point, s->root_initial_point + bb.n);
    bb.queue.push(root);
    bb.started = std::chrono::steady_clock::now();
    bb.worker();
    if (bb.final_bound == -kInf) bb.final_bound = bb.queue.best_bound(bb.inc);
    res->objective = bb.inc;
    res->dual_bound = bb.final_bound;
    res->nodes_processed = bb.nodes_done;
    res->elapsed_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - bb.started).count();
    res->reached_tolerance = bb.reached_tol;
    res->reached_time_limit = bb.reached_time;
    res->reached_node_limit = bb.reached_nodes;
    res->batches = bb.generation;
    res->has_incumbent = !bb.inc_x.empty();
    if (res->x && res->has_incumbent)
        std::copy(bb.inc_x.begin(), bb.inc_x.end(), res->x);
    return GBX_OK;
}

}  // extern "C"
