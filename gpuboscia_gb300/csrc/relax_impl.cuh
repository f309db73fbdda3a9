#pragma once
// relax_impl.cuh -- device code of the node relaxation (FW / DICG) for sm_103a,
// shared by the translation units that instantiate its kernels.
//
// One 256-thread CTA relaxes one B&B node (the reference's node-per-block
// decomposition, device_resident_solver.cuh:631-660), but the node's working
// set (iterate, gradient, vertices, bounds, residual, objective matrices) is
// staged in shared memory whenever it fits, so an iteration touches HBM only
// for the objective data of large instances. The Birkhoff oracle runs as a
// warp-level Hungarian (shuffle argmin, no block barriers per Dijkstra step),
// and the DICG forward and in-face oracles run concurrently on warps 0 and 1.
//
// Arithmetic follows a fixed order so results are reproducible on any GPU and
// by the oracle: block reductions are 256 lanes folded by the warp shuffle
// tree; products marked fma() are fused, nothing else is (-fmad=false).
//
// Reference semantics restated: drs_fw_relax_node (device_resident_solver.cuh:
// 337-629), SecantLS / QuadraticExactLS (algorithms.cuh:121-296), BoxLMO /
// UnitSimplexLMO / BirkhoffLMO (lmo.cuh:212-1417), drs_integer_value and the
// rounding heuristic (device_resident_solver.cuh:295-335, heuristics.h:23-35).
#include <cuda_runtime.h>
#include <math_constants.h>

#include <algorithm>
#include <cstdio>

#include "relax.cuh"

namespace gbx {

constexpr unsigned kFull = 0xffffffffu;
constexpr double kInfD = __builtin_huge_val();   // +infinity

// ------------------------------------------------------------------ layout

struct HW {
    double *u, *pv, *minv;
    int *p, *way, *fcol, *frow, *rows, *cols, *pi, *pinv, *scal;
    uint8_t* used;
};

__device__ inline HW hw_at(unsigned char* base, int m) {
    HW w;
    size_t o = 0;
    w.u = reinterpret_cast<double*>(base + o);
    w.pv = w.u + (m + 1);
    w.minv = w.pv + (m + 1);
    o += align16(3 * (size_t)(m + 1) * sizeof(double));
    w.p = reinterpret_cast<int*>(base + o);
    w.way = w.p + (m + 1);
    o += align16(2 * (size_t)(m + 1) * sizeof(int));
    w.fcol = reinterpret_cast<int*>(base + o);
    w.frow = w.fcol + m;
    w.rows = w.frow + m;
    w.cols = w.rows + m;
    w.pi = w.cols + m;
    w.pinv = w.pi + m;
    o += align16(6 * (size_t)m * sizeof(int));
    w.scal = reinterpret_cast<int*>(base + o);
    o += align16(8 * sizeof(int));
    w.used = base + o;
    return w;
}

// ------------------------------------------------------------------ reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = v + __shfl_down_sync(kFull, v, off);
    return v;
}
__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = fmin(v, __shfl_down_sync(kFull, v, off));
    return v;
}

// 256-lane sum, result broadcast to every thread.
static __device__ double bsum(double v, double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        double r = lane < kWarps ? red[lane] : 0.0;
        r = warp_sum(r);
        if (lane == 0) red[32] = r;
    }
    __syncthreads();
    return red[32];
}
// 256-lane min; lanes past the warp count read 1.0 (drs_block_min).
static __device__ double bmin(double v, double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warp_min(v);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        double r = lane < kWarps ? red[lane] : 1.0;
        r = warp_min(r);
        if (lane == 0) red[33] = r;
    }
    __syncthreads();
    return red[33];
}

// ------------------------------------------------------------------ context
struct Ctx {
    int n, tid;
    double* red;          // >= 40 doubles
    int* flag;            // shared ints
    // objective
    int ok;               // objective kind
    int m;                // graph order
    const double* Q;
    const double* c;
    double s, ls, k0;
    const double* A;
    const double* B;
    double* R;
    SparseAB sp;          // nonzero lists of A and B (valid when use_sp)
    bool use_sp;
    // lmo
    int lk;
    double rhs;
    const uint8_t* is_int;
    int lorder;
    const double* U;      // linked cardinality: per-asset bounds U_i
    int S;
    double* keys;
    double* prefix;
    int* idx;
    uint8_t* fixed;
    unsigned char* hung[2];
    size_t hung_bytes;
    // problem
    const uint8_t* flags;
    double tol;
    // a node on a pair of CTAs (a two-CTA cluster, dense quadratic objective):
    // this CTA's rank (-1: one CTA per node) and the 256-double buffer through
    // which the pair exchanges per-lane partial sums
    int pr = -1;
    double* xch = nullptr;
};

// ---- the pair's exchange: the peer's copy of a shared-memory object, a
// remote FP64 store, and the cluster-wide barrier (both CTAs, all threads)
__device__ __forceinline__ unsigned pair_addr(const void* p, int rank) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;"
                 : "=r"(r) : "r"((unsigned)__cvta_generic_to_shared(p)), "r"(rank));
    return r;
}
__device__ __forceinline__ void pair_store(const double* p, int rank, double v) {
    asm volatile("st.shared::cluster.f64 [%0], %1;" :: "r"(pair_addr(p, rank)), "d"(v) : "memory");
}
__device__ __forceinline__ void pair_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// A per-lane partial computed by the lane's owner (lanes of parity pr) made
// visible to both CTAs, then the 256-lane sum in the usual order.
__device__ __forceinline__ double pair_lane_value(const Ctx& c, double v) {
    if (!((c.tid & 1) ^ c.pr)) {
        c.xch[c.tid] = v;
        pair_store(c.xch + c.tid, c.pr ^ 1, v);
    }
    pair_sync();
    return c.xch[c.tid];
}

// ------------------------------------------------------------------ objective
static __device__ bool all_finite(const Ctx& c, const double* v) {
    bool f = true;
    for (int e = c.tid; e < c.n; e += kThreads) f = f && isfinite(v[e]);
    return __syncthreads_and(f) != 0;
}

// R = A X - X B. With the nonzero lists the terms of zero coefficients are
// skipped, in the same order as the dense loop (bit-identical for finite X).
static __device__ void residual(const Ctx& c, const double* X, double* R) {
    const int m = c.m;
    if (c.use_sp && all_finite(c, X)) {
        const SparseAB& S = c.sp;
        for (int e = c.tid; e < c.n; e += kThreads) {
            const int i = e / m, j = e - (e / m) * m;
            int ia = S.ptr[0][i], ib = S.ptr[1][j];
            const int ea = S.ptr[0][i + 1], eb = S.ptr[1][j + 1];
            double r = 0.0;
            while (ia < ea || ib < eb) {
                const int ka = ia < ea ? S.idx[0][ia] : m;
                const int kb = ib < eb ? S.idx[1][ib] : m;
                if (ka <= kb) { r = fma(S.val[0][ia], X[ka * m + j], r); ++ia; }
                else { r = fma(-X[i * m + kb], S.val[1][ib], r); ++ib; }
            }
            R[e] = r;
        }
        return;
    }
    for (int e = c.tid; e < c.n; e += kThreads) {
        const int i = e / m, j = e - (e / m) * m;
        double r = 0.0;
        for (int k = 0; k < m; ++k) {
            r = fma(c.A[i * m + k], X[k * m + j], r);
            r = fma(-X[i * m + k], c.B[k * m + j], r);
        }
        R[e] = r;
    }
}

// g = 2s (A'R - R B') from the residual in c.R (graph matching).
static __device__ void grad_from_residual(const Ctx& c, double* g) {
    const int n = c.n;
    {
        const int m = c.m;
        const double two_s = 2.0 * c.s;
        if (c.use_sp && all_finite(c, c.R)) {
            const SparseAB& S = c.sp;
            for (int e = c.tid; e < n; e += kThreads) {
                const int p = e / m, q = e - (e / m) * m;
                double acc = 0.0;
                for (int t = S.ptr[2][p]; t < S.ptr[2][p + 1]; ++t)
                    acc = fma(S.val[2][t], c.R[S.idx[2][t] * m + q], acc);
                for (int t = S.ptr[3][q]; t < S.ptr[3][q + 1]; ++t)
                    acc = fma(-c.R[p * m + S.idx[3][t]], S.val[3][t], acc);
                g[e] = two_s * acc;
            }
        } else {
            for (int e = c.tid; e < n; e += kThreads) {
                const int p = e / m, q = e - (e / m) * m;
                double acc = 0.0;
                for (int r = 0; r < m; ++r) acc = fma(c.A[r * m + p], c.R[r * m + q], acc);
                for (int k = 0; k < m; ++k) acc = fma(-c.R[p * m + k], c.B[q * m + k], acc);
                g[e] = two_s * acc;
            }
        }
    }
    __syncthreads();
}

// g = grad f(x). Graph matching leaves the residual of x in c.R.
static __device__ void obj_grad(const Ctx& c, const double* x, double* g) {
    const int n = c.n;
    if (c.ok == GBX_OBJ_GRAPH_MATCHING) {
        residual(c, x, c.R);
        __syncthreads();
        grad_from_residual(c, g);
        return;
    } else {
        // a pair of CTAs computes the elements of its parity and stores them in
        // both copies of g (g is in shared memory in the pair shape); the first
        // barrier keeps the peer's previous g until it is done with it
        if (c.pr >= 0) pair_sync();
        for (int j = c.tid; j < n; j += kThreads) {
            if (c.pr >= 0 && (j & 1) != c.pr) continue;
            double acc = 0.0;
            for (int k = 0; k < n; ++k) acc = fma(c.Q[(size_t)k * n + j], x[k], acc);
            const double lin = c.c ? c.ls * c.c[j] : 0.0;
            g[j] = c.s * (acc + lin);
            if (c.pr >= 0) pair_store(g + j, c.pr ^ 1, g[j]);
        }
        if (c.pr >= 0) pair_sync();
    }
    __syncthreads();
}

static __device__ double value_from_residual(const Ctx& c) {
    double loc = 0.0;
    for (int e = c.tid; e < c.n; e += kThreads) loc = fma(c.R[e], c.R[e], loc);
    return c.s * bsum(loc, c.red);
}

// f(x) from the gradient g just evaluated at x (graph matching: from the
// residual obj_grad left in c.R; dense quadratic: f = x'g/2 + s l c'x/2 + k),
// for the incumbent cutoff. Lane order as bsum.
static __device__ double value_at_grad(const Ctx& c, const double* x, const double* g) {
    if (c.ok == GBX_OBJ_GRAPH_MATCHING) return value_from_residual(c);
    const double hb = 0.5 * c.s * c.ls;
    double loc = 0.0;
    for (int j = c.tid; j < c.n; j += kThreads) {
        loc = fma(0.5 * x[j], g[j], loc);
        if (c.c) loc = fma(hb * c.c[j], x[j], loc);
    }
    return bsum(loc, c.red) + c.k0;
}

static __device__ double obj_value(const Ctx& c, const double* x) {
    const int n = c.n;
    if (c.ok == GBX_OBJ_GRAPH_MATCHING) {
        residual(c, x, c.R);
        __syncthreads();
        return value_from_residual(c);
    }
    const double a = 0.5 * c.s, b = c.s * c.ls;
    double quad = 0.0, lin = 0.0;
    const bool mine = c.pr < 0 || !((c.tid & 1) ^ c.pr);   // a pair: the lanes of this CTA's parity
    if (c.pr >= 0) pair_sync();
    for (int j = c.tid; mine && j < n; j += kThreads) {
        double qx = 0.0;
        for (int k = 0; k < n; ++k) qx = fma(c.Q[(size_t)k * n + j], x[k], qx);
        quad = fma(x[j], qx, quad);
        if (c.c) lin = fma(c.c[j], x[j], lin);
    }
    double val = a * quad + b * lin;
    if (c.tid == 0) val += c.k0;
    if (c.pr >= 0) val = pair_lane_value(c, val);
    return bsum(val, c.red);
}

static __device__ double obj_curvature(const Ctx& c, const double* d) {
    const int n = c.n;
    if (c.ok == GBX_OBJ_GRAPH_MATCHING) {
        residual(c, d, c.R);
        __syncthreads();
        double loc = 0.0;
        for (int e = c.tid; e < n; e += kThreads) loc = fma(c.R[e], c.R[e], loc);
        return (2.0 * c.s) * bsum(loc, c.red);
    }
    double curv = 0.0;
    const bool mine = c.pr < 0 || !((c.tid & 1) ^ c.pr);
    if (c.pr >= 0) pair_sync();
    for (int j = c.tid; mine && j < n; j += kThreads) {
        double prod = 0.0;
        for (int k = 0; k < n; ++k) prod = fma(c.Q[(size_t)k * n + j], d[k], prod);
        curv = fma(c.s * d[j], prod, curv);
    }
    if (c.pr >= 0) curv = pair_lane_value(c, curv);
    return bsum(curv, c.red);
}

// Value of a permutation vertex of the graph-matching objective in O(m^2):
// with exactly one unit per row and column, every residual entry of the
// generic O(m^3) loop reduces to one rounding of A[i,pinv(j)] - B[pi(i),j],
// so this is bit-identical to obj_value on the same vertex.
static __device__ double perm_value(const Ctx& c, const int* pi, int* pinv) {
    const int m = c.m;
    for (int r = c.tid; r < m; r += kThreads) pinv[pi[r]] = r;
    __syncthreads();
    double loc = 0.0;
    for (int e = c.tid; e < c.n; e += kThreads) {
        const int i = e / m, j = e - (e / m) * m;
        const double r = c.A[i * m + pinv[j]] - c.B[pi[i] * m + j];
        loc = fma(r, r, loc);
    }
    return c.s * bsum(loc, c.red);
}

}  // namespace gbx
#include "mixed.cuh"
#include "tc_grad.cuh"
#include "cluster.cuh"
namespace gbx {

// ------------------------------------------------------------------ Hungarian
// Order-preserving 64-bit key of a double (zeros of both signs map to +0's key,
// so keys tie exactly when the doubles compare equal); finite values only.
__device__ __forceinline__ unsigned long long fp64_key(double v) {
    const long long b = __double_as_longlong(v == 0.0 ? 0.0 : v);
    return b >= 0 ? (unsigned long long)b ^ 0x8000000000000000ull : ~(unsigned long long)b;
}

// Solve phase of the FP64 Hungarian with the column state in registers: lane l
// owns the compacted columns l+1, l+33, ... (CPL per lane; k <= 32*CPL). The
// arithmetic is the shared-memory loop's, operation for operation (same
// potentials, slacks and updates), and the step argmin -- lowest slack, lowest
// column on ties -- takes three warp min-reductions over the slack's key.
template <int CPL>
static __device__ bool hung_solve_reg(const HW& w, int m, int k, const double* cost, double sign,
                                      const double* ub, const double* face, double* out, const uint8_t* code) {
    const int lane = threadIdx.x & 31;
    int colE[CPL], way[CPL], pr[CPL];
    double minv[CPL], pv[CPL];
    bool valid[CPL], used[CPL];
#pragma unroll
    for (int t = 0; t < CPL; ++t) {
        const int j = lane + 1 + 32 * t;
        valid[t] = j <= k;
        colE[t] = valid[t] ? w.cols[j - 1] : 0;
        pv[t] = 0.0;
        pr[t] = 0;
        way[t] = 0;
    }
    for (int j = lane; j <= k; j += 32) w.u[j] = 0.0;
    __syncwarp();
    for (int i = 1; i <= k; ++i) {
#pragma unroll
        for (int t = 0; t < CPL; ++t) { minv[t] = kNone; used[t] = false; }
        int j0 = 0;
        bool done = false;
        for (int step = 0; step <= k; ++step) {
            // row of column j0 (column 0 holds the row being inserted)
            int i0 = i;
            if (j0 != 0) {
                const int owner = (j0 - 1) & 31, slot = (j0 - 1) >> 5;
                i0 = __shfl_sync(kFull, lane_slot<CPL>(pr, slot), owner);
            }
            const double ui0 = w.u[i0];
            const int rb = w.rows[i0 - 1] * m;
            unsigned long long bkey = ~0ull;
            int bj = 0x7fffffff;
            // every column's permission and cost of the row first (invalid slots
            // read column 0 of the same row), then the scan in column order
            double cc[CPL];
            bool al[CPL];
#pragma unroll
            for (int t = 0; t < CPL; ++t) {
                const int e = rb + colE[t];
                const bool a1 = code ? (code[e] & kAllowed) != 0 : ub[e] >= 0.5;
                const bool a2 = !face || face[e] > 1e-9;
                al[t] = a1 && a2;
                cc[t] = cost ? cost[e] : 0.0;
            }
#pragma unroll
            for (int t = 0; t < CPL; ++t) {
                if (!valid[t] || used[t]) continue;
                double mv = minv[t];
                if (al[t]) {
                    const double ce = cost ? sign * cc[t] : 0.0;
                    const double cur = ce - ui0 - pv[t];
                    if (cur < mv) { mv = cur; minv[t] = cur; way[t] = j0; }
                }
                if (mv < kNone) {
                    const unsigned long long key = fp64_key(mv);
                    const int j = lane + 1 + 32 * t;
                    if (key < bkey) { bkey = key; bj = j; }
                }
            }
            const unsigned hi = __reduce_min_sync(kFull, (unsigned)(bkey >> 32));
            const unsigned lo = __reduce_min_sync(kFull, (unsigned)(bkey >> 32) == hi ? (unsigned)bkey : ~0u);
            const unsigned long long best = ((unsigned long long)hi << 32) | lo;
            const int j1 = (int)__reduce_min_sync(kFull, bkey == best ? (unsigned)bj : 0x7fffffffu);
            if (j1 == 0x7fffffff) return false;
            const int owner = (j1 - 1) & 31, slot = (j1 - 1) >> 5;
            double bvl = 0.0;
#pragma unroll
            for (int t = 0; t < CPL; ++t)
                if (t == slot) bvl = minv[t];
            const double bv = __shfl_sync(kFull, bvl, owner);
            if (!isfinite(bv)) return false;
            // potentials: used columns (and column 0) move with the tree, the others' slacks shrink
            if (lane == 0) w.u[i] += bv;
#pragma unroll
            for (int t = 0; t < CPL; ++t) {
                if (!valid[t]) continue;
                if (used[t]) { w.u[pr[t]] += bv; pv[t] -= bv; }
                else minv[t] -= bv;
            }
            __syncwarp();
            j0 = j1;
            const int pj = __shfl_sync(kFull, lane_slot<CPL>(pr, slot), owner);
            if (lane == owner) {
#pragma unroll
                for (int t = 0; t < CPL; ++t)
                    if (t == slot) used[t] = true;
            }
            if (pj == 0) { done = true; break; }
        }
        if (!done) return false;   // no augmenting path within k+1 steps
        // flip the path: column jj takes the row of way[jj] (column 0 holds row i)
        int jj = j0;
        for (int guard = 0; guard <= k && jj != 0; ++guard) {
            const int owner = (jj - 1) & 31, slot = (jj - 1) >> 5;
            const int j1 = __shfl_sync(kFull, lane_slot<CPL>(way, slot), owner);
            int np = i;
            if (j1 != 0) np = __shfl_sync(kFull, lane_slot<CPL>(pr, (j1 - 1) >> 5), (j1 - 1) & 31);
            if (lane == owner) {
#pragma unroll
                for (int t = 0; t < CPL; ++t)
                    if (t == slot) pr[t] = np;
            }
            jj = j1;
        }
        __syncwarp();
    }
#pragma unroll
    for (int t = 0; t < CPL; ++t) {
        if (!valid[t]) continue;
        const int r = w.rows[pr[t] - 1];
        out[r * m + colE[t]] = 1.0;
        w.pi[r] = colE[t];
    }
    __syncwarp();
    return true;
}

// Exact min-cost assignment over the Birkhoff order-m polytope with forced
// (lb > 1/2), forbidden (ub < 1/2) and face restrictions, ties to the lowest
// column (lmo.cuh:1239-1417). Executed by ONE warp; `out` must be zeroed and
// visible. cost may be null (zero costs); the cost of edge e is sign*cost[e].
// Returns a warp-uniform success flag and leaves the row->column map in w.pi.
// Pre-pass of the Hungarian (one warp): forced (lb > 1/2 or face-forced) edges,
// contradictions, and the compacted free rows / columns; writes the forced
// entries of `out` and w.pi. Returns the number k of free rows, or -1.
static __device__ int hung_prepass(const HW& w, int m, const double* lb, const double* ub, const double* face,
                                   double* out) {
    const int lane = threadIdx.x & 31;
    for (int i = lane; i < m; i += 32) { w.fcol[i] = -1; w.frow[i] = -1; }
    __syncwarp();
    bool ok = true;
    const int nn = m * m;
    for (int e = lane; e < nn; e += 32) {
        const double le = lb[e], ue = ub[e];
        if (le > ue + 1e-9) ok = false;
        const bool forced = le > 0.5 || (face && face[e] >= 1.0 - 1e-9);
        if (forced) {
            const int r = e / m, col = e - r * m;
            if (ue < 0.5) ok = false;
            if (atomicCAS(&w.fcol[r], -1, col) != -1) ok = false;
            if (atomicCAS(&w.frow[col], -1, r) != -1) ok = false;
        }
    }
    ok = __all_sync(kFull, ok);
    __syncwarp();
    if (!ok) return -1;
    int k = 0, kc = 0;
    const unsigned lt = (1u << lane) - 1u;
    for (int base = 0; base < m; base += 32) {
        const int i = base + lane;
        const bool fr = i < m && w.fcol[i] < 0;
        const bool fc = i < m && w.frow[i] < 0;
        const unsigned mr = __ballot_sync(kFull, fr), mc = __ballot_sync(kFull, fc);
        if (fr) w.rows[k + __popc(mr & lt)] = i;
        if (fc) w.cols[kc + __popc(mc & lt)] = i;
        k += __popc(mr);
        kc += __popc(mc);
    }
    if (k != kc) return -1;
    for (int i = lane; i < m; i += 32)
        if (w.fcol[i] >= 0) { out[i * m + w.fcol[i]] = 1.0; w.pi[i] = w.fcol[i]; }
    __syncwarp();
    return k;
}

// Solve phase with the column state in shared memory (one warp; any k).
static __device__ bool hung_solve_smem(const HW& w, int m, int k, const double* cost, double sign,
                                       const double* ub, const double* face, double* out, const uint8_t* code) {
    const int lane = threadIdx.x & 31;
    for (int j = lane; j <= k; j += 32) { w.u[j] = 0.0; w.pv[j] = 0.0; w.p[j] = 0; w.way[j] = 0; }
    __syncwarp();
    for (int i = 1; i <= k; ++i) {
        for (int j = lane; j <= k; j += 32) { w.minv[j] = kNone; w.used[j] = 0; }
        if (lane == 0) w.p[0] = i;
        __syncwarp();
        int j0 = 0;
        for (int step = 0; step <= k; ++step) {
            if (lane == 0) w.used[j0] = 1;
            __syncwarp();
            const int i0 = w.p[j0];
            const double ui0 = w.u[i0];
            const int rb = w.rows[i0 - 1] * m;
            double bv = kNone;
            int bj = -1;
            for (int j = lane + 1; j <= k; j += 32) {
                if (w.used[j]) continue;
                const int e = rb + w.cols[j - 1];
                double mv = w.minv[j];
                const bool allowed = code ? (code[e] & kAllowed) != 0 : ub[e] >= 0.5;
                if (allowed && (!face || face[e] > 1e-9)) {
                    const double ce = cost ? sign * cost[e] : 0.0;
                    const double cur = ce - ui0 - w.pv[j];
                    if (cur < mv) { mv = cur; w.minv[j] = cur; w.way[j] = j0; }
                }
                if (mv < kNone && (bj < 0 || mv < bv)) { bv = mv; bj = j; }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const double ov = __shfl_down_sync(kFull, bv, off);
                const int oj = __shfl_down_sync(kFull, bj, off);
                if (oj >= 0 && (bj < 0 || ov < bv || (ov == bv && oj < bj))) { bv = ov; bj = oj; }
            }
            bv = __shfl_sync(kFull, bv, 0);
            bj = __shfl_sync(kFull, bj, 0);
            if (bj < 0 || !isfinite(bv)) return false;
            __syncwarp();
            for (int j = lane; j <= k; j += 32) {
                if (w.used[j]) { w.u[w.p[j]] += bv; w.pv[j] -= bv; }
                else w.minv[j] -= bv;
            }
            __syncwarp();
            j0 = bj;
            if (w.p[j0] == 0) break;
        }
        if (w.p[j0] != 0) return false;  // no augmenting path within k+1 steps
        if (lane == 0) {
            int jj = j0;
            for (int guard = 0; guard <= k && jj != 0; ++guard) {
                const int j1 = w.way[jj];
                w.p[jj] = w.p[j1];
                jj = j1;
            }
        }
        __syncwarp();
    }
    for (int j = lane + 1; j <= k; j += 32) {
        const int r = w.rows[w.p[j] - 1], col = w.cols[j - 1];
        out[r * m + col] = 1.0;
        w.pi[r] = col;
    }
    __syncwarp();
    return true;
}

template <int MAXCPL = 8>
static __device__ bool hungarian_warp(const HW& w, int m, const double* cost, double sign,
                               const double* lb, const double* ub, const double* face,
                               double* out, const uint8_t* code = nullptr) {
    const int k = hung_prepass(w, m, lb, ub, face, out);
    if (k < 0) return false;
    // register-resident solve up to 32*MAXCPL free columns (MAXCPL bounds the
    // registers a kernel spends on it), the shared-memory loop beyond
    if (k <= 64) return hung_solve_reg<2>(w, m, k, cost, sign, ub, face, out, code);
    if constexpr (MAXCPL >= 4)
        if (k <= 128) return hung_solve_reg<4>(w, m, k, cost, sign, ub, face, out, code);
    if constexpr (MAXCPL >= 8)
        if (k <= 256) return hung_solve_reg<8>(w, m, k, cost, sign, ub, face, out, code);
    return hung_solve_smem(w, m, k, cost, sign, ub, face, out, code);
}

// ---- the same Hungarian on a group of four warps (one per SM sub-partition:
// on GB300 each sub-partition executes its own FP64 instructions, so the
// per-step slack updates of 128 lanes cost what 32 lanes' did). Groups are
// threads [0,128) (g = 0, named barrier 1) and [128,256) (g = 1, barrier 2);
// a lone oracle (the FP64 forward LMO of Frank-Wolfe, the certificate) runs on
// the whole CTA as one group of eight warps (GW = 8, g = 0, named barrier 1).
constexpr int kHungWarps = 4;
constexpr int kHungThreads = kHungWarps * 32;

template <int GW = kHungWarps>
__device__ __forceinline__ void group_bar(int g) {
    asm volatile("bar.sync %0, %1;" :: "r"(1 + g), "r"(GW * 32) : "memory");
}

__device__ __forceinline__ double key_fp64(unsigned long long key) {
    const unsigned long long b = (key >> 63) ? key ^ 0x8000000000000000ull : ~key;
    return __longlong_as_double((long long)b);
}

// Solve phase: thread gt of the group owns the compacted columns gt+1,
// gt+1+32*GW, ... (CPL per thread; k <= 32*GW*CPL). Per step every warp reduces
// its best (slack key, column) with three REDUX, the GW warp results meet in
// shared memory, and every thread derives the step value from the winning key
// (the key maps back to the slack exactly, up to the sign of a zero, which no
// comparison sees). Potential updates and the tie rule are those of the
// single-warp loop, so the assignment is identical.
template <int CPL, int GW = kHungWarps>
static __device__ bool hung_solve_group(const HW& w, int m, int k, const double* cost, double sign,
                                        const double* ub, const double* face, double* out, const uint8_t* code,
                                        int g) {
    constexpr int GT = GW * 32;
    __shared__ unsigned long long s_key[2][GW];
    __shared__ int s_j[2][GW];
    __shared__ int s_row[2];
    const int gt = threadIdx.x - GT * g, lane = gt & 31, gw = gt >> 5;
    int colE[CPL], way[CPL], pr[CPL];
    double minv[CPL], pv[CPL];
    bool valid[CPL], used[CPL];
#pragma unroll
    for (int t = 0; t < CPL; ++t) {
        const int j = gt + 1 + GT * t;
        valid[t] = j <= k;
        colE[t] = valid[t] ? w.cols[j - 1] : 0;
        pv[t] = 0.0;
        pr[t] = 0;
        way[t] = 0;
    }
    for (int j = gt; j <= k; j += GT) w.u[j] = 0.0;
    group_bar<GW>(g);
    for (int i = 1; i <= k; ++i) {
#pragma unroll
        for (int t = 0; t < CPL; ++t) { minv[t] = kNone; used[t] = false; }
        int j0 = 0, i0 = i;
        bool done = false;
        for (int step = 0; step <= k; ++step) {
            const double ui0 = w.u[i0];
            const int rb = w.rows[i0 - 1] * m;
            unsigned long long bkey = ~0ull;
            int bj = 0x7fffffff;
            // every column's permission and cost of the row first (invalid slots
            // read column 0 of the same row), then the scan in column order
            double cc[CPL];
            bool al[CPL];
#pragma unroll
            for (int t = 0; t < CPL; ++t) {
                const int e = rb + colE[t];
                const bool a1 = code ? (code[e] & kAllowed) != 0 : ub[e] >= 0.5;
                const bool a2 = !face || face[e] > 1e-9;
                al[t] = a1 && a2;
                cc[t] = cost ? cost[e] : 0.0;
            }
#pragma unroll
            for (int t = 0; t < CPL; ++t) {
                if (!valid[t] || used[t]) continue;
                double mv = minv[t];
                if (al[t]) {
                    const double ce = cost ? sign * cc[t] : 0.0;
                    const double cur = ce - ui0 - pv[t];
                    if (cur < mv) { mv = cur; minv[t] = cur; way[t] = j0; }
                }
                if (mv < kNone) {
                    const unsigned long long key = fp64_key(mv);
                    const int j = gt + 1 + GT * t;
                    if (key < bkey) { bkey = key; bj = j; }
                }
            }
            const unsigned hi = __reduce_min_sync(kFull, (unsigned)(bkey >> 32));
            const unsigned lo = __reduce_min_sync(kFull, (unsigned)(bkey >> 32) == hi ? (unsigned)bkey : ~0u);
            const unsigned long long wkey = ((unsigned long long)hi << 32) | lo;
            const int wj = (int)__reduce_min_sync(kFull, bkey == wkey ? (unsigned)bj : 0x7fffffffu);
            if (lane == 0) { s_key[g][gw] = wkey; s_j[g][gw] = wj; }
            group_bar<GW>(g);
            unsigned long long best = s_key[g][0];
            int j1 = s_j[g][0];
#pragma unroll
            for (int q = 1; q < GW; ++q) {
                const unsigned long long kq = s_key[g][q];
                const int jq = s_j[g][q];
                if (kq < best || (kq == best && jq < j1)) { best = kq; j1 = jq; }
            }
            if (j1 == 0x7fffffff) return false;
            const double bv = key_fp64(best);
            if (!isfinite(bv)) return false;
            if (gt == 0) w.u[i] += bv;
#pragma unroll
            for (int t = 0; t < CPL; ++t) {
                if (!valid[t]) continue;
                if (used[t]) { w.u[pr[t]] += bv; pv[t] -= bv; }
                else minv[t] -= bv;
            }
            const int owner = (j1 - 1) % GT, slot = (j1 - 1) / GT;
            if (gt == owner) {
#pragma unroll
                for (int t = 0; t < CPL; ++t)
                    if (t == slot) { used[t] = true; s_row[g] = pr[t]; }
            }
            group_bar<GW>(g);
            const int pj = s_row[g];
            j0 = j1;
            if (pj == 0) { done = true; break; }
            i0 = pj;
        }
        if (!done) return false;   // no augmenting path within k+1 steps
        // flip the path in shared memory: column jj takes the row of way[jj]
#pragma unroll
        for (int t = 0; t < CPL; ++t)
            if (valid[t]) {
                const int j = gt + 1 + GT * t;
                w.way[j] = way[t];
                w.p[j] = pr[t];
            }
        group_bar<GW>(g);
        if (gt == 0) {
            w.p[0] = i;
            int jj = j0;
            for (int guard = 0; guard <= k && jj != 0; ++guard) {
                const int jp = w.way[jj];
                w.p[jj] = w.p[jp];
                jj = jp;
            }
        }
        group_bar<GW>(g);
#pragma unroll
        for (int t = 0; t < CPL; ++t)
            if (valid[t]) pr[t] = w.p[gt + 1 + GT * t];
    }
#pragma unroll
    for (int t = 0; t < CPL; ++t) {
        if (!valid[t]) continue;
        const int r = w.rows[pr[t] - 1];
        out[r * m + colE[t]] = 1.0;
        w.pi[r] = colE[t];
    }
    group_bar<GW>(g);
    return true;
}

// The Hungarian on group g (all 32*GW of its threads call it): pre-pass on the
// group's first warp, solve on all of them; beyond 128*GW free columns the
// first warp runs the shared-memory loop. Same result as hungarian_warp.
template <int GW = kHungWarps>
static __device__ bool hungarian_group(const HW& w, int m, const double* cost, double sign, const double* lb,
                                       const double* ub, const double* face, double* out, const uint8_t* code,
                                       int g) {
    constexpr int GT = GW * 32;
    __shared__ int s_k[2];
    const int gt = threadIdx.x - GT * g;
    if (gt < 32) {
        const int k = hung_prepass(w, m, lb, ub, face, out);
        if (gt == 0) s_k[g] = k;
    }
    group_bar<GW>(g);
    const int k = s_k[g];
    if (k < 0) return false;
    if (k <= GT) return hung_solve_group<1, GW>(w, m, k, cost, sign, ub, face, out, code, g);
    if (k <= 2 * GT) return hung_solve_group<2, GW>(w, m, k, cost, sign, ub, face, out, code, g);
    if (k <= 4 * GT) return hung_solve_group<4, GW>(w, m, k, cost, sign, ub, face, out, code, g);
    if (gt < 32) {
        const bool ok = hung_solve_smem(w, m, k, cost, sign, ub, face, out, code);
        if (gt == 0) s_k[g] = ok ? 1 : 0;
    }
    group_bar<GW>(g);
    return s_k[g] != 0;
}

// Perfect matching of the allowed edges honouring the forced ones, for the
// feasibility test of a Birkhoff node: greedy lowest-column choice, then
// augmenting paths for the rows it could not place. Executed by ONE warp;
// `out` must be zeroed and visible. Returns 0 when no perfect matching exists
// (contradictory bounds included), 1 with a perfect matching in out and w.pi,
// and 2 only above order 1024 (the augmenting-path search's visited set) --
// then the caller falls back to the Hungarian.
static __device__ int greedy_matching_warp(const HW& w, int m, const double* lb, const double* ub,
                                           double* out) {
    const int lane = threadIdx.x & 31;
    for (int i = lane; i < m; i += 32) { w.fcol[i] = -1; w.frow[i] = -1; }
    __syncwarp();
    bool ok = true;
    const int nn = m * m;
    for (int e = lane; e < nn; e += 32) {
        const double le = lb[e], ue = ub[e];
        if (le > ue + 1e-9) ok = false;
        if (le > 0.5) {
            const int r = e / m, col = e - r * m;
            if (ue < 0.5) ok = false;
            if (atomicCAS(&w.fcol[r], -1, col) != -1) ok = false;
            if (atomicCAS(&w.frow[col], -1, r) != -1) ok = false;
        }
    }
    ok = __all_sync(kFull, ok);
    __syncwarp();
    if (!ok) return 0;
    int k = 0, kc = 0;
    const unsigned lt = (1u << lane) - 1u;
    for (int base = 0; base < m; base += 32) {
        const int i = base + lane;
        const bool fr = i < m && w.fcol[i] < 0;
        const bool fc = i < m && w.frow[i] < 0;
        const unsigned mr = __ballot_sync(kFull, fr), mc = __ballot_sync(kFull, fc);
        if (fr) w.rows[k + __popc(mr & lt)] = i;
        if (fc) w.cols[kc + __popc(mc & lt)] = i;
        k += __popc(mr);
        kc += __popc(mc);
    }
    if (k != kc) return 0;
    // matchR[t] = column position of compacted row t (w.p), matchC[pos] = row (w.way)
    int* matchR = w.p;
    int* matchC = w.way;
    for (int j = lane; j < k; j += 32) { w.used[j] = 0; matchR[j] = -1; matchC[j] = -1; }
    __syncwarp();
    int first = 0;  // lowest position that may still be free
    int stuck = 0;
    for (int t = 0; t < k; ++t) {
        const int r = w.rows[t];
        int pick = -1;
        for (int base = first & ~31; base < k && pick < 0; base += 32) {
            const int pos = base + lane;
            const bool cand = pos < k && !w.used[pos] && ub[r * m + w.cols[pos]] >= 0.5;
            const unsigned b = __ballot_sync(kFull, cand);
            if (b) pick = base + __ffs(b) - 1;
        }
        if (pick < 0) { ++stuck; continue; }
        if (lane == 0) { w.used[pick] = 1; matchR[t] = pick; matchC[pick] = t; }
        __syncwarp();
        while (first < k && w.used[first]) ++first;
    }
    if (stuck) {
        // augmenting paths (Kuhn) over allowed-edge bitmasks of the compacted
        // rows: exact, so a row without an augmenting path means no perfect matching
        const int W = (k + 31) >> 5;
        if (W > 32) return 2;   // beyond the visited set below (orders above 1024)
        // [k][W] words over u, pv, minv, or over the caller's m*m doubles when
        // larger (k W <= m ceil(m/32) <= 2 m^2 words); the latter are cleared
        // before the matching is written
        const bool in_out = (size_t)k * W > 6 * (size_t)(m + 1);
        unsigned* mask = reinterpret_cast<unsigned*>(in_out ? out : w.u);
        for (int t = 0; t < k; ++t) {
            const int r = w.rows[t];
            for (int base = 0; base < k; base += 32) {
                const int pos = base + lane;
                const unsigned b = __ballot_sync(kFull, pos < k && ub[r * m + w.cols[pos]] >= 0.5);
                if (lane == 0) mask[t * W + (base >> 5)] = b;
            }
        }
        __syncwarp();
        int ok = 1;
        if (lane == 0) {
            int* queue = w.pi;      // BFS queue of compacted rows (pi is written last)
            int* parent = w.pinv;   // row that reached each column position
            unsigned vis[32];
            for (int t0 = 0; t0 < k && ok; ++t0) {
                if (matchR[t0] >= 0) continue;
                for (int q = 0; q < W; ++q) vis[q] = 0u;
                int head = 0, tail = 0, found = -1;
                queue[tail++] = t0;
                while (head < tail && found < 0) {
                    const int t = queue[head++];
                    for (int q = 0; q < W && found < 0; ++q) {
                        unsigned cand = mask[t * W + q] & ~vis[q];
                        while (cand && found < 0) {
                            const int bit = __ffs(cand) - 1;
                            cand &= cand - 1;
                            const int pos = q * 32 + bit;
                            vis[q] |= 1u << bit;
                            parent[pos] = t;
                            if (matchC[pos] < 0) found = pos;
                            else queue[tail++] = matchC[pos];
                        }
                    }
                }
                if (found < 0) { ok = 0; break; }
                for (int pos = found; pos >= 0;) {   // flip the path back to t0
                    const int t = parent[pos];
                    const int prev = matchR[t];
                    matchR[t] = pos;
                    matchC[pos] = t;
                    pos = t == t0 ? -1 : prev;
                }
            }
        }
        ok = __shfl_sync(kFull, ok, 0);
        __syncwarp();
        if (in_out) {
            for (int e = lane; e < nn; e += 32) out[e] = 0.0;
            __syncwarp();
        }
        if (!ok) return 0;
    }
    for (int t = lane; t < k; t += 32) {
        const int r = w.rows[t], col = w.cols[matchR[t]];
        w.pi[r] = col;
        out[r * m + col] = 1.0;
    }
    for (int i = lane; i < m; i += 32)
        if (w.fcol[i] >= 0) { out[i * m + w.fcol[i]] = 1.0; w.pi[i] = w.fcol[i]; }
    __syncwarp();
    return 1;
}

// ------------------------------------------------------------------ simplex
// parallel_greedy_allocate_cooperative (lmo.cuh:529-618); key of j is sign*g[j].
static __device__ void simplex_greedy(const Ctx& c, const double* g, double sign, const double* ub,
                               double* out, const uint8_t* fixed, double remaining,
                               bool force_full, bool floor_int) {
    const int S = c.S, n = c.n, tid = c.tid;
    const bool eq = c.lk == GBX_LMO_EQUALITY_SIMPLEX;
    for (int pos = tid; pos < S; pos += kThreads) {
        bool el = pos < n && (!fixed || !fixed[pos]);
        double key = CUDART_INF;
        if (el) {
            key = sign * g[pos];
            el = force_full || key <= 0.0;
        }
        c.keys[pos] = el ? key : CUDART_INF;
        c.idx[pos] = el ? pos : -1;
    }
    __syncthreads();
    for (int width = 2; width <= S; width <<= 1)
        for (int stride = width >> 1; stride > 0; stride >>= 1) {
            for (int left = tid; left < S; left += kThreads) {
                const int right = left ^ stride;
                if (right <= left) continue;
                const double lk = c.keys[left], rk = c.keys[right];
                const int li = c.idx[left], ri = c.idx[right];
                const bool after = rk < lk || (rk == lk && ri >= 0 && (li < 0 || ri < li));
                const bool asc = (left & width) == 0;
                if (after == asc) {
                    c.keys[left] = rk; c.keys[right] = lk;
                    c.idx[left] = ri; c.idx[right] = li;
                }
            }
            __syncthreads();
        }
    const uint8_t* isint = c.is_int;
    for (int pos = tid; pos < S; pos += kThreads) {
        const int j = c.idx[pos];
        c.prefix[pos] = j < 0 ? 0.0
            : ((isint && isint[j]) ? fmax(ub[j] - out[j], 0.0) : remaining);
    }
    __syncthreads();
    for (int off = 1; off < S; off <<= 1) {
        for (int op = tid; op < S / (off << 1); op += kThreads) {
            const int right = (op + 1) * (off << 1) - 1;
            c.prefix[right] += c.prefix[right - off];
        }
        __syncthreads();
    }
    if (tid == 0) c.prefix[S - 1] = 0.0;
    __syncthreads();
    for (int off = S >> 1; off > 0; off >>= 1) {
        for (int op = tid; op < S / (off << 1); op += kThreads) {
            const int right = (op + 1) * (off << 1) - 1;
            const double ls = c.prefix[right - off];
            c.prefix[right - off] = c.prefix[right];
            c.prefix[right] += ls;
        }
        __syncthreads();
    }
    for (int pos = tid; pos < S; pos += kThreads) {
        const int j = c.idx[pos];
        if (j < 0) continue;
        const bool ij = isint && isint[j];
        double add = fmax(remaining - c.prefix[pos], 0.0);
        const double cap = ij ? fmax(ub[j] - out[j], 0.0) : remaining;
        add = fmin(add, cap);
        if (floor_int && ij) add = floor(add + (eq ? 1e-9 : 0.0));
        out[j] += add;
    }
    __syncthreads();
}

// ------------------------------------------------------------------ cardinality LMO
// 256-lane min padded with +inf (bmin pads with 1.0 for step sizes).
static __device__ double bmin_inf(double v, double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warp_min(v);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        double r = lane < kWarps ? red[lane] : CUDART_INF;
        r = warp_min(r);
        if (lane == 0) red[34] = r;
    }
    __syncthreads();
    return red[34];
}

// min <g, (w, z)> over {sum w = 1, 0 <= w <= z, sum z <= K, 0 <= z <= 1} with z
// forced (lb > 1/2) or forbidden (ub < 1/2). A vertex puts w = e_a on one asset
// a (z_a = 1) and switches on z for the forced assets and for the most negative
// remaining z-costs while slots are left. With L = free assets of negative
// z-cost sorted by (cost, index) and P its prefix sums (left to right), base =
// sum of forced z-costs (index order), r0 = K - #forced, r1 = r0 - 1:
//   a forced:              (g_w[a] + base) + P[r0]
//   a among first r1 of L: (g_w[a] + base) + P[r1 + 1]
//   otherwise:             (g_w[a] + base) + (g_z[a] + P[r1])
// (P clamped at |L|); the minimum, lowest asset on ties, is the vertex.
static __device__ bool card_forward(const Ctx& c, const double* g, const double* lb, const double* ub,
                                    double* v) {
    __shared__ int s_arg;
    const int n = c.n, N = n / 2, tid = c.tid;
    const int K = (int)floor(c.rhs + 1e-9);
    int* pos = reinterpret_cast<int*>(c.keys);
    int* ord = c.idx;
    double* P = c.prefix;
    for (int j = tid; j < n; j += kThreads) v[j] = 0.0;
    for (int j = tid; j < N; j += kThreads) {
        const double gz = g[N + j];
        int rank = -1;
        if (!(lb[N + j] > 0.5) && !(ub[N + j] < 0.5) && gz < 0.0) {
            rank = 0;
            for (int k = 0; k < N; ++k) {
                const double gk = g[N + k];
                if (lb[N + k] > 0.5 || ub[N + k] < 0.5 || !(gk < 0.0)) continue;
                if (gk < gz || (gk == gz && k < j)) ++rank;
            }
            ord[rank] = j;
        }
        pos[j] = rank;
    }
    __syncthreads();
    if (tid == 0) {
        int nf = 0, nl = 0;
        double base = 0.0;
        for (int j = 0; j < N; ++j) {
            if (lb[N + j] > 0.5) { ++nf; base = base + g[N + j]; }
            if (pos[j] >= 0) ++nl;
        }
        P[0] = 0.0;
        for (int t = 0; t < nl; ++t) P[t + 1] = P[t] + g[N + ord[t]];
        c.flag[6] = nf;
        c.flag[7] = nl;
        c.red[38] = base;
        s_arg = 0x7fffffff;
    }
    __syncthreads();
    const int nf = c.flag[6], nl = c.flag[7];
    const double base = c.red[38];
    if (nf > K) return false;
    const int r0 = K - nf, r1 = K - nf - 1;
    auto value = [&](int a) -> double {
        if (ub[N + a] < 0.5) return CUDART_INF;
        const double head = g[a] + base;
        double val;
        if (lb[N + a] > 0.5) val = head + P[min(r0, nl)];
        else if (r1 < 0) return CUDART_INF;
        else if (pos[a] >= 0 && pos[a] < r1) val = head + P[min(r1 + 1, nl)];
        else val = head + (g[N + a] + P[min(r1, nl)]);
        return val < CUDART_INF ? val : CUDART_INF;
    };
    double best = CUDART_INF;
    for (int a = tid; a < N; a += kThreads) best = fmin(best, value(a));
    const double vmin = bmin_inf(best, c.red);
    if (!(vmin < CUDART_INF)) return false;
    for (int a = tid; a < N; a += kThreads)
        if (value(a) == vmin) { atomicMin(&s_arg, a); break; }
    __syncthreads();
    const int a = s_arg;
    const bool af = lb[N + a] > 0.5;
    int limit;
    if (af) limit = min(r0, nl);
    else if (pos[a] >= 0 && pos[a] < r1) limit = min(r1 + 1, nl);
    else limit = min(r1, nl);
    for (int j = tid; j < N; j += kThreads)
        if (lb[N + j] > 0.5 || (pos[j] >= 0 && pos[j] < limit) || j == a) v[N + j] = 1.0;
    if (tid == 0) v[a] = 1.0;
    __syncthreads();
    return true;
}

// Linked cardinality {(v, y): 0 <= v_i <= U_i y_i, sum y <= m, 0 <= y <= 1}
// (the sparse-Sharpe LinkedCardinalityLMO, examples/sparse_sharpe.cu:266-546):
// v_i at i, y_i at n/2 + i for the first `order` assets (the rest of each half
// is padding and stays 0); branching fixes y. Ranks by (cost, asset) are
// counted directly instead of sorted: rank(i) = #{k eligible : (c_k, k) < (c_i, i)}.
struct Linked {
    int half, assets, m;
};
static __device__ inline Linked linked_of(const Ctx& c) {
    Linked L;
    L.half = c.n / 2;
    L.assets = c.lorder > 0 ? min(c.lorder, L.half) : L.half;
    L.m = (int)floor(c.rhs + 1e-9);
    return L;
}

// compute_v: the mandatory assets (lb_y > 1/2), then up to m - mandatory
// optional assets of negative joint cost g_y + min(0, U g_v), cheapest first;
// a selected asset takes v = U when g_v < 0
static __device__ void linked_forward(const Ctx& c, const double* g, const double* lb, const double* ub,
                                      double* v) {
    const Linked L = linked_of(c);
    const int h = L.half;
    int mand = 0;
    for (int j = c.tid; j < c.n; j += kThreads) v[j] = 0.0;
    for (int i = c.tid; i < L.assets; i += kThreads) mand += lb[h + i] > 0.5 ? 1 : 0;
    const int nm = (int)bsum((double)mand, c.red);
    if (nm > L.m) return;   // node_feasible rejects such nodes first
    const int slots = L.m - nm;
    auto cost = [&](int i) { return g[h + i] + fmin(0.0, c.U[i] * g[i]); };
    auto eligible = [&](int i, double ci) { return ci < 0.0 && lb[h + i] <= 0.5 && ub[h + i] > 0.5; };
    for (int i = c.tid; i < L.assets; i += kThreads) {
        bool take = lb[h + i] > 0.5;
        if (!take && slots > 0) {
            const double ci = cost(i);
            if (eligible(i, ci)) {
                int rank = 0;
                for (int k = 0; k < L.assets && rank < slots; ++k) {
                    if (k == i) continue;
                    const double ck = cost(k);
                    if (eligible(k, ck) && (ck < ci || (ck == ci && k < i))) ++rank;
                }
                take = rank < slots;
            }
        }
        if (take) {
            v[h + i] = 1.0;
            v[i] = g[i] < 0.0 ? c.U[i] : 0.0;
        }
    }
    __syncthreads();
}

// compute_inface_v on the direction sign*g: y entries at a bound stay there,
// v keeps its zero / linked (v = U y) state, and the free y take the cheapest
// costs (all of them, cheapest first, when sum y = m is active)
static __device__ void linked_inface(const Ctx& c, const double* g, double sign, const double* x,
                                     const double* lb, const double* ub, double* a) {
    const double atol = 1e-6, rtol = 1e-4;
    const Linked L = linked_of(c);
    const int h = L.half;
    struct Face { bool yf, vz, la; double fy; };
    auto face = [&](int i) {
        Face f;
        const double U = c.U[i], vi = x[i], yi = x[h + i];
        const bool lo = fabs(yi - lb[h + i]) <= atol + rtol * fmax(fabs(yi), fabs(lb[h + i]));
        const bool up = fabs(yi - ub[h + i]) <= atol + rtol * fmax(fabs(yi), fabs(ub[h + i]));
        f.yf = lo || up;
        f.fy = lo ? lb[h + i] : ub[h + i];
        f.vz = fabs(vi) <= atol + rtol * fabs(vi);
        f.la = fabs(vi - U * yi) <= atol + rtol * fmax(fabs(vi), fabs(U * yi));
        return f;
    };
    auto cost = [&](int i, const Face& f) {
        const double gv = sign * g[i];
        double ci = sign * g[h + i];
        if (f.la) ci += c.U[i] * gv;
        else if (!f.vz) ci += fmin(0.0, c.U[i] * gv);
        return ci;
    };
    for (int j = c.tid; j < c.n; j += kThreads) a[j] = 0.0;
    int fsel = 0;
    double sy = 0.0;
    for (int i = c.tid; i < L.assets; i += kThreads) {
        const Face f = face(i);
        if (f.yf) {
            a[h + i] = f.fy;
            if (f.fy > 0.5) ++fsel;
            if (!f.vz) a[i] = f.la ? c.U[i] * f.fy : (sign * g[i] < 0.0 ? c.U[i] * f.fy : 0.0);
        }
        sy += x[h + i];
    }
    const int fixed_sel = (int)bsum((double)fsel, c.red);
    const double sum_y = bsum(sy, c.red);
    const bool full = fabs(sum_y - L.m) <= atol + rtol * fmax(fabs(sum_y), (double)L.m);
    const int slots = L.m - fixed_sel;
    for (int i = c.tid; i < L.assets; i += kThreads) {
        const Face f = face(i);
        if (f.yf || slots <= 0) continue;
        const double ci = cost(i, f);
        if (!(full || ci < 0.0)) continue;
        int rank = 0;
        for (int k = 0; k < L.assets && rank < slots; ++k) {
            if (k == i) continue;
            const Face fk = face(k);
            if (fk.yf) continue;
            const double ck = cost(k, fk);
            if ((full || ck < 0.0) && (ck < ci || (ck == ci && k < i))) ++rank;
        }
        if (rank < slots) {
            a[h + i] = 1.0;
            a[i] = f.la ? c.U[i] : (!f.vz ? (sign * g[i] < 0.0 ? c.U[i] : 0.0) : 0.0);
        }
    }
    __syncthreads();
}

// integer_candidate_device: the mandatory assets plus the largest positive v
// of x up to m, v taken from x (or the asset of largest mu = -ls c when x has
// no positive v), scaled to the objective's minimum along that direction,
// t = -ls c'd / d'Qd, capped by U_i / d_i. Thread 0, assets in order.
static __device__ void linked_candidate(const Ctx& c, const double* x, const double* lb, const double* ub,
                                        double* cand) {
    const Linked L = linked_of(c);
    const int h = L.half, n = c.n;
    for (int j = c.tid; j < n; j += kThreads) cand[j] = 0.0;
    __syncthreads();
    if (c.tid == 0) {
        auto mu = [&](int i) { return c.c ? -c.ls * c.c[i] : 0.0; };
        int selected = 0;
        for (int i = 0; i < L.assets; ++i)
            if (lb[h + i] > 0.5) { cand[h + i] = 1.0; ++selected; }
        while (selected < L.m) {
            int best = -1;
            for (int i = 0; i < L.assets; ++i)
                if (cand[h + i] == 0.0 && ub[h + i] > 0.5 && x[i] > 1e-12 && (best < 0 || x[i] > x[best])) best = i;
            if (best < 0) break;
            cand[h + best] = 1.0;
            ++selected;
        }
        bool direction = false;
        for (int i = 0; i < L.assets; ++i)
            if (cand[h + i] == 1.0) {
                cand[i] = fmax(0.0, x[i]);
                direction = direction || cand[i] > 0.0;
            }
        if (!direction) {
            int best = -1;
            for (int i = 0; i < L.assets; ++i)
                if ((cand[h + i] == 1.0 || (selected < L.m && ub[h + i] > 0.5)) && (best < 0 || mu(i) > mu(best)))
                    best = i;
            if (best >= 0 && mu(best) > 0.0) {
                cand[h + best] = 1.0;
                cand[best] = 1.0;
            }
        }
        double lin = 0.0, quad = 0.0, cap = CUDART_INF;
        for (int i = 0; i < L.assets; ++i) {
            lin += mu(i) * cand[i];
            if (cand[i] > 0.0) cap = fmin(cap, c.U[i] / cand[i]);
            for (int j = 0; j < L.assets; ++j) quad += cand[i] * c.Q[(size_t)i * n + j] * cand[j];
        }
        const double t = lin > 0.0 && quad > 0.0 ? fmin(lin / quad, cap) : 0.0;
        for (int i = 0; i < L.assets; ++i) cand[i] *= t;
    }
    __syncthreads();
}

// ------------------------------------------------------------------ LMOs
template <int LK>
static __device__ bool lmo_forward(const Ctx& c, const double* g, const double* lb,
                            const double* ub, double* v) {
    const int n = c.n;
    if constexpr (LK == GBX_LMO_BOX) {
        for (int j = c.tid; j < n; j += kThreads) v[j] = g[j] > 0.0 ? lb[j] : ub[j];
        __syncthreads();
        return false;
    } else if constexpr (LK == GBX_LMO_BIRKHOFF) {
        for (int j = c.tid; j < n; j += kThreads) v[j] = 0.0;
        __syncthreads();
        if (n != c.lorder * c.lorder) return false;
        {   // a lone oracle: the whole CTA as one group of eight warps
            const HW w = hw_at(c.hung[0], c.lorder);
            const bool ok = hungarian_group<8>(w, c.lorder, g, 1.0, lb, ub, nullptr, v, nullptr, 0);
            if (threadIdx.x == 0) c.flag[0] = ok;
        }
        __syncthreads();
        return c.flag[0] != 0;
    } else if constexpr (LK == GBX_LMO_CARDINALITY) {
        card_forward(c, g, lb, ub, v);
        return false;
    } else if constexpr (LK == GBX_LMO_LINKED_CARDINALITY) {
        linked_forward(c, g, lb, ub, v);
        return false;
    } else {
        double loc = 0.0;
        for (int j = c.tid; j < n; j += kThreads) {
            if (c.is_int && c.is_int[j]) { v[j] = lb[j]; loc += v[j]; }
            else v[j] = 0.0;
        }
        const double mass = bsum(loc, c.red);
        const bool eq = LK == GBX_LMO_EQUALITY_SIMPLEX;
        simplex_greedy(c, g, 1.0, ub, v, nullptr, c.rhs - mass, eq, eq);
        return false;
    }
}

// In-face away oracle on the direction sign*g over the minimal face of x.
template <int LK>
static __device__ bool lmo_inface(const Ctx& c, const double* g, double sign, const double* x,
                           const double* lb, const double* ub, double* a, int hw_slot) {
    const int n = c.n;
    const double atol = 1e-6, rtol = 1e-4;
    if constexpr (LK == GBX_LMO_BOX) {
        for (int j = c.tid; j < n; j += kThreads) {
            const double ut = atol + rtol * fabs(ub[j]);
            const double lt = atol + rtol * fabs(lb[j]);
            if (fabs(x[j] - ub[j]) <= ut) a[j] = ub[j];
            else if (fabs(x[j] - lb[j]) <= lt) a[j] = lb[j];
            else a[j] = sign * g[j] > 0.0 ? lb[j] : ub[j];
        }
        __syncthreads();
        return false;
    } else if constexpr (LK == GBX_LMO_BIRKHOFF) {
        // caller zeroes `a` and runs this on one warp
        const HW w = hw_at(c.hung[hw_slot], c.lorder);
        return hungarian_warp(w, c.lorder, g, sign, lb, ub, x, a);
    } else if constexpr (LK == GBX_LMO_CARDINALITY) {
        // Frank-Wolfe only: the host rejects DICG and in-face probes for this set
        for (int j = c.tid; j < n; j += kThreads) a[j] = x[j];
        __syncthreads();
        return false;
    } else if constexpr (LK == GBX_LMO_LINKED_CARDINALITY) {
        linked_inface(c, g, sign, x, lb, ub, a);
        return false;
    } else {
        double lm = 0.0, lx = 0.0;
        for (int j = c.tid; j < n; j += kThreads) {
            const bool ij = c.is_int && c.is_int[j];
            c.fixed[j] = 0;
            a[j] = ij ? lb[j] : 0.0;
            const double lower = ij ? lb[j] : 0.0;
            const double ltol = atol + rtol * fmax(fabs(x[j]), fabs(lower));
            if (fabs(x[j] - lower) <= ltol) {
                c.fixed[j] = 1;
                a[j] = lower;
            } else if (ij) {
                const double utol = atol + rtol * fmax(fabs(x[j]), fabs(ub[j]));
                if (fabs(x[j] - ub[j]) <= utol) { c.fixed[j] = 1; a[j] = ub[j]; }
            }
            lm += a[j];
            lx += x[j];
        }
        const double mass = bsum(lm, c.red);
        const double xmass = bsum(lx, c.red);
        const bool eq = LK == GBX_LMO_EQUALITY_SIMPLEX;
        const bool force = eq || fabs(xmass - c.rhs) <= atol + rtol * fmax(fabs(xmass), fabs(c.rhs));
        simplex_greedy(c, g, sign, ub, a, c.fixed, c.rhs - mass, force, true);
        return false;
    }
}

// max(0, min(coordinate step, aggregate step)) for x - gamma*d.
template <int LK>
static __device__ double lmo_max_step(const Ctx& c, const double* d, const double* x,
                               const double* lb, const double* ub) {
    const int n = c.n;
    double res = 1.0;
    if constexpr (LK == GBX_LMO_LINKED_CARDINALITY) {
        // dicg_maximum_step_local and dicg_sum_maximum_step
        const Linked L = linked_of(c);
        const int h = L.half;
        const double tol = 1e-9;
        double sx = 0.0, sd = 0.0;
        for (int i = c.tid; i < L.assets; i += kThreads) {
            const double dv = d[i], dy = d[h + i];
            if (dv > tol) res = fmin(res, x[i] / dv);
            const double link_d = dv - c.U[i] * dy;
            const double link_x = x[i] - c.U[i] * x[h + i];
            if (link_d < -tol) res = fmin(res, link_x / link_d);
            if (dy > tol) res = fmin(res, (x[h + i] - lb[h + i]) / dy);
            else if (dy < -tol) res = fmin(res, (ub[h + i] - x[h + i]) / -dy);
            sx += x[h + i];
            sd += dy;
        }
        const double coord = bmin(res, c.red);
        const double sum_x = bsum(sx, c.red);
        const double sum_d = bsum(sd, c.red);
        const double agg = sum_d < -1e-9 ? fmax(0.0, fmin(1.0, (sum_x - L.m) / sum_d)) : 1.0;
        return fmax(0.0, fmin(coord, agg));
    } else {
        for (int j = c.tid; j < n; j += kThreads) {
            const double dj = d[j];
            if constexpr (LK == GBX_LMO_BOX) {
                if (dj < 0.0) res = fmin(res, (ub[j] - x[j]) / -dj);
                else if (dj > 0.0) res = fmin(res, (x[j] - lb[j]) / dj);
            } else if constexpr (LK == GBX_LMO_BIRKHOFF || LK == GBX_LMO_CARDINALITY) {
                if (dj > 0.0) res = fmin(res, (x[j] - lb[j]) / dj);
                else if (dj < 0.0) res = fmin(res, (ub[j] - x[j]) / -dj);
            } else {
                const bool ij = c.is_int && c.is_int[j];
                if (dj > 1e-6) res = fmin(res, (x[j] - (ij ? lb[j] : 0.0)) / dj);
                else if (dj < -1e-6) res = fmin(res, ((ij ? ub[j] : c.rhs) - x[j]) / -dj);
            }
        }
        const double coord = bmin(res, c.red);
        double agg = 1.0;
        if constexpr (LK == GBX_LMO_SIMPLEX || LK == GBX_LMO_EQUALITY_SIMPLEX) {
            double sx = 0.0, sd = 0.0;
            for (int j = c.tid; j < n; j += kThreads) { sx += x[j]; sd += d[j]; }
            const double sum_x = bsum(sx, c.red);
            const double sum_d = bsum(sd, c.red);
            if (LK == GBX_LMO_EQUALITY_SIMPLEX && fabs(sum_d) > 1e-9) agg = 0.0;
            else agg = sum_d < 0.0 ? fmin(1.0, (sum_x - c.rhs) / sum_d) : 1.0;
        }
        return fmax(0.0, fmin(coord, agg));
    }
}

// drs_node_feasible (device_resident_solver.cuh:206-217) + LMO check.
template <int LK>
static __device__ bool node_feasible(const Ctx& c, const double* lb, const double* ub,
                              double* scratch) {
    const int n = c.n;
    bool valid = true;
    for (int j = c.tid; j < n; j += kThreads)
        if (isnan(lb[j]) || isnan(ub[j]) || lb[j] > ub[j]
                || (c.flags && c.flags[j] && ceil(lb[j]) > floor(ub[j])))
            valid = false;
    if (!__syncthreads_and(valid)) return false;
    if constexpr (LK == GBX_LMO_BOX) {
        return true;
    } else if constexpr (LK == GBX_LMO_BIRKHOFF) {
        if (n != c.lorder * c.lorder) return false;
        for (int j = c.tid; j < n; j += kThreads) scratch[j] = 0.0;
        __syncthreads();
        // a perfect matching of the allowed edges exists (the reference runs the
        // Hungarian on zero costs); the greedy matching settles almost every node
        if (threadIdx.x < 32) {
            const HW w = hw_at(c.hung[0], c.lorder);
            int r = greedy_matching_warp(w, c.lorder, lb, ub, scratch);
            if (r == 2) {
                for (int j = threadIdx.x; j < n; j += 32) scratch[j] = 0.0;
                __syncwarp();
                r = hungarian_warp<2>(w, c.lorder, nullptr, 1.0, lb, ub, nullptr, scratch) ? 1 : 0;
            }
            if (threadIdx.x == 0) c.flag[1] = r;
        }
        __syncthreads();
        return c.flag[1] != 0;
    } else if constexpr (LK == GBX_LMO_CARDINALITY) {
        const int N = n / 2;
        const int K = (int)floor(c.rhs + 1e-9);
        int forced = 0;
        bool open = false;
        for (int j = c.tid; j < N; j += kThreads) {
            forced += lb[N + j] > 0.5 ? 1 : 0;
            open = open || !(ub[N + j] < 0.5);
        }
        const int nf = (int)bsum((double)forced, c.red);
        const bool any_open = __syncthreads_or(open) != 0;
        return nf <= K && (nf >= 1 || (K >= 1 && any_open));
    } else if constexpr (LK == GBX_LMO_LINKED_CARDINALITY) {
        const Linked L = linked_of(c);
        int mand = 0;
        for (int i = c.tid; i < L.assets; i += kThreads) mand += lb[L.half + i] > 0.5 ? 1 : 0;
        return (int)bsum((double)mand, c.red) <= L.m;
    } else {
        bool v2 = true, cont = false;
        double mand = 0.0, cap = 0.0;
        for (int j = c.tid; j < n; j += kThreads) {
            const bool integer = c.flags ? c.flags[j] != 0 : (c.is_int && c.is_int[j]);
            const double lo = integer ? ceil(fmax(0.0, lb[j])) : fmax(0.0, lb[j]);
            const double hi = integer ? floor(ub[j]) : ub[j];
            v2 = v2 && lo <= hi;
            mand += lo;
            cap += hi;
            cont = cont || !integer;
        }
        const bool iv = __syncthreads_and(v2);
        const double ms = bsum(mand, c.red);
        bool feas = iv && ms <= c.rhs + 1e-9;
        if (LK == GBX_LMO_EQUALITY_SIMPLEX) {
            const double cs = bsum(cap, c.red);
            const bool hc = __syncthreads_or(cont);
            feas = feas && cs >= c.rhs - 1e-9
                && (hc || fabs(c.rhs - round(c.rhs)) <= 1e-9);
        }
        return feas;
    }
}

template <int LK>
static __device__ bool rounded_feasible(const Ctx& c, const double* x) {
    const int n = c.n;
    const double tol = c.tol;
    if constexpr (LK == GBX_LMO_BOX) {
        return true;
    } else if constexpr (LK == GBX_LMO_BIRKHOFF) {
        const int m = c.lorder;
        if (n != m * m) return false;
        bool valid = true;
        for (int i = c.tid; i < m; i += kThreads) {
            double row = 0.0, col = 0.0;
            for (int j = 0; j < m; ++j) {
                if (x[i * m + j] < -tol) valid = false;
                row += x[i * m + j];
                col += x[j * m + i];
            }
            if (fabs(row - 1.0) > tol || fabs(col - 1.0) > tol) valid = false;
        }
        return __syncthreads_and(valid);
    } else if constexpr (LK == GBX_LMO_CARDINALITY) {
        const int N = n / 2;
        bool valid = true;
        double sw = 0.0, sz = 0.0;
        for (int j = c.tid; j < N; j += kThreads) {
            const double w = x[j], z = x[N + j];
            valid = valid && w >= -tol && z >= -tol && z <= 1.0 + tol && w <= z + tol;
            sw += w;
            sz += z;
        }
        const bool nn = __syncthreads_and(valid);
        const double SW = bsum(sw, c.red);
        const double SZ = bsum(sz, c.red);
        return nn && fabs(SW - 1.0) <= tol && SZ <= floor(c.rhs + 1e-9) + tol;
    } else if constexpr (LK == GBX_LMO_LINKED_CARDINALITY) {
        // candidate_feasible_device: 0 <= v <= U y, sum y <= m
        const Linked L = linked_of(c);
        bool valid = true;
        double sy = 0.0;
        for (int i = c.tid; i < L.assets; i += kThreads) {
            const double y = x[L.half + i];
            valid = valid && x[i] >= -tol && x[i] <= c.U[i] * y + tol;
            sy += y;
        }
        const bool ok = __syncthreads_and(valid);
        const double SY = bsum(sy, c.red);
        return ok && SY <= L.m + tol;
    } else {
        bool valid = true;
        double s = 0.0;
        for (int j = c.tid; j < n; j += kThreads) { valid = valid && x[j] >= -tol; s += x[j]; }
        const bool nn = __syncthreads_and(valid);
        const double sum = bsum(s, c.red);
        return nn && (LK == GBX_LMO_EQUALITY_SIMPLEX ? fabs(sum - c.rhs) <= tol
                                                    : sum <= c.rhs + tol);
    }
}

// drs_integer_value: score of an LMO vertex or rounded candidate.
static __device__ double integer_value(const Ctx& c, const double* x, const double* lb,
                                const double* ub, const int* pi, int* pinv) {
    bool valid = true;
    const double tol = c.tol;
    for (int j = c.tid; j < c.n; j += kThreads)
        if (!isfinite(x[j]) || x[j] < lb[j] - tol || x[j] > ub[j] + tol
                || (c.flags && c.flags[j] && x[j] != round(x[j])))
            valid = false;
    if (!__syncthreads_and(valid)) return kNone;
    const double val = pi ? perm_value(c, pi, pinv) : obj_value(c, x);
    return isfinite(val) ? val : kNone;
}


// ------------------------------------------------------------------ mixed loop
// Score of a permutation vertex pi (drs_integer_value on a 0/1 point): bounds
// are checked through the per-edge code bytes, the value through perm_value.
static __device__ double perm_score(const Ctx& c, const uint8_t* code, const int* pi, int* pinv) {
    bool valid = true;
    for (int e = c.tid; e < c.n; e += kThreads) {
        const int i = e / c.m, j = e - (e / c.m) * c.m;
        if (!(code[e] & (pi[i] == j ? kOneOk : kZeroOk))) valid = false;
    }
    if (!__syncthreads_and(valid)) return kNone;
    const double val = perm_value(c, pi, pinv);
    return isfinite(val) ? val : kNone;
}

// R = A X - X B and G = 2s (A'R - R B') in FP32 over the nonzero lists of A
// and B (rows of A, columns of B for R; columns of A, rows of B for G): for
// d-regular graphs 4 m^2 d multiply-adds instead of 4 m^3.
static __device__ void grad_f32_sparse(const SparseAB& S, int m, float two_s, const float* X, float* R, float* G) {
    const int n = m * m;
    for (int e = threadIdx.x; e < n; e += kThreads) {
        const int i = e / m, j = e - (e / m) * m;
        float r = 0.f;
        for (int t = S.ptr[0][i]; t < S.ptr[0][i + 1]; ++t) r = fmaf((float)S.val[0][t], X[S.idx[0][t] * m + j], r);
        for (int t = S.ptr[1][j]; t < S.ptr[1][j + 1]; ++t) r = fmaf(-X[i * m + S.idx[1][t]], (float)S.val[1][t], r);
        R[e] = r;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n; e += kThreads) {
        const int p = e / m, q = e - (e / m) * m;
        float acc = 0.f;
        for (int t = S.ptr[2][p]; t < S.ptr[2][p + 1]; ++t) acc = fmaf((float)S.val[2][t], R[S.idx[2][t] * m + q], acc);
        for (int t = S.ptr[3][q]; t < S.ptr[3][q + 1]; ++t) acc = fmaf(-R[p * m + S.idx[3][t]], (float)S.val[3][t], acc);
        G[e] = two_s * acc;
    }
    __syncthreads();
}

// The same R and G for large orders, where X and R live in the workspace,
// bit-identical to grad_f32_sparse. X is sparse (a convex combination of a few
// permutations), so R = A X - X B is built from X's nonzeros: a pass lists
// each row's nonzeros (ascending columns) in the scratch `xc`, `xv`, `xn`;
// then warp w takes rows w, w+8, ... and accumulates row i of R in its
// shared-memory buffer `rows + w*m`: first the rows k of X for the neighbours
// k of i in A (ascending), then, for each nonzero X[i][l] (ascending l), row l
// of B. Every element receives the same multiply-adds in the same order as
// grad_f32_sparse, minus those whose X factor is zero, which leave the sum
// unchanged (a sum started at +0 never becomes -0). G = 2s (A'R - R B') reads
// R densely: the rows of R named by column p of A (coalesced, the list held
// in the lanes' registers), and row p of R staged in the same buffer for the
// gathers through B's rows. B's rows are staged in `lst` when they fit in
// `lst_bytes`, otherwise read from the lists in global memory.
template <int NJ>
static __device__ void grad_f32_rows(const SparseAB& S, int m, float two_s, const float* X, float* R, float* G,
                                     float* rows, unsigned char* lst, size_t lst_bytes, uint16_t* xc, float* xv,
                                     int* xn) {
    constexpr int PB = 8;   // neighbour rows of X fetched together
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    float* acc = rows + (size_t)warp * m;
    // B's rows (list 3): staged in shared memory when they fit
    const int nb = S.ptr[3][m];
    const size_t o_idx = align16((size_t)(m + 1) * sizeof(int));
    const size_t o_val = o_idx + align16((size_t)nb * sizeof(uint16_t));
    const bool staged = lst && o_val + align16((size_t)nb * sizeof(float)) <= lst_bytes && m <= 65535;
    const int* bptr = staged ? reinterpret_cast<const int*>(lst) : S.ptr[3];
    const uint16_t* sidx = reinterpret_cast<const uint16_t*>(lst + o_idx);
    const float* sval = reinterpret_cast<const float*>(lst + o_val);
    if (staged) {
        int* p = reinterpret_cast<int*>(lst);
        uint16_t* ix = reinterpret_cast<uint16_t*>(lst + o_idx);
        float* vl = reinterpret_cast<float*>(lst + o_val);
        for (int q = threadIdx.x; q <= m; q += kThreads) p[q] = S.ptr[3][q];
        for (int t = threadIdx.x; t < nb; t += kThreads) {
            ix[t] = (uint16_t)S.idx[3][t];
            vl[t] = (float)S.val[3][t];
        }
    }
    auto bcol = [&](int t) -> int { return staged ? (int)sidx[t] : S.idx[3][t]; };
    auto bv = [&](int t) -> float { return staged ? sval[t] : (float)S.val[3][t]; };
    // X's nonzeros, row by row, ascending columns (NaN counts as nonzero);
    // orders divisible by 4 read X as float4 and place each lane's nonzeros
    // after the prefix count of the lanes before it
    if ((m & 3) == 0) {
        for (int i = warp; i < m; i += kWarps) {
            int cnt = 0;
            for (int j0 = 0; j0 < m; j0 += 128) {
                const int j = j0 + 4 * lane;
                const float4 v = j < m ? *reinterpret_cast<const float4*>(X + (size_t)i * m + j)
                                       : make_float4(0.f, 0.f, 0.f, 0.f);
                const float vv[4] = {v.x, v.y, v.z, v.w};
                int mine = 0;
#pragma unroll
                for (int cc = 0; cc < 4; ++cc) mine += vv[cc] != 0.f;
                int pre = mine;
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    const int t = __shfl_up_sync(kFull, pre, off);
                    if (lane >= off) pre += t;
                }
                int o = cnt + pre - mine;
#pragma unroll
                for (int cc = 0; cc < 4; ++cc)
                    if (vv[cc] != 0.f) {
                        xc[(size_t)i * m + o] = (uint16_t)(j + cc);
                        xv[(size_t)i * m + o] = vv[cc];
                        ++o;
                    }
                cnt += __shfl_sync(kFull, pre, 31);
            }
            if (lane == 0) xn[i] = cnt;
        }
    } else
    for (int i = warp; i < m; i += kWarps) {
        int cnt = 0;
#pragma unroll 4
        for (int j0 = 0; j0 < m; j0 += 32) {
            const int j = j0 + lane;
            const float v = j < m ? X[(size_t)i * m + j] : 0.f;
            const bool nz = j < m && v != 0.f;
            const unsigned b = __ballot_sync(kFull, nz);
            if (nz) {
                const int o = cnt + __popc(b & lt);
                xc[(size_t)i * m + o] = (uint16_t)j;
                xv[(size_t)i * m + o] = v;
            }
            cnt += __popc(b);
        }
        if (lane == 0) xn[i] = cnt;
    }
    __syncthreads();
    // R, row by row
    for (int i = warp; i < m; i += kWarps) {
        for (int j = lane; j < m; j += 32) acc[j] = 0.f;
        __syncwarp();
        const int a0 = S.ptr[0][i], a1 = S.ptr[0][i + 1];
        for (int tb = a0; tb < a1; tb += PB) {
            const int tc = min(PB, a1 - tb);
            int kk = 0, nk = 0;
            float aa = 0.f;
            if (lane < tc) {
                kk = S.idx[0][tb + lane];
                aa = (float)S.val[0][tb + lane];
                nk = xn[kk];
            }
            // the first 32 nonzeros of each neighbour row, all in flight together
            int pc[PB];
            float pv[PB];
#pragma unroll
            for (int u = 0; u < PB; ++u) {
                const int k = __shfl_sync(kFull, kk, u);
                const int cn = __shfl_sync(kFull, nk, u);
                pc[u] = -1;
                pv[u] = 0.f;
                if (u < tc && lane < cn) {
                    pc[u] = xc[(size_t)k * m + lane];
                    pv[u] = xv[(size_t)k * m + lane];
                }
            }
#pragma unroll
            for (int u = 0; u < PB; ++u) {
                if (u >= tc) break;
                const float a = __shfl_sync(kFull, aa, u);
                const int cn = __shfl_sync(kFull, nk, u);
                if (pc[u] >= 0) acc[pc[u]] = fmaf(a, pv[u], acc[pc[u]]);
                if (cn > 32) {
                    const int k = __shfl_sync(kFull, kk, u);
                    for (int e = 32 + lane; e < cn; e += 32) {
                        const int j = xc[(size_t)k * m + e];
                        acc[j] = fmaf(a, xv[(size_t)k * m + e], acc[j]);
                    }
                }
                __syncwarp();
            }
        }
        // - X B: for each nonzero X[i][l], ascending l, row l of B
        const int ci = xn[i];
        for (int eb = 0; eb < ci; eb += 32) {
            int lc = 0;
            float lx = 0.f;
            if (eb + lane < ci) {
                lc = xc[(size_t)i * m + eb + lane];
                lx = xv[(size_t)i * m + eb + lane];
            }
            const int ec = min(32, ci - eb);
            for (int u = 0; u < ec; ++u) {
                const int l = __shfl_sync(kFull, lc, u);
                const float x = __shfl_sync(kFull, lx, u);
                const int b0 = bptr[l], b1 = bptr[l + 1];
                for (int t = b0 + lane; t < b1; t += 32) {
                    const int j = bcol(t);
                    acc[j] = fmaf(-x, bv(t), acc[j]);
                }
                __syncwarp();
            }
        }
        for (int j = lane; j < m; j += 32) R[(size_t)i * m + j] = acc[j];
        __syncwarp();
    }
    __syncthreads();
    // G's gathers through B's rows read them as a padded table when it fits
    // (entry u of row q at u*m + q: a warp's reads of one entry are
    // consecutive, free of bank conflicts)
    __shared__ int s_dmax;
    if (threadIdx.x == 0) s_dmax = 0;
    __syncthreads();
    {
        int dl = 0;
        for (int q = threadIdx.x; q < m; q += kThreads) dl = max(dl, S.ptr[3][q + 1] - S.ptr[3][q]);
        if (dl) atomicMax(&s_dmax, dl);
    }
    __syncthreads();
    const int D = s_dmax;
    const size_t e_val = align16((size_t)D * m * sizeof(uint16_t));
    const size_t e_len = e_val + align16((size_t)D * m * sizeof(float));
    const bool ell = lst && D > 0 && e_len + align16((size_t)m * sizeof(int)) <= lst_bytes && m <= 65535;
    uint16_t* eidx = reinterpret_cast<uint16_t*>(lst);
    float* evl = reinterpret_cast<float*>(lst + e_val);
    int* elen = reinterpret_cast<int*>(lst + e_len);
    if (ell) {
        for (int x = threadIdx.x; x < D * m; x += kThreads) {
            const int u = x / m, q = x - (x / m) * m;
            const int b0 = S.ptr[3][q], len = S.ptr[3][q + 1] - b0;
            eidx[x] = u < len ? (uint16_t)S.idx[3][b0 + u] : (uint16_t)0;
            evl[x] = u < len ? (float)S.val[3][b0 + u] : 0.f;
        }
        for (int q = threadIdx.x; q < m; q += kThreads) elen[q] = S.ptr[3][q + 1] - S.ptr[3][q];
    }
    __syncthreads();
    // G, row by row: A' R through column p of A, then - R B' through B's rows.
    // Orders divisible by 4 read R's rows as float4 (lane l takes columns
    // 4l .. 4l+3 of every 128): a quarter of the load instructions.
    if ((m & 3) == 0) {
        constexpr int NH = (NJ + 3) / 4;   // 128-column groups per row
        for (int p = warp; p < m; p += kWarps) {
            for (int j = 4 * lane; j < m; j += 128)
                *reinterpret_cast<float4*>(acc + j) = *reinterpret_cast<const float4*>(R + (size_t)p * m + j);
            __syncwarp();
            float4 r4[NH];
#pragma unroll
            for (int h = 0; h < NH; ++h) r4[h] = make_float4(0.f, 0.f, 0.f, 0.f);
            const int a0 = S.ptr[2][p], a1 = S.ptr[2][p + 1];
            for (int tb = a0; tb < a1; tb += 32) {
                const int tc = min(32, a1 - tb);
                int kk = 0;
                float aa = 0.f;
                if (lane < tc) {
                    kk = S.idx[2][tb + lane];
                    aa = (float)S.val[2][tb + lane];
                }
#pragma unroll 2
                for (int u = 0; u < tc; ++u) {
                    const int k = __shfl_sync(kFull, kk, u);
                    const float a = __shfl_sync(kFull, aa, u);
                    const float* row = R + (size_t)k * m;
#pragma unroll
                    for (int h = 0; h < NH; ++h) {
                        const int j = 4 * lane + 128 * h;
                        if (j < m) {
                            const float4 x = *reinterpret_cast<const float4*>(row + j);
                            r4[h].x = fmaf(a, x.x, r4[h].x);
                            r4[h].y = fmaf(a, x.y, r4[h].y);
                            r4[h].z = fmaf(a, x.z, r4[h].z);
                            r4[h].w = fmaf(a, x.w, r4[h].w);
                        }
                    }
                }
            }
#pragma unroll
            for (int h = 0; h < NH; ++h) {
                const int j0 = 4 * lane + 128 * h;
                if (j0 >= m) continue;
                float v4[4] = {r4[h].x, r4[h].y, r4[h].z, r4[h].w};
#pragma unroll
                for (int cc = 0; cc < 4; ++cc) {
                    const int j = j0 + cc;
                    float v = v4[cc];
                    if (ell) {
                        const int len = elen[j];
                        for (int u = 0; u < len; ++u) v = fmaf(-acc[eidx[u * m + j]], evl[u * m + j], v);
                    } else if (staged) {
                        for (int t = bptr[j]; t < bptr[j + 1]; ++t) v = fmaf(-acc[sidx[t]], sval[t], v);
                    } else {
                        for (int t = S.ptr[3][j]; t < S.ptr[3][j + 1]; ++t)
                            v = fmaf(-acc[S.idx[3][t]], (float)S.val[3][t], v);
                    }
                    v4[cc] = two_s * v;
                }
                *reinterpret_cast<float4*>(G + (size_t)p * m + j0) = make_float4(v4[0], v4[1], v4[2], v4[3]);
            }
            __syncwarp();
        }
        __syncthreads();
        return;
    }
    for (int p = warp; p < m; p += kWarps) {
        for (int j = lane; j < m; j += 32) acc[j] = R[(size_t)p * m + j];
        __syncwarp();
        float r[NJ];
#pragma unroll
        for (int q = 0; q < NJ; ++q) r[q] = 0.f;
        const int a0 = S.ptr[2][p], a1 = S.ptr[2][p + 1];
        for (int tb = a0; tb < a1; tb += 32) {
            const int tc = min(32, a1 - tb);
            int kk = 0;
            float aa = 0.f;
            if (lane < tc) {
                kk = S.idx[2][tb + lane];
                aa = (float)S.val[2][tb + lane];
            }
#pragma unroll 2
            for (int u = 0; u < tc; ++u) {
                const int k = __shfl_sync(kFull, kk, u);
                const float a = __shfl_sync(kFull, aa, u);
                const float* row = R + (size_t)k * m;
#pragma unroll
                for (int q = 0; q < NJ; ++q) {
                    const int j = lane + 32 * q;
                    if (j < m) r[q] = fmaf(a, row[j], r[q]);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < NJ; ++q) {
            const int j = lane + 32 * q;
            if (j >= m) continue;
            float v = r[q];
            if (ell) {
                const int len = elen[j];
                for (int u = 0; u < len; ++u) v = fmaf(-acc[eidx[u * m + j]], evl[u * m + j], v);
            } else if (staged) {   // the staged lists are still in place
                for (int t = bptr[j]; t < bptr[j + 1]; ++t) v = fmaf(-acc[sidx[t]], sval[t], v);
            } else {
                for (int t = S.ptr[3][j]; t < S.ptr[3][j + 1]; ++t)
                    v = fmaf(-acc[S.idx[3][t]], (float)S.val[3][t], v);
            }
            G[(size_t)p * m + j] = two_s * v;
        }
        __syncwarp();
    }
    __syncthreads();
}

// The certificate's FP64 residual and gradient at large orders, bit-identical
// to residual() + grad_from_residual(): every element gets the same fused
// multiply-adds in the same order, minus those whose X factor is zero, which
// leave a sum started at +0 unchanged. X's nonzeros are listed by row
// (xc, xv, xn: scratch in global memory); row i of R merges A's row i with
// X's row i by column index, as the residual's two-list walk does (A's term
// first on a tie): a neighbour k scatters a * X[k][:], a nonzero X[i][l]
// scatters -X[i][l] * B[l][:], into the warp's shared-memory row. The gradient
// reads the rows of R named by column p of A and gathers row p of R (staged)
// through B's rows; B's rows are staged in `scr` beside the warps' rows
// (lists for the residual, a padded table for the gradient) when they fit.
static __device__ void grad64_rows(const Ctx& c, const double* X, double* R, double* g, unsigned char* scr,
                                   size_t scr_bytes, uint16_t* xc, double* xv, int* xn) {
    const SparseAB& S = c.sp;
    const int m = c.m, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const size_t rows_bytes = align16((size_t)kWarps * m * sizeof(double));
    double* acc = reinterpret_cast<double*>(scr) + (size_t)warp * m;
    unsigned char* lst = scr + rows_bytes;
    const size_t lst_bytes = scr_bytes > rows_bytes ? scr_bytes - rows_bytes : 0;
    const int nb = S.ptr[3][m];
    // B's rows as lists (residual)
    const size_t o_idx = align16((size_t)(m + 1) * sizeof(int));
    const size_t o_val = o_idx + align16((size_t)nb * sizeof(uint16_t));
    const bool staged = o_val + align16((size_t)nb * sizeof(double)) <= lst_bytes && m <= 65535;
    const int* bptr = staged ? reinterpret_cast<const int*>(lst) : S.ptr[3];
    const uint16_t* sidx = reinterpret_cast<const uint16_t*>(lst + o_idx);
    const double* sval = reinterpret_cast<const double*>(lst + o_val);
    if (staged) {
        int* pp = reinterpret_cast<int*>(lst);
        uint16_t* ix = reinterpret_cast<uint16_t*>(lst + o_idx);
        double* vl = reinterpret_cast<double*>(lst + o_val);
        for (int q = threadIdx.x; q <= m; q += kThreads) pp[q] = S.ptr[3][q];
        for (int t = threadIdx.x; t < nb; t += kThreads) {
            ix[t] = (uint16_t)S.idx[3][t];
            vl[t] = S.val[3][t];
        }
    }
    // X's nonzeros by row, ascending columns
    for (int i = warp; i < m; i += kWarps) {
        int cnt = 0;
        for (int j0 = 0; j0 < m; j0 += 32) {
            const int j = j0 + lane;
            const double v = j < m ? X[(size_t)i * m + j] : 0.0;
            const bool nz = j < m && v != 0.0;
            const unsigned b = __ballot_sync(kFull, nz);
            if (nz) {
                const int o = cnt + __popc(b & lt);
                xc[(size_t)i * m + o] = (uint16_t)j;
                xv[(size_t)i * m + o] = v;
            }
            cnt += __popc(b);
        }
        if (lane == 0) xn[i] = cnt;
    }
    __syncthreads();
    // R, row by row: the merged walk over A's row i and X's row i, with the
    // first 32 entries of both lists held in the lanes
    for (int i = warp; i < m; i += kWarps) {
        for (int j = lane; j < m; j += 32) acc[j] = 0.0;
        __syncwarp();
        int ia = S.ptr[0][i];
        const int ea = S.ptr[0][i + 1];
        int ib = 0;
        const int eb = xn[i];
        while (ia < ea || ib < eb) {
            // the next 32 of each list
            const int ha = ia + lane, hb = ib + lane;
            const int lka = ha < ea ? S.idx[0][ha] : m;
            const double la = ha < ea ? S.val[0][ha] : 0.0;
            const int lcn = ha < ea ? xn[lka] : 0;
            const int lkb = hb < eb ? (int)xc[(size_t)i * m + hb] : m;
            const double lx = hb < eb ? xv[(size_t)i * m + hb] : 0.0;
            int ua = 0, ub = 0;
            while ((ua < 32 && ia + ua < ea) || (ub < 32 && ib + ub < eb)) {
                const bool has_a = ua < 32 && ia + ua < ea, has_b = ub < 32 && ib + ub < eb;
                // a list whose held window ran out first ends this pass (the
                // other's next entry may precede the window's successor)
                if ((!has_a && ia + ua < ea) || (!has_b && ib + ub < eb)) break;
                const int ka = has_a ? __shfl_sync(kFull, lka, ua) : m;
                const int kb = has_b ? __shfl_sync(kFull, lkb, ub) : m;
                if (ka <= kb) {
                    const double a = __shfl_sync(kFull, la, ua);
                    const int cn = __shfl_sync(kFull, lcn, ua);
                    for (int e = lane; e < cn; e += 32) {
                        const int j = xc[(size_t)ka * m + e];
                        acc[j] = fma(a, xv[(size_t)ka * m + e], acc[j]);
                    }
                    ++ua;
                } else {
                    const double x = __shfl_sync(kFull, lx, ub);
                    const int b0 = bptr[kb], b1 = bptr[kb + 1];
                    for (int t = b0 + lane; t < b1; t += 32) {
                        const int j = staged ? (int)sidx[t] : S.idx[3][t];
                        acc[j] = fma(-x, staged ? sval[t] : S.val[3][t], acc[j]);
                    }
                    ++ub;
                }
                __syncwarp();
            }
            ia += ua;
            ib += ub;
        }
        for (int j = lane; j < m; j += 32) R[(size_t)i * m + j] = acc[j];
        __syncwarp();
    }
    __syncthreads();
    if (!all_finite(c, R)) {   // as grad_from_residual: the dense sums
        grad_from_residual(c, g);
        return;
    }
    // B's rows as a padded table (gradient)
    __shared__ int s_dmax64;
    if (threadIdx.x == 0) s_dmax64 = 0;
    __syncthreads();
    {
        int dl = 0;
        for (int q = threadIdx.x; q < m; q += kThreads) dl = max(dl, S.ptr[3][q + 1] - S.ptr[3][q]);
        if (dl) atomicMax(&s_dmax64, dl);
    }
    __syncthreads();
    const int D = s_dmax64;
    const size_t e_val = align16((size_t)D * m * sizeof(uint16_t));
    const size_t e_len = e_val + align16((size_t)D * m * sizeof(double));
    const bool ell = D > 0 && e_len + align16((size_t)m * sizeof(int)) <= lst_bytes && m <= 65535;
    uint16_t* eidx = reinterpret_cast<uint16_t*>(lst);
    double* evl = reinterpret_cast<double*>(lst + e_val);
    int* elen = reinterpret_cast<int*>(lst + e_len);
    if (ell) {
        for (int x = threadIdx.x; x < D * m; x += kThreads) {
            const int u = x / m, q = x - (x / m) * m;
            const int b0 = S.ptr[3][q], len = S.ptr[3][q + 1] - b0;
            eidx[x] = u < len ? (uint16_t)S.idx[3][b0 + u] : (uint16_t)0;
            evl[x] = u < len ? S.val[3][b0 + u] : 0.0;
        }
        for (int q = threadIdx.x; q < m; q += kThreads) elen[q] = S.ptr[3][q + 1] - S.ptr[3][q];
    }
    __syncthreads();
    const double two_s = 2.0 * c.s;
    for (int p = warp; p < m; p += kWarps) {
        for (int j = lane; j < m; j += 32) acc[j] = R[(size_t)p * m + j];
        __syncwarp();
        const int a0 = S.ptr[2][p], a1 = S.ptr[2][p + 1];
        for (int j = lane; j < m; j += 32) {
            double v = 0.0;
            for (int t = a0; t < a1; ++t) v = fma(S.val[2][t], R[(size_t)S.idx[2][t] * m + j], v);
            if (ell) {
                const int len = elen[j];
                for (int u = 0; u < len; ++u) v = fma(-acc[eidx[u * m + j]], evl[u * m + j], v);
            } else {
                for (int t = S.ptr[3][j]; t < S.ptr[3][j + 1]; ++t) v = fma(-acc[S.idx[3][t]], S.val[3][t], v);
            }
            g[(size_t)p * m + j] = two_s * v;
        }
        __syncwarp();
    }
    __syncthreads();
}

// Oracle costs and edge codes of a mixed-precision node: shared memory, or the
// node's workspace for large orders.
static __device__ inline unsigned char* mixed_costs(const Params& P, unsigned char* dsm, int node) {
    return P.L.cost_global ? P.mixed + (size_t)node * P.L.mixed_node_bytes + P.L.mx_cost_off : dsm + P.L.sm_cost;
}
static __device__ inline uint8_t* mixed_codes(const Params& P, unsigned char* dsm, int node) {
    return P.L.cost_global ? P.mixed + (size_t)node * P.L.mixed_node_bytes + P.L.mx_code_off : dsm + P.L.sm_code;
}

// Mixed-precision DICG / FW iterations (see mixed.cuh). Works on the FP64
// iterate X in place and returns the cumulative iteration count; the caller
// then computes the FP64 certificate at the returned iterate. MODE 1: FP32
// SIMT gradient; 2: tensor-core gradient; 3: large orders (costs in the
// workspace, FP32 gradient over the nonzero lists, 16 columns per lane);
// 4: large orders on a cluster of CTAs (the leader's side; cluster.cuh).
template <int MODE>
static __device__ int mixed_loop(Ctx& c, const Params& P, unsigned char* dsm, int node, double* X,
                          const double* LB, const double* UB, double* best, double& best_val,
                          double eps, int it0, bool dicg, int ls, double cutv) {
    constexpr bool TC = MODE == 2;
    constexpr bool CL = MODE == 4;
    constexpr bool BIG = MODE == 3 || CL;
    const Layout& L = P.L;
    const int n = c.n, m = c.m, tid = c.tid;
    unsigned char* mx = L.mx_global ? P.mixed + (size_t)node * L.mixed_node_bytes : dsm + L.sm_mx;
    float* xf = reinterpret_cast<float*>(mx);
    float* gf = xf + n;
    float* Rf = gf + n;
    float* Af = Rf + n;
    float* Bf = Af + n;
    float* Btf = Bf + n;
    int8_t* Ai = reinterpret_cast<int8_t*>(mx + align16(6 * (size_t)n * sizeof(float)));  // A, B as small
    int8_t* Bi = Ai + align16((size_t)n);      // integers when they are (exact integer scores, curvature)
    int* costf = reinterpret_cast<int*>(mixed_costs(P, dsm, node));   // forward oracle costs
    int* costa = costf + n;   // in-face oracle costs (negated, face only), unless derived on the fly
    uint8_t* code = mixed_codes(P, dsm, node);   // edge codes, with the iterate's face bits
    const bool derive = L.derive_inface != 0;
    // the oracles' row->column maps (and scratch inverses): the integer
    // Hungarian workspaces, or on a cluster the leader's four arrays
    IHW w0 = ihw_at(dsm + L.sm_ihw, m);
    IHW w1 = ihw_at(dsm + L.sm_ihw + L.ihw_bytes, m);
    if constexpr (CL) {
        int* lpi = reinterpret_cast<int*>(dsm + L.sm_lpi);
        w0.pi = lpi;
        w0.pinv = lpi + m;
        w1.pi = lpi + 2 * m;
        w1.pinv = lpi + 3 * m;
    }
    const double tol = c.tol;
    // tensor-core gradient: operand images in the cost matrices' shared memory,
    // the node's A / -B images after its FP32 arrays in the workspace
    constexpr bool tcg = TC;
    __shared__ uint64_t tc_bars[2];
    __shared__ uint32_t tc_slot;
    tc::Grad tg;
    if constexpr (tcg) {
        unsigned char* un = dsm + L.sm_cost;
        tg.opA = un;
        tg.opB = un + tc::kImgBytes;
        tg.op0 = un + 2 * tc::kImgBytes;
        tg.op1 = un + 3 * tc::kImgBytes;
        tg.bar_tma = &tc_bars[0];
        tg.bar_mma = &tc_bars[1];
        tg.tmem_slot = &tc_slot;
        unsigned char* img = mx + (mixed_array_bytes(n) + 255) / 256 * 256;
        tg.img = img;
        tg.ph_tma = tg.ph_mma = 0;
        tc::build_images(img, c.A, c.B, m);
        tc::fence_async_all();
        if (tid < 32) tc::tmem_alloc(&tc_slot);
        if (tid == 0) {
            tc::bar_init(&tc_bars[0], 1);
            tc::bar_init(&tc_bars[1], 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
    }
    bool int_ok = true;
    for (int e = tid; e < n; e += kThreads) {
        const int i = e / m, j = e - (e / m) * m;
        if (!tcg && !(BIG && c.use_sp)) {   // the dense FP32 gradient's copies
            Af[e] = (float)c.A[e];
            Bf[e] = (float)c.B[e];
            Btf[e] = (float)c.B[j * m + i];
        }
        const double ae = c.A[e], be = c.B[e];
        if (!(ae == rint(ae) && fabs(ae) <= 127.0 && be == rint(be) && fabs(be) <= 127.0)) int_ok = false;
        Ai[e] = (int8_t)(fabs(ae) <= 127.0 ? (int)ae : 0);
        Bi[e] = (int8_t)(fabs(be) <= 127.0 ? (int)be : 0);
        const double lo = LB[e], up = UB[e];
        uint8_t cd = 0;
        if (lo > 0.5) cd |= kForced;
        if (up >= 0.5) cd |= kAllowed;
        if (lo > up + 1e-9) cd |= kBad;
        if (!(0.0 < lo - tol) && !(0.0 > up + tol)) cd |= kZeroOk;
        if (!(1.0 < lo - tol) && !(1.0 > up + tol)) cd |= kOneOk;
        const double xe = X[e];
        xf[e] = (float)xe;
        code[e] = (uint8_t)(cd | (xe > 1e-9 ? kFaceIn : 0) | (xe >= 1.0 - 1e-9 ? kFaceOne : 0));
    }
    // Oracle warps: a warp issues on SM sub-partition (hardware slot % 4), and
    // two of these CTAs share an SM, so the CTA in the upper half of the SM's
    // warp slots runs its two oracles on warps 2 and 3 -- the four latency-bound
    // oracle warps of an SM then sit on four different sub-partitions.
    __shared__ int s_owarp;
    if (tid == 0) {
        unsigned slot;
        asm volatile("mov.u32 %0, %%warpid;" : "=r"(slot));
        s_owarp = ((slot >> 3) & 1) ? 2 : 0;
    }
    if constexpr (!CL) {   // (a cluster's oracles reset their state at launch)
        if (tid == 0) { w0.scal[0] = 0; w0.scal[1] = 0; w0.scal[2] = 0; }
        if (tid == 32) { w1.scal[0] = 0; w1.scal[1] = 0; w1.scal[2] = 0; }
        // warm state of every column: the in-face oracle's free columns change with
        // the face, so a column may be read before any call has written it
        for (int j = tid; j < m; j += kThreads) {
            w0.colpot[j] = 0;
            w1.colpot[j] = 0;
            w0.match[j] = -1;
            w1.match[j] = -1;
        }
    }
    if (tid == 0) c.flag[4] = 0;  // set when a face-forced bit of x changes
    if (tid == 0) c.flag[5] = 0;  // set when a tensor-core wait timed out
    // small-integer A and B (graph adjacency): permutation residuals are
    // integers, so scores and curvatures are exact integer sums (the FP64 sums
    // of the same integers are exact too, hence bit-identical)
    const bool ints = __syncthreads_and(int_ok) != 0;
    // Large orders with sparse small-integer graphs score permutations and
    // pairwise directions in O(nnz): ||AP - PB||^2 = ||A||^2 + ||B||^2 -
    // 2 sum_i sum_{k in row i of A} A[i][k] B[pi[i]][pi[k]], exact integers, so
    // the sums equal the O(m^2) ones; a permutation's bounds are checked per row
    // against the one column (if any) that must not be 0 (zreq: -1 none, -2
    // more than one, found once: the kZeroOk bits do not change in the loop).
    const bool sparse_ints = BIG && ints && c.use_sp;
    int* zreq = reinterpret_cast<int*>(Btf) + m;   // after the gradient's row counts
    double norms = 0.0;                            // ||A||^2 + ||B||^2
    if (sparse_ints) {
        const int lane = tid & 31, warp = tid >> 5;
        for (int r = warp; r < m; r += kWarps) {
            int cnt = 0, col = -1;
            for (int j0 = 0; j0 < m; j0 += 32) {
                const int j = j0 + lane;
                const unsigned b = __ballot_sync(kFull, j < m && !(code[r * m + j] & kZeroOk));
                if (b && col < 0) col = j0 + __ffs(b) - 1;
                cnt += __popc(b);
            }
            if (lane == 0) zreq[r] = cnt == 0 ? -1 : (cnt == 1 ? col : -2);
        }
        double loc = 0.0;
        for (int t = tid; t < c.sp.ptr[0][m]; t += kThreads) loc += c.sp.val[0][t] * c.sp.val[0][t];
        for (int t = tid; t < c.sp.ptr[3][m]; t += kThreads) loc += c.sp.val[3][t] * c.sp.val[3][t];
        norms = bsum(loc, c.red);   // (a barrier: zreq is visible after it)
    }
    auto a_int = [&](int t) -> long long { return (long long)c.sp.val[0][t]; };

    auto score = [&](const int* pi, int* pinv) -> double {
        if (!ints) return perm_score(c, code, pi, pinv);
        if (sparse_ints) {
            bool valid = true;
            for (int r = tid; r < m; r += kThreads) {
                pinv[pi[r]] = r;
                const int z = zreq[r];
                if (!(code[r * m + pi[r]] & kOneOk) || z == -2 || (z >= 0 && z != pi[r])) valid = false;
            }
            if (!__syncthreads_and(valid)) return kNone;
            long long cross = 0;
            for (int i = tid; i < m; i += kThreads) {
                const int pr = pi[i] * m;
                for (int t = c.sp.ptr[0][i]; t < c.sp.ptr[0][i + 1]; ++t)
                    cross += a_int(t) * (long long)Bi[pr + pi[c.sp.idx[0][t]]];
            }
            return c.s * bsum((double)(-2 * cross) + (tid == 0 ? norms : 0.0), c.red);
        }
        bool valid = true;
        for (int r = tid; r < m; r += kThreads) pinv[pi[r]] = r;
        for (int e = tid; e < n; e += kThreads) {
            const int i = e / m, j = e - (e / m) * m;
            if (!(code[e] & (pi[i] == j ? kOneOk : kZeroOk))) valid = false;
        }
        if (!__syncthreads_and(valid)) return kNone;
        int acc = 0;
        for (int e = tid; e < n; e += kThreads) {
            const int i = e / m, j = e - (e / m) * m;
            const int r = (int)Ai[i * m + pinv[j]] - (int)Bi[pi[i] * m + j];
            acc += r * r;
        }
        return c.s * bsum((double)acc, c.red);
    };

    // Large orders keep the best vertex as its permutation (m ints after zreq)
    // and write the n-vector once, after the loop: the last permutation taken
    // is the one the per-vertex writes would have left.
    int* best_pi = zreq + m;
    bool best_lazy = false;
    auto take = [&](const int* pi, double fv) {
        if (fv < best_val) {
            best_val = fv;
            if (tid == 0) P.b.best_vertex_val[node] = fv;
        }
        if (fv < 1e299 && fv == best_val) {
            if (sparse_ints) {
                for (int r = tid; r < m; r += kThreads) best_pi[r] = pi[r];
                best_lazy = true;
            } else {
                for (int e = tid; e < n; e += kThreads) best[e] = pi[e / m] == e - (e / m) * m ? 1.0 : 0.0;
            }
        }
        __syncthreads();
    };

    const float two_s = (float)(2.0 * c.s);
    const float limit = 16777216.0f / (float)m;  // integer costs stay below 2^24 / m
    int iters = it0;
    for (int iter = 0; iter < P.b.max_iters; ++iter) {
        iters = it0 + iter + 1;
        if constexpr (tcg) {
            if (!tc::gradient(tg, m, xf, two_s, gf, (dicg && !(cutv < kInfD)) ? nullptr : Rf)) {
                iters = it0 + iter;  // the iteration did not happen
                if (tid == 0) c.flag[5] = 1;
                __syncthreads();
                break;
            }
        } else if (c.use_sp && BIG) {
            // large orders: row by row, the factor's rows and B's lists staged in
            // shared memory that is free during the gradient (the FP64 Hungarian
            // workspace and the integer oracles' column state; on a cluster, the
            // leader's cost slice, staged again after the gradient)
            unsigned char* base = CL ? dsm + L.sm_slice : dsm + L.sm_hung;
            const size_t rows_bytes = align16((size_t)kWarps * m * sizeof(float));
            unsigned char* lst = CL ? base + rows_bytes : dsm + L.sm_cs;
            const size_t avail = CL ? (size_t)L.cl_cols * m * sizeof(int) : 2 * L.cs_bytes;
            const size_t lst_bytes = CL ? (avail > rows_bytes ? avail - rows_bytes : 0) : avail;
            // X's nonzero lists in the dense FP32 copies of A and B, which only
            // the dense gradient reads
            uint16_t* xc = reinterpret_cast<uint16_t*>(Af);
            float* xv = Bf;
            int* xn = reinterpret_cast<int*>(Btf);
            float* rb = reinterpret_cast<float*>(base);
            if (m <= 256) grad_f32_rows<8>(c.sp, m, two_s, xf, Rf, gf, rb, lst, lst_bytes, xc, xv, xn);
            else grad_f32_rows<16>(c.sp, m, two_s, xf, Rf, gf, rb, lst, lst_bytes, xc, xv, xn);
        } else if (c.use_sp && m > 64) {
            // sparse graphs above order 64: products over the nonzero lists
            grad_f32_sparse(c.sp, m, two_s, xf, Rf, gf);
        } else {
            grad_f32(m, two_s, Af, Bf, Btf, xf, Rf, gf);
        }
        const float gmx = bmax_abs(gf, n, c.red);
        int shift = 0;
        if (gmx > 0.f) {
            int ex = 0;
            frexpf(limit / gmx, &ex);
            shift = max(-120, min(120, ex - 1));
        }
        if constexpr (CL) {
            // post the command, stage this CTA's slice, run the oracle warps
            // with the helpers (each CTA scales its own slice of the costs)
            ClCtl* ctl = reinterpret_cast<ClCtl*>(dsm + L.sm_cl);
            if (tid == 0) {
                ctl->cmd[0] = CL_ORACLE;
                ctl->cmd[1] = shift;
                ctl->cmd[2] = c.flag[4] == 0 ? 1 : 0;
                ctl->cmd[3] = dicg ? 1 : 0;
            }
            __threadfence();
            __syncthreads();
            if (tid == 0) {
                cl_fence();
                for (int r = 1; r < kClCtas; ++r) cl_arrive(cl_map(&ctl->bar_go, (unsigned)r));
            }
            int* slice = reinterpret_cast<int*>(dsm + L.sm_slice);
            cl_stage(slice, L.cl_cols, 0, m, gf, code, shift);
            __syncthreads();
            const int wid = tid >> 5;
            if (wid == 0 || (dicg && wid == 1)) {
                const bool ok = wid == 0
                    ? cl_hungarian<0>(chw_at(dsm + L.sm_chw, m), slice, L.cl_cols, m, shift, code, true, w0.pi,
                                      &ctl->err)
                    : cl_hungarian<2>(chw_at(dsm + L.sm_chw + L.chw_bytes, m), slice, L.cl_cols, m, shift, code,
                                      c.flag[4] == 0, w1.pi, &ctl->err);
                if ((tid & 31) == 0) c.flag[wid == 0 ? 0 : 2] = ok;
            }
        } else {
        if (BIG && (n & 3) == 0) {
            // four costs per thread and access (orders divisible by 2)
            for (int e4 = tid; e4 < n / 4; e4 += kThreads) {
                const float4 g4 = reinterpret_cast<const float4*>(gf)[e4];
                const uchar4 c4 = reinterpret_cast<const uchar4*>(code)[e4];
                int4 o;
                o.x = pack_cost(__float2int_rn(scalbnf(g4.x, shift)), c4.x & kAllowed, c4.x & kFaceIn);
                o.y = pack_cost(__float2int_rn(scalbnf(g4.y, shift)), c4.y & kAllowed, c4.y & kFaceIn);
                o.z = pack_cost(__float2int_rn(scalbnf(g4.z, shift)), c4.z & kAllowed, c4.z & kFaceIn);
                o.w = pack_cost(__float2int_rn(scalbnf(g4.w, shift)), c4.w & kAllowed, c4.w & kFaceIn);
                reinterpret_cast<int4*>(costf)[e4] = o;
            }
        } else
        for (int e = tid; e < n; e += kThreads) {
            const int ci = __float2int_rn(scalbnf(gf[e], shift));
            const uint8_t cd = code[e];
            const bool allowed = (cd & kAllowed) != 0;
            if constexpr (BIG) {
                // one packed array read by both oracles (half the bytes the
                // Dijkstra steps stream from L2)
                costf[e] = pack_cost(ci, allowed, (cd & kFaceIn) != 0);
            } else {
                costf[e] = allowed ? ci : kIntInf;
                if (dicg && !derive) costa[e] = (allowed && (cd & kFaceIn)) ? -ci : kIntInf;
            }
        }
        __syncthreads();
        const int owarp = (int)(threadIdx.x >> 5) - s_owarp;
        bool group_done = false;
        if constexpr (BIG) {
            if (L.oracle_group) {   // forward oracle on warps 0-3, in-face on warps 4-7
                group_done = true;
                const int g = tid >> 7;
                if (g == 0 || dicg) {
                    int* cs = reinterpret_cast<int*>(dsm + L.sm_cs + (g == 0 ? 0 : L.cs_bytes));
                    bool ok;
                    if (m <= 256)
                        ok = g == 0 ? int_hungarian_group_cs<2, 3>(w0, cs, m, costf, shift, code, true, 0)
                                    : int_hungarian_group_cs<2, 4>(w1, cs, m, costf, shift, code, c.flag[4] == 0, 1);
                    else
                        ok = g == 0 ? int_hungarian_group_cs<4, 3>(w0, cs, m, costf, shift, code, true, 0)
                                    : int_hungarian_group_cs<4, 4>(w1, cs, m, costf, shift, code, c.flag[4] == 0, 1);
                    if ((tid & 127) == 0) c.flag[g == 0 ? 0 : 2] = ok;
                }
            }
        }
        if (!group_done && (owarp == 0 || (dicg && owarp == 1))) {
            const bool fwd = owarp == 0;
            const IHW& w = fwd ? w0 : w1;
            const bool same = fwd || c.flag[4] == 0;
            bool ok;
            if constexpr (BIG) {   // column state in shared memory: two nodes per SM
                int* cs = reinterpret_cast<int*>(dsm + L.sm_cs + (fwd ? 0 : L.cs_bytes));
                if (m <= 256) ok = fwd ? int_hungarian_warp_cs<8, 3>(w, cs, m, costf, shift, code, same)
                                       : int_hungarian_warp_cs<8, 4>(w, cs, m, costf, shift, code, same);
                else ok = fwd ? int_hungarian_warp_cs<16, 3>(w, cs, m, costf, shift, code, same)
                              : int_hungarian_warp_cs<16, 4>(w, cs, m, costf, shift, code, same);
            } else if constexpr (TC) {   // orders 17..128, costs beside the operand images
                if (m <= 64) ok = fwd ? int_hungarian_warp<2, 0>(w, m, costf, shift, code, same)
                                      : int_hungarian_warp<2, 1>(w, m, costa, shift, code, same);
                else ok = fwd ? int_hungarian_warp<4, 0>(w, m, costf, shift, code, same)
                              : int_hungarian_warp<4, 1>(w, m, costa, shift, code, same);
            } else {   // orders up to 128; in-face costs derived where that fits two nodes per SM
                if (m <= 64) ok = fwd ? int_hungarian_warp<2, 0>(w, m, costf, shift, code, same)
                                      : int_hungarian_warp<2, 1>(w, m, costa, shift, code, same);
                else if (fwd) ok = int_hungarian_warp<4, 0>(w, m, costf, shift, code, same);
                else ok = derive ? int_hungarian_warp<4, 2>(w, m, costf, shift, code, same)
                                 : int_hungarian_warp<4, 1>(w, m, costa, shift, code, same);
            }
            if ((threadIdx.x & 31) == 0) c.flag[fwd ? 0 : 2] = ok;
        }
        }   // one CTA's oracles
        __syncthreads();
        if (tid == 0) c.flag[4] = 0;
        if (!c.flag[0] || (dicg && !c.flag[2])) break;
        take(w0.pi, score(w0.pi, w0.pinv));
        double loc = 0.0;
        for (int e = tid; e < n; e += kThreads) {
            const double ve = w0.pi[e / m] == e - (e / m) * m ? 1.0 : 0.0;
            loc = fma((double)gf[e], X[e] - ve, loc);
        }
        const double gap = bsum(loc, c.red);
        if (gap >= 0.0 && gap < eps) break;
        if (cutv < kInfD && iter > 0) {
            // the FP32 residual's bound clears the incumbent by a margin that
            // covers its rounding; the certificate is recomputed exactly
            double l2 = 0.0;
            for (int e = tid; e < n; e += kThreads) l2 = fma((double)Rf[e], (double)Rf[e], l2);
            const double fv = c.s * bsum(l2, c.red);
            if (fv - gap >= cutv + 1e-5 * (1.0 + fabs(cutv))) break;
        }

        if (!dicg) {
            double gm;
            if (ls == GBX_LS_QUADRATIC_EXACT) {
                for (int r = tid; r < m; r += kThreads) w0.pinv[w0.pi[r]] = r;
                __syncthreads();
                double cl = 0.0;
                for (int e = tid; e < n; e += kThreads) {
                    const int i = e / m, j = e - (e / m) * m;
                    const double rv = c.A[i * m + w0.pinv[j]] - c.B[w0.pi[i] * m + j];
                    const double d = rv - (double)Rf[e];
                    cl = fma(d, d, cl);
                }
                const double curv = (2.0 * c.s) * bsum(cl, c.red);
                if (curv > 0.0) gm = gap <= 0.0 ? 0.0 : fmin(gap / curv, 1.0);
                else gm = -gap + 0.5 * curv * 1.0 < 0.0 ? 1.0 : 0.0;
            } else {
                gm = 2.0 / (double)(it0 + iter + 2);
            }
            for (int e = tid; e < n; e += kThreads) {
                const double ve = w0.pi[e / m] == e - (e / m) * m ? 1.0 : 0.0;
                X[e] = fma(gm, ve - X[e], X[e]);
                xf[e] = (float)X[e];
            }
            __syncthreads();
            continue;
        }
        take(w1.pi, score(w1.pi, w1.pinv));
        for (int r = tid; r < m; r += kThreads) {
            w0.pinv[w0.pi[r]] = r;
            w1.pinv[w1.pi[r]] = r;
        }
        __syncthreads();
        double res = 1.0;
        for (int i = tid; i < m; i += kThreads) {
            const int pa = w1.pi[i], pv = w0.pi[i];
            if (pa == pv) continue;
            const int ea = i * m + pa, ev = i * m + pv;
            res = fmin(res, (X[ea] - LB[ea]) / 1.0);
            res = fmin(res, (UB[ev] - X[ev]) / 1.0);
        }
        const double gmax = fmax(0.0, fmin(bmin(res, c.red), 1.0));
        double gm;
        if (ls == GBX_LS_QUADRATIC_EXACT) {
            double pl = 0.0, cl = 0.0;
            for (int i = tid; i < m; i += kThreads) {
                const int pa = w1.pi[i], pv = w0.pi[i];
                if (pa != pv) pl += (double)gf[i * m + pa] - (double)gf[i * m + pv];
            }
            if (sparse_ints) {
                // ||A D - D B||^2 for D = P1 - P0 (P1 the in-face vertex): the
                // squares of the O(m^2) sum expanded into 2||A||^2 + 2||B||^2
                // and O(nnz) cross sums, exact integers
                const int* p1 = w1.pi;
                const int* p0 = w0.pi;
                const int* p0inv = w0.pinv;
                long long cross = 0;
                for (int i = tid; i < m; i += kThreads) {
                    const int r1 = p1[i] * m, r0 = p0[i] * m;
                    for (int t = c.sp.ptr[0][i]; t < c.sp.ptr[0][i + 1]; ++t) {
                        const int k = c.sp.idx[0][t];
                        const long long a = a_int(t);
                        const long long a1a0 = (long long)Ai[i * m + p0inv[p1[k]]];
                        const long long b11 = Bi[r1 + p1[k]], b01 = Bi[r0 + p1[k]];
                        const long long b10 = Bi[r1 + p0[k]], b00 = Bi[r0 + p0[k]];
                        cross += a * (-a1a0 - b11 + b01 + b10 - b00);
                    }
                    for (int t = c.sp.ptr[3][p1[i]]; t < c.sp.ptr[3][p1[i] + 1]; ++t)
                        cross -= (long long)c.sp.val[3][t] * (long long)Bi[r0 + c.sp.idx[3][t]];
                }
                cl = (double)(2 * cross) + (tid == 0 ? 2.0 * norms : 0.0);
            } else if (ints) {
                int acc = 0;
                for (int e = tid; e < n; e += kThreads) {
                    const int i = e / m, j = e - (e / m) * m;
                    const int rd = ((int)Ai[i * m + w1.pinv[j]] - (int)Ai[i * m + w0.pinv[j]])
                                 - ((int)Bi[w1.pi[i] * m + j] - (int)Bi[w0.pi[i] * m + j]);
                    acc += rd * rd;
                }
                cl = (double)acc;
            } else {
                for (int e = tid; e < n; e += kThreads) {
                    const int i = e / m, j = e - (e / m) * m;
                    const double rd = (c.A[i * m + w1.pinv[j]] - c.A[i * m + w0.pinv[j]])
                                    - (c.B[w1.pi[i] * m + j] - c.B[w0.pi[i] * m + j]);
                    cl = fma(rd, rd, cl);
                }
            }
            const double pgap = bsum(pl, c.red);
            const double curv = (2.0 * c.s) * bsum(cl, c.red);
            if (gmax <= 0.0) gm = 0.0;
            else if (curv > 0.0) gm = pgap <= 0.0 ? 0.0 : fmin(pgap / curv, gmax);
            else gm = -pgap + 0.5 * curv * gmax < 0.0 ? gmax : 0.0;
        } else {
            const double open = 2.0 / (double)(it0 + iter + 2);
            if (ls == GBX_LS_SAFEGUARDED_SCALED_OPEN_LOOP) gm = gmax <= open ? gmax : gmax * open;
            else if (ls == GBX_LS_SCALED_OPEN_LOOP) gm = gmax * open;
            else gm = fmin(gmax, open);
        }
        for (int i = tid; i < m; i += kThreads) {
            const int pa = w1.pi[i], pv = w0.pi[i];
            if (pa == pv) continue;
            const int ea = i * m + pa, ev = i * m + pv;
            X[ea] = fma(-gm, 1.0, X[ea]);
            X[ev] = fma(-gm, -1.0, X[ev]);
            xf[ea] = (float)X[ea];
            xf[ev] = (float)X[ev];
            const uint8_t fa = (uint8_t)((X[ea] > 1e-9 ? kFaceIn : 0) | (X[ea] >= 1.0 - 1e-9 ? kFaceOne : 0));
            const uint8_t fv = (uint8_t)((X[ev] > 1e-9 ? kFaceIn : 0) | (X[ev] >= 1.0 - 1e-9 ? kFaceOne : 0));
            if (((fa ^ code[ea]) | (fv ^ code[ev])) & kFaceOne) c.flag[4] = 1;
            code[ea] = (uint8_t)((code[ea] & ~kFaceBits) | fa);
            code[ev] = (uint8_t)((code[ev] & ~kFaceBits) | fv);
        }
        __syncthreads();
    }
    if (best_lazy)
        for (int e = tid; e < n; e += kThreads) best[e] = best_pi[e / m] == e - (e / m) * m ? 1.0 : 0.0;
    __syncthreads();
    if constexpr (CL) cl_release(reinterpret_cast<ClCtl*>(dsm + L.sm_cl));   // the helpers leave
    if constexpr (tcg) {
        // a gradient that timed out may still have MMAs in flight: wait (bounded)
        // for them before the accumulator columns are released
        if (c.flag[5] && tid == 0) tc::bar_wait(tg.bar_mma, tg.ph_mma);
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
        if (tid < 32) tc::tmem_dealloc(tc_slot);
    }
    return iters;
}

// ------------------------------------------------------------------ kernel
struct Scalars {
    double red[40];
    int flag[8];
};

__device__ inline double* vecp(double* sbase, double* gbase, const Layout& L, int b) {
    if (L.off[b] < 0) return nullptr;
    return (L.in_smem[b] ? sbase : gbase) + L.off[b];
}

// MIX: 0 FP64 iterations, 1 mixed precision with the FP32 SIMT gradient (two
// nodes per SM), 2 mixed precision with the tensor-core gradient
template <int OK, int LK, int MIX>
static __device__ __forceinline__ void relax_node(const Params& P, const int node, unsigned char* dsm, Scalars& sh) {
    const int tid = threadIdx.x;
    const int n = P.obj.n;
    const Layout& L = P.L;

    double* sb = reinterpret_cast<double*>(dsm + L.sm_vec);
    double* gb = P.ws + (size_t)node * L.node_stride;
    double* X = vecp(sb, gb, L, B_X);
    double* G = vecp(sb, gb, L, B_G);
    double* V = vecp(sb, gb, L, B_V);
    double* AW = vecp(sb, gb, L, B_AW);
    double* TX = vecp(sb, gb, L, B_TX);
    double* TG = vecp(sb, gb, L, B_TG);
    double* LB = vecp(sb, gb, L, B_LB);
    double* UB = vecp(sb, gb, L, B_UB);
    double* CAND = vecp(sb, gb, L, B_CAND);

    const size_t off = (size_t)node * n;
    double* gx = P.b.x + off;
    double* best = P.b.best_vertex + off;

    Ctx c;
    c.n = n;
    c.tid = tid;
    c.red = sh.red;
    c.flag = sh.flag;
    c.ok = OK;
    c.m = P.obj.order;
    c.c = P.obj.c;
    c.s = P.obj.scale;
    c.ls = P.obj.linear_scale;
    c.k0 = P.obj.constant;
    c.R = vecp(sb, gb, L, B_R);
    c.use_sp = false;
    if (OK == GBX_OBJ_GRAPH_MATCHING && P.sparse) {
        c.sp = sparse_at(P.sparse, P.obj.order, L.sparse_cap);
        c.use_sp = c.sp.ok[0] && c.sp.ok[1] && c.sp.ok[2] && c.sp.ok[3];
    }
    c.lk = LK;
    c.rhs = P.lmo.right_side;
    c.is_int = P.lmo.is_int;
    c.lorder = P.lmo.order;
    c.U = P.lmo.upper;
    c.S = L.sort_size;
    c.keys = reinterpret_cast<double*>(dsm + L.sm_keys);
    c.prefix = reinterpret_cast<double*>(dsm + L.sm_prefix);
    c.idx = reinterpret_cast<int*>(dsm + L.sm_idx);
    c.fixed = dsm + L.sm_fixed;
    c.hung[0] = dsm + L.sm_hung;
    c.hung[1] = dsm + L.sm_hung + L.hung_bytes;
    c.hung_bytes = L.hung_bytes;
    c.flags = P.b.integer_flags;
    c.tol = P.b.candidate_tol;
    c.pr = -1;
    c.xch = nullptr;
    if (L.pair) {   // a two-CTA cluster per node: this CTA's rank, the exchange buffer
        unsigned rk;
        asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(rk));
        c.pr = (int)rk;
        c.xch = reinterpret_cast<double*>(dsm + L.sm_xch);
    }
    // in a pair, rank 0 alone writes the node's results (rank 1 computes the same)
    const bool writer = c.pr <= 0;

    // stage node data and objective matrices
    for (int j = tid; j < n; j += kThreads) {
        X[j] = gx[j];
        LB[j] = P.b.lb[off + j];
        UB[j] = P.b.ub[off + j];
    }
    if (OK == GBX_OBJ_GRAPH_MATCHING) {
        if (L.obj_smem) {
            double* As = reinterpret_cast<double*>(dsm + L.sm_obj);
            double* Bs = As + (size_t)c.m * c.m;
            for (int e = tid; e < c.m * c.m; e += kThreads) { As[e] = P.obj.A[e]; Bs[e] = P.obj.B[e]; }
            c.A = As;
            c.B = Bs;
        } else {
            c.A = P.obj.A;
            c.B = P.obj.B;
        }
        c.Q = nullptr;
    } else {
        if (L.obj_smem) {
            double* Qs = reinterpret_cast<double*>(dsm + L.sm_obj);
            for (size_t e = tid; e < (size_t)n * n; e += kThreads) Qs[e] = P.obj.Q[e];
            c.Q = Qs;
        } else {
            c.Q = P.obj.Q;
        }
        c.A = c.B = nullptr;
    }
    const double eps = P.b.eps[node];
    const double cutv = P.b.cutoff ? *P.b.cutoff : kInfD;   // incumbent cutoff (+inf: none)
    const int it0 = P.b.iterations[node];
    const bool supplied = (P.b.status[node] & GBX_NODE_INITIAL_POINT_SUPPLIED) != 0;
    __syncthreads();
    if (tid == 0 && writer) P.b.best_vertex_val[node] = kNone;
    double best_val = kNone;

    if (!node_feasible<LK>(c, LB, UB, V)) {
        if (tid == 0 && writer) {
            P.b.status[node] = GBX_NODE_INFEASIBLE;
            P.b.value[node] = CUDART_INF;
            P.b.gap[node] = 0.0;
            P.b.iterations[node] = it0;
        }
        return;
    }

    const bool dicg = P.alg.kind == GBX_ALG_DICG;
    const int ls = P.alg.line_search;
    const bool search = ls == GBX_LS_SECANT || ls == GBX_LS_QUADRATIC_EXACT;
    const HW hw0 = hw_at(c.hung[0], LK == GBX_LMO_BIRKHOFF ? c.lorder : 0);
    const HW hw1 = hw_at(c.hung[1], LK == GBX_LMO_BIRKHOFF ? c.lorder : 0);
    const bool graph_perm = OK == GBX_OBJ_GRAPH_MATCHING && LK == GBX_LMO_BIRKHOFF;

    if (it0 == 0 && !supplied) {
        // the reference starts at the vertex of the direction -1 - j/(n+1); the
        // mixed-precision iterations start at the feasibility test's matching
        // (any vertex is a valid start, and this one costs no oracle call)
        if constexpr (MIX == 0) {
            for (int j = tid; j < n; j += kThreads) G[j] = -1.0 - static_cast<double>(j) / (n + 1.0);
            __syncthreads();
            lmo_forward<LK>(c, G, LB, UB, V);
        }
        for (int j = tid; j < n; j += kThreads) X[j] = V[j];
        __syncthreads();
    }

    // score an integral vertex (drs_integer_value + best-vertex bookkeeping)
    auto score = [&](const double* vert, const int* pi, int* pinv) {
        const double fv = integer_value(c, vert, LB, UB, pi, pinv);
        if (fv < best_val) {
            best_val = fv;
            if (tid == 0 && writer) P.b.best_vertex_val[node] = fv;
        }
        if (fv < 1e299 && fv == best_val && writer)
            for (int j = tid; j < n; j += kThreads) best[j] = vert[j];
        __syncthreads();
    };

    // line searches (SecantLS::search, QuadraticExactLS::search)
    auto line_search = [&](double gap, double maxg, const double* dir) -> double {
        if (ls == GBX_LS_QUADRATIC_EXACT) {
            const double curv = obj_curvature(c, dir);
            if (maxg <= 0.0) return 0.0;
            if (curv > 0.0) {
                if (gap <= 0.0) return 0.0;
                const double st = gap / curv;
                return st < maxg ? st : maxg;
            }
            return -gap + 0.5 * curv * maxg < 0.0 ? maxg : 0.0;
        }
        const double tol = P.alg.secant_tol, deps = P.alg.secant_denom_eps;
        const double f_base = obj_value(c, X);
        double lo = 0.0, hi = maxg, best_f = f_base, best_gamma = 0.0;
        double phi_lo = -gap, phi_hi = 0.0, gamma = 0.0;
        bool done = phi_lo >= -tol;
        const double f_abs = f_base >= 0.0 ? f_base : -f_base;
        const double allow = tol * (1.0 + f_abs);
        auto probe = [&](double gm, double& phi, double& f) {
            for (int j = tid; j < n; j += kThreads) TX[j] = fma(gm, dir[j], X[j]);
            __syncthreads();
            obj_grad(c, TX, TG);
            double loc = 0.0;
            for (int j = tid; j < n; j += kThreads) loc = fma(TG[j], dir[j], loc);
            phi = bsum(loc, c.red);
            f = OK == GBX_OBJ_GRAPH_MATCHING ? value_from_residual(c) : obj_value(c, TX);
        };
        double f_hi;
        probe(maxg, phi_hi, f_hi);
        if (f_hi < best_f || (best_gamma == 0.0 && f_hi <= f_base + allow)) { best_f = f_hi; best_gamma = maxg; }
        if (!done && phi_hi <= tol && f_hi <= f_base + allow) { gamma = maxg; done = true; }
        for (int it = 0; it < P.alg.secant_iters; ++it) {
            if (done) break;
            const double denom = phi_hi - phi_lo;
            double gm = (denom > deps || denom < -deps) ? hi - phi_hi * (hi - lo) / denom : 0.5 * (lo + hi);
            if (!(gm > lo && gm < hi)) gm = 0.5 * (lo + hi);
            gamma = gm;
            double phi, ft;
            probe(gamma, phi, ft);
            if (ft < best_f || (best_gamma == 0.0 && ft <= f_base + allow)) { best_f = ft; best_gamma = gamma; }
            if (phi < 0.0) { lo = gamma; phi_lo = phi; }
            else { hi = gamma; phi_hi = phi; }
            if ((phi <= tol && phi >= -tol) || (hi - lo) <= tol) { gamma = 0.5 * (lo + hi); done = true; }
        }
        if (best_gamma > 0.0 && best_f <= f_base + allow) gamma = best_gamma;
        else if (!done) gamma = 0.0;
        return gamma;
    };

    int iters = it0;
    constexpr bool kMixedLoop = MIX != 0 && OK == GBX_OBJ_GRAPH_MATCHING && LK == GBX_LMO_BIRKHOFF;
    if constexpr (kMixedLoop)
        iters = mixed_loop<MIX>(c, P, dsm, node, X, LB, UB, best, best_val, eps, it0, dicg, ls, cutv);
    for (int iter = 0; !kMixedLoop && iter < P.b.max_iters; ++iter) {
        iters = it0 + iter + 1;
        obj_grad(c, X, G);
        // f(x) for the incumbent cutoff, before vertex scoring reuses the residual
        const double fcut = (cutv < kInfD && iter > 0) ? value_at_grad(c, X, G) : 0.0;
        bool fwd_perm = false, away_perm = false;
        if constexpr (LK == GBX_LMO_BIRKHOFF) {
            // forward oracle on warps 0-3, DICG away oracle on warps 4-7
            for (int j = tid; j < n; j += kThreads) { V[j] = 0.0; if (dicg) AW[j] = 0.0; }
            __syncthreads();
            if (n == c.lorder * c.lorder) {
                if (!dicg) {   // Frank-Wolfe: the forward oracle alone, on all eight warps
                    const bool ok = hungarian_group<8>(hw0, c.lorder, G, 1.0, LB, UB, nullptr, V, nullptr, 0);
                    if (threadIdx.x == 0) sh.flag[0] = ok;
                } else if (threadIdx.x < kHungThreads) {
                    const bool ok = hungarian_group(hw0, c.lorder, G, 1.0, LB, UB, nullptr, V, nullptr, 0);
                    if (threadIdx.x == 0) sh.flag[0] = ok;
                } else {
                    const bool ok = hungarian_group(hw1, c.lorder, G, -1.0, LB, UB, X, AW, nullptr, 1);
                    if (threadIdx.x == kHungThreads) sh.flag[2] = ok;
                }
            } else if (tid == 0) {
                sh.flag[0] = 0;
                sh.flag[2] = 0;
            }
            __syncthreads();
            fwd_perm = graph_perm && sh.flag[0];
            away_perm = graph_perm && dicg && sh.flag[2];
        } else {
            lmo_forward<LK>(c, G, LB, UB, V);
        }
        score(V, fwd_perm ? hw0.pi : nullptr, hw0.pinv);
        double loc = 0.0;
        for (int j = tid; j < n; j += kThreads) loc = fma(G[j], X[j] - V[j], loc);
        const double gap = bsum(loc, c.red);
        if (gap >= 0.0 && gap < eps) break;
        if (cutv < kInfD && iter > 0 && fcut - gap >= cutv) break;

        if (!dicg) {
            if (search) {
                for (int j = tid; j < n; j += kThreads) V[j] -= X[j];
                __syncthreads();
                const double gm = line_search(gap, 1.0, V);
                for (int j = tid; j < n; j += kThreads) X[j] = fma(gm, V[j], X[j]);
            } else {
                const double gm = 2.0 / (double)(it0 + iter + 2);
                for (int j = tid; j < n; j += kThreads) X[j] = fma(gm, V[j] - X[j], X[j]);
            }
            __syncthreads();
            continue;
        }
        if constexpr (LK != GBX_LMO_BIRKHOFF) lmo_inface<LK>(c, G, -1.0, X, LB, UB, AW, 1);
        score(AW, away_perm ? hw1.pi : nullptr, hw1.pinv);
        for (int j = tid; j < n; j += kThreads) AW[j] -= V[j];
        __syncthreads();
        const double gmax = lmo_max_step<LK>(c, AW, X, LB, UB);
        if (search) {
            for (int j = tid; j < n; j += kThreads) AW[j] = -AW[j];
            __syncthreads();
            double pl = 0.0;
            for (int j = tid; j < n; j += kThreads) pl = fma(-G[j], AW[j], pl);
            const double pgap = bsum(pl, c.red);
            const double gm = line_search(pgap, gmax, AW);
            for (int j = tid; j < n; j += kThreads) X[j] = fma(gm, AW[j], X[j]);
        } else {
            const double open = 2.0 / (double)(it0 + iter + 2);
            double gm;
            if (ls == GBX_LS_SAFEGUARDED_SCALED_OPEN_LOOP) gm = gmax <= open ? gmax : gmax * open;
            else if (ls == GBX_LS_SCALED_OPEN_LOOP) gm = gmax * open;
            else gm = fmin(gmax, open);
            for (int j = tid; j < n; j += kThreads) X[j] = fma(-gm, AW[j], X[j]);
        }
        __syncthreads();
    }

    // certificate at the returned iterate (the graph-matching value comes from
    // the residual the gradient leaves behind: the same sums as obj_value)
    bool rows64 = false;
    if constexpr (kMixedLoop && MIX == 3) {
        // large orders: row by row, with the node's FP32 arrays (free now) as
        // scratch for X's nonzero lists and the shared memory of the integer
        // oracles and the FP64 Hungarian (not yet in use) for rows and B
        if (c.use_sp && all_finite(c, X)) {
            unsigned char* mxb = P.mixed + (size_t)node * L.mixed_node_bytes;
            grad64_rows(c, X, c.R, G, dsm + L.sm_hung, L.sm_total - L.sm_hung,
                        reinterpret_cast<uint16_t*>(mxb + 2 * (size_t)n * sizeof(float)),
                        reinterpret_cast<double*>(mxb),
                        reinterpret_cast<int*>(mxb + 3 * (size_t)n * sizeof(float)));
            rows64 = true;
        }
    }
    if (!rows64) obj_grad(c, X, G);
    double fval = 0.0;
    if constexpr (OK == GBX_OBJ_GRAPH_MATCHING) fval = value_from_residual(c);
    bool fok;
    if constexpr (kMixedLoop) {
        // the integer costs' shared memory is free now: the FP64 Hungarian reads
        // the gradient from there and edge permissions from the code bytes
        // (kAllowed is ub >= 1/2), the same arithmetic as lmo_forward
        double* Gs = L.cert_stage ? reinterpret_cast<double*>(mixed_costs(P, dsm, node)) : G;
        for (int j = tid; j < n; j += kThreads) {
            if (L.cert_stage) Gs[j] = G[j];
            V[j] = 0.0;
        }
        __syncthreads();
        {   // the certificate's lone oracle: the whole CTA as one group of eight warps
            const bool ok = hungarian_group<8>(hw0, c.lorder, Gs, 1.0, LB, UB, nullptr, V, mixed_codes(P, dsm, node), 0);
            if (threadIdx.x == 0) sh.flag[0] = ok;
        }
        __syncthreads();
        fok = sh.flag[0] != 0;
    } else {
        fok = lmo_forward<LK>(c, G, LB, UB, V);
    }
    score(V, (graph_perm && fok) ? hw0.pi : nullptr, hw0.pinv);
    double loc = 0.0;
    for (int j = tid; j < n; j += kThreads) loc = fma(G[j], X[j] - V[j], loc);
    const double fgap = bsum(loc, c.red);
    if constexpr (OK != GBX_OBJ_GRAPH_MATCHING) fval = obj_value(c, X);
    int st = (fgap >= 0.0 && fgap < eps) ? 1 : 0;
    if (c.flags) {
        bool zero_one = true;
        if constexpr (LK == GBX_LMO_LINKED_CARDINALITY) {
            linked_candidate(c, X, LB, UB, CAND);
            zero_one = false;
        } else {
            for (int j = tid; j < n; j += kThreads) {
                const double r = c.flags[j] ? round(X[j]) : X[j];
                CAND[j] = r;
                if (r != 0.0 && r != 1.0) zero_one = false;
            }
            __syncthreads();
        }
        if (rounded_feasible<LK>(c, CAND)) {
            // a 0/1 point with unit row and column sums is a permutation: its
            // value in O(m^2) is bit-identical to the generic one
            const bool perm = graph_perm && c.tol < 0.5 && __syncthreads_and(zero_one);
            int* cpi = hw1.pi;
            int* cpinv = hw1.pinv;
            if constexpr (kMixedLoop) {
                if (L.cluster) {
                    // the leader's in-face map arrays are free now
                    cpi = reinterpret_cast<int*>(dsm + L.sm_lpi) + 2 * c.m;
                    cpinv = cpi + c.m;
                } else if (L.hung_warps < 2) {
                    // one FP64 workspace: the in-face integer oracle's arrays are free now
                    const IHW wi = ihw_at(dsm + L.sm_ihw + L.ihw_bytes, c.m);
                    cpi = wi.pi;
                    cpinv = wi.pinv;
                }
            }
            if (perm) {
                for (int j = tid; j < n; j += kThreads)
                    if (CAND[j] == 1.0) cpi[j / c.m] = j - (j / c.m) * c.m;
                __syncthreads();
            }
            const double cv = integer_value(c, CAND, LB, UB, perm ? cpi : nullptr, cpinv);
            if (cv < best_val && writer) {
                for (int j = tid; j < n; j += kThreads) best[j] = CAND[j];
                if (tid == 0) P.b.best_vertex_val[node] = cv;
            }
        }
    }
    bool integral = true;
    for (int j = tid; j < n; j += kThreads)
        if (!isfinite(X[j]) || (c.flags && c.flags[j] && fabs(X[j] - round(X[j])) > c.tol))
            integral = false;
    if (__syncthreads_and(integral)) st = st ? GBX_NODE_INTEGRAL_CONVERGED : GBX_NODE_INTEGRAL_UNCONVERGED;
    if (!writer) return;
    for (int j = tid; j < n; j += kThreads) gx[j] = X[j];
    if (tid == 0) {
        P.b.value[node] = fval;
        P.b.gap[node] = fgap;
        P.b.status[node] = (uint8_t)st;
        P.b.iterations[node] = iters;
    }
}

// One CTA per node (grid = nodes), or a persistent grid whose CTAs take the
// next node from an atomic queue in the workspace until the batch is done.
template <int OK, int LK, int MIX, int MB>
__global__ void __launch_bounds__(kThreads, MB) relax_kernel(const __grid_constant__ Params P) {
    extern __shared__ __align__(16) unsigned char dsm[];
    __shared__ Scalars sh;
    // a batch assembled on the device (frontier rounds) carries its size in
    // device memory; the grid is sized for the largest batch
    const int n_nodes = P.live_count ? min(*P.live_count, P.b.n_nodes) : P.b.n_nodes;
    if (!P.queue) {
        if ((int)blockIdx.x < n_nodes) relax_node<OK, LK, MIX>(P, blockIdx.x, dsm, sh);
        return;
    }
    __shared__ int next;
    for (;;) {
        if (threadIdx.x == 0) next = atomicAdd(P.queue, 1);
        __syncthreads();
        const int node = next;
        __syncthreads();
        if (node >= n_nodes) return;
        relax_node<OK, LK, MIX>(P, node, dsm, sh);
        __syncthreads();
    }
}

// A pair of CTAs per node (a two-CTA cluster, FP64 dense quadratic objective):
// both run the node's relaxation on their own copy of it, each computing half
// of the objective's products and the lanes of its parity in the sums, which
// the pair exchanges through distributed shared memory; rank 0 writes the
// results. Every decision follows from values both CTAs compute identically, so
// they meet every cluster barrier; the last one keeps either CTA's shared
// memory alive until the peer's final stores into it are done.
template <int OK, int LK>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kThreads, 1)
    relax_pair_kernel(const __grid_constant__ Params P) {
    extern __shared__ __align__(16) unsigned char dsm[];
    __shared__ Scalars sh;
    const int n_nodes = P.live_count ? min(*P.live_count, P.b.n_nodes) : P.b.n_nodes;
    const int node = (int)(blockIdx.x >> 1);
    if (node < n_nodes) relax_node<OK, LK, 0>(P, node, dsm, sh);
    pair_sync();
}

// A cluster of kClCtas CTAs per node (the large-order mixed relaxation of
// cluster.cuh): CTA 0 relaxes the node, the others serve its oracles until
// it lets them go. Every CTA resets its oracle state and barriers before the
// cluster barrier that opens the launch, so no remote arrive meets an
// uninitialised barrier.
template <int OK, int LK>
__global__ void __cluster_dims__(kClCtas, 1, 1) __launch_bounds__(kThreads, 1)
    relax_cluster_kernel(const __grid_constant__ Params P) {
    extern __shared__ __align__(16) unsigned char dsm[];
    __shared__ Scalars sh;
    const Layout& L = P.L;
    const int m = P.obj.order;
    ClCtl* ctl = reinterpret_cast<ClCtl*>(dsm + L.sm_cl);
    if (threadIdx.x == 0) {
        cl_bar_init(&ctl->bar_go, 1);
        cl_bar_init(&ctl->bar_done, kClCtas - 1);
        ctl->released = 0;
        ctl->err = 0;
        chw_reset(chw_at(dsm + L.sm_chw, m));
        chw_reset(chw_at(dsm + L.sm_chw + L.chw_bytes, m));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    cl_sync_all();
    const int node = (int)(blockIdx.x / kClCtas);
    const int n_nodes = P.live_count ? min(*P.live_count, P.b.n_nodes) : P.b.n_nodes;
    if (cl_rank() == 0) {
        if (node < n_nodes) relax_node<OK, LK, 4>(P, node, dsm, sh);
        cl_release(ctl);   // (an infeasible or absent node lets the helpers go here)
    } else {
        cl_helper(P, node, dsm);
    }
}

// ------------------------------------------------------------------ LMO probes
template <int LK>
__global__ void __launch_bounds__(kThreads, 1) lmo_probe_kernel(
    gbx_lmo lmo, Layout L, int cases, int mode, const double* dir, const double* x,
    const double* lb, const double* ub, double* out, double* out_step, double* ws) {
    extern __shared__ __align__(16) unsigned char dsm[];
    __shared__ Scalars sh;
    const int cs = blockIdx.x;
    if (cs >= cases) return;
    const int n = lmo.n, tid = threadIdx.x;
    const size_t off = (size_t)cs * n;
    Ctx c;
    c.use_sp = false;
    c.n = n;
    c.tid = tid;
    c.red = sh.red;
    c.flag = sh.flag;
    c.lk = LK;
    c.rhs = lmo.right_side;
    c.is_int = lmo.is_int;
    c.lorder = lmo.order;
    c.U = lmo.upper;
    c.S = L.sort_size;
    c.keys = reinterpret_cast<double*>(dsm + L.sm_keys);
    c.prefix = reinterpret_cast<double*>(dsm + L.sm_prefix);
    c.idx = reinterpret_cast<int*>(dsm + L.sm_idx);
    c.fixed = dsm + L.sm_fixed;
    c.hung[0] = dsm + L.sm_hung;
    c.hung[1] = dsm + L.sm_hung + L.hung_bytes;
    c.flags = nullptr;
    c.tol = 0.0;
    c.pr = -1;
    c.xch = nullptr;
    double* o = out + off;
    if (mode == 0) {
        lmo_forward<LK>(c, dir + off, lb + off, ub + off, o);
        return;
    }
    if constexpr (LK == GBX_LMO_BIRKHOFF) {
        for (int j = tid; j < n; j += kThreads) o[j] = 0.0;
        __syncthreads();
        if (n == c.lorder * c.lorder && threadIdx.x < 32) lmo_inface<LK>(c, dir + off, 1.0, x + off, lb + off, ub + off, o, 0);
        __syncthreads();
    } else {
        lmo_inface<LK>(c, dir + off, 1.0, x + off, lb + off, ub + off, o, 0);
    }
    if (!out_step) return;
    // forward vertex of -direction, then the DICG maximum step
    double* fwd = ws + off * 2;
    double* d = fwd + n;
    double* neg = ws + (size_t)cases * n * 2 + off;
    for (int j = tid; j < n; j += kThreads) neg[j] = -dir[off + j];
    __syncthreads();
    lmo_forward<LK>(c, neg, lb + off, ub + off, fwd);
    for (int j = tid; j < n; j += kThreads) d[j] = o[j] - fwd[j];
    __syncthreads();
    const double st = lmo_max_step<LK>(c, d, x + off, lb + off, ub + off);
    if (tid == 0) out_step[cs] = st;
}

template <int LK>
__global__ void __launch_bounds__(kThreads, 1) feasible_kernel(
    gbx_lmo lmo, Layout L, int cases, const double* lb, const double* ub,
    const uint8_t* flags, uint8_t* out, double* ws) {
    extern __shared__ __align__(16) unsigned char dsm[];
    __shared__ Scalars sh;
    const int cs = blockIdx.x;
    if (cs >= cases) return;
    const int n = lmo.n;
    Ctx c;
    c.use_sp = false;
    c.n = n;
    c.tid = threadIdx.x;
    c.red = sh.red;
    c.flag = sh.flag;
    c.lk = LK;
    c.rhs = lmo.right_side;
    c.is_int = lmo.is_int;
    c.lorder = lmo.order;
    c.U = lmo.upper;
    c.S = L.sort_size;
    c.hung[0] = dsm + L.sm_hung;
    c.hung[1] = dsm + L.sm_hung + L.hung_bytes;
    c.flags = flags;
    c.tol = 0.0;
    c.pr = -1;
    c.xch = nullptr;
    const bool ok = node_feasible<LK>(c, lb + (size_t)cs * n, ub + (size_t)cs * n, ws + (size_t)cs * n);
    if (threadIdx.x == 0) out[cs] = ok ? 1 : 0;
}


// ------------------------------------------------------------------ launchers
// One kernel variant (MIX) of a kind; each variant of the graph-matching
// Birkhoff kernel is instantiated in its own translation unit.
// MB: CTAs per SM the kernel is compiled for (its register cap): two for the
// SIMT mixed shapes, one for the tensor-core shape, either for FP64.
template <int OK, int LK, int MIX, int MB = (MIX == 1 || MIX == 3) ? 2 : 1>
int launch_mix(const Params& p, cudaStream_t st, std::string* err) {
    auto k = relax_kernel<OK, LK, MIX, MB>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)std::max<size_t>(p.L.sm_total, 1));
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    int grid = p.b.n_nodes;
    if (p.queue) {
        // persistent: as many CTAs as stay resident, each pulling nodes
        int dev = 0, sms = 0, per_sm = 0;
        e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, p.L.sm_total);
        if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
        grid = std::max(1, std::min(grid, sms * std::max(per_sm, 1)));
        e = cudaMemsetAsync(p.queue, 0, sizeof(int), st);
        if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    }
    k<<<grid, kThreads, p.L.sm_total, st>>>(p);
    e = cudaGetLastError();
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    return GBX_OK;
}

// The pair launch: two CTAs per node (grid = 2 * nodes).
template <int OK, int LK>
int launch_pair(const Params& p, cudaStream_t st, std::string* err) {
    if constexpr (OK == GBX_OBJ_DENSE_QUADRATIC) {
        auto k = relax_pair_kernel<OK, LK>;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.L.sm_total);
        if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
        k<<<p.b.n_nodes * 2, kThreads, p.L.sm_total, st>>>(p);
        e = cudaGetLastError();
        if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
        return GBX_OK;
    } else {
        (void)p;
        (void)st;
        *err = "a pair of CTAs per node covers the dense quadratic objective";
        return GBX_ERR_UNSUPPORTED;
    }
}

// The cluster launch: kClCtas CTAs per node (grid = nodes * kClCtas).
template <int OK, int LK>
int launch_cluster(const Params& p, cudaStream_t st, std::string* err) {
    if constexpr (OK == GBX_OBJ_GRAPH_MATCHING && LK == GBX_LMO_BIRKHOFF) {
        auto k = relax_cluster_kernel<OK, LK>;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.L.sm_total);
        if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
        k<<<p.b.n_nodes * kClCtas, kThreads, p.L.sm_total, st>>>(p);
        e = cudaGetLastError();
        if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
        return GBX_OK;
    } else {
        (void)p;
        (void)st;
        *err = "a cluster per node covers mixed-precision graph matching over the Birkhoff polytope";
        return GBX_ERR_UNSUPPORTED;
    }
}

template <int OK, int LK>
int launch_one(const Params& p, cudaStream_t st, std::string* err) {
    if constexpr (OK == GBX_OBJ_DENSE_QUADRATIC)
        if (p.L.pair) return launch_pair<OK, LK>(p, st, err);
    if constexpr (OK == GBX_OBJ_GRAPH_MATCHING && LK == GBX_LMO_BIRKHOFF) {
        if (p.L.cluster) return launch_cluster<OK, LK>(p, st, err);
        if (p.L.mixed) {
            if (p.L.tc) return launch_mix<OK, LK, 2>(p, st, err);
            if (p.L.cost_global) return launch_mix<OK, LK, 3>(p, st, err);
            return launch_mix<OK, LK, 1>(p, st, err);
        }
    }
    return p.L.per_sm2 ? launch_mix<OK, LK, 0, 2>(p, st, err) : launch_mix<OK, LK, 0, 1>(p, st, err);
}

template <int LK>
int probe_one(const gbx_lmo& l, const Layout& L, int cases, int mode, const double* dir,
                     const double* x, const double* lb, const double* ub, double* out,
                     double* out_step, cudaStream_t st, std::string* err) {
    double* ws = nullptr;
    cudaError_t e = cudaSuccess;
    if (out_step) {
        e = cudaMallocAsync(&ws, (size_t)cases * l.n * 3 * sizeof(double), st);
        if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    }
    auto k = lmo_probe_kernel<LK>;
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max<size_t>(L.sm_total, 1));
    if (e == cudaSuccess) {
        k<<<cases, kThreads, L.sm_total, st>>>(l, L, cases, mode, dir, x, lb, ub, out, out_step, ws);
        e = cudaGetLastError();
    }
    if (ws) cudaFreeAsync(ws, st);
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    return GBX_OK;
}

template <int LK>
int feas_one(const gbx_lmo& l, const Layout& L, int cases, const double* lb,
                    const double* ub, const uint8_t* flags, uint8_t* out, cudaStream_t st,
                    std::string* err) {
    double* ws = nullptr;
    cudaError_t e = cudaMallocAsync(&ws, (size_t)cases * l.n * sizeof(double), st);
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    auto k = feasible_kernel<LK>;
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max<size_t>(L.sm_total, 1));
    if (e == cudaSuccess) {
        k<<<cases, kThreads, L.sm_total, st>>>(l, L, cases, lb, ub, flags, out, ws);
        e = cudaGetLastError();
    }
    cudaFreeAsync(ws, st);
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    return GBX_OK;
}

}  // namespace gbx
