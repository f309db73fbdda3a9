// mixed.cuh -- mixed-precision DICG / FW iteration for the Birkhoff
// graph-matching relaxation (GBX_PRECISION_MIXED), included by relax.cu.
//
// Per iteration the FP64 iterate x steers, but the O(m^3) gradient and the
// O(m^3) assignment oracles leave the FP64 pipe (2 ops/clk/SM on GB300):
//   * gradient  g = 2s(A'R - RB'), R = AX - XB in FP32 (X rounded to FP32);
//   * oracles   exact min-cost assignment on integer costs round(g * 2^k)
//               (k chosen per call so |cost| <= 2^24/m), solved by a warp-level
//               shortest-augmenting-path Hungarian whose column potentials and
//               matching persist between iterations (warm start): each call
//               re-derives row potentials from the kept column potentials, keeps
//               the still-tight matched edges and augments only the rest;
//   * DICG step on permutations: the pairwise direction a - v has at most 2m
//               non-zeros, so the gap, the maximum step, the update of x and the
//               exact quadratic curvature 2s||A(a-v) - (a-v)B||^2 (gathers) are
//               O(m) / O(m^2).
// The certificate at the returned iterate stays FP64 and exact (relax.cu).
#pragma once

namespace gbx {

constexpr int kIntInf = 0x3fffffff;
// |kept column potential| is clamped here; costs stay below 2^24/m, so every
// reduced cost c - u - v of a call fits comfortably in 32 bits.
constexpr long long kPotLimit = 1ll << 26;

// per-edge code bytes of a node (computed once per launch)
constexpr uint8_t kForced = 1;     // lb > 1/2
constexpr uint8_t kAllowed = 2;    // ub >= 1/2
constexpr uint8_t kBad = 4;        // lb > ub + 1e-9
constexpr uint8_t kZeroOk = 8;     // 0 lies in [lb - tol, ub + tol]
constexpr uint8_t kOneOk = 16;     // 1 lies in [lb - tol, ub + tol]
// face bytes (DICG in-face oracle)
constexpr uint8_t kFaceIn = 1;     // x > 1e-9
constexpr uint8_t kFaceOne = 2;    // x >= 1 - 1e-9

struct IHW {
    int *u, *pv, *minv, *p, *way;
    int *rows, *cols, *rowpos, *fcol, *frow, *pi, *colpot, *match, *pinv;
    uint8_t *used, *rmatch;
    int* scal;   // [0] warm state valid, [1] shift of the stored potentials
};

__device__ inline IHW ihw_at(unsigned char* base, int m) {
    IHW w;
    size_t o = 0;
    w.u = reinterpret_cast<int*>(base);
    w.pv = w.u + (m + 1);
    w.minv = w.pv + (m + 1);
    w.p = w.minv + (m + 1);
    w.way = w.p + (m + 1);
    o += align16(5 * (size_t)(m + 1) * sizeof(int));
    w.rows = reinterpret_cast<int*>(base + o);
    w.cols = w.rows + m;
    w.rowpos = w.cols + m;
    w.fcol = w.rowpos + m;
    w.frow = w.fcol + m;
    w.pi = w.frow + m;
    w.colpot = w.pi + m;
    w.match = w.colpot + m;
    w.pinv = w.match + m;
    o += align16(9 * (size_t)m * sizeof(int));
    w.used = base + o;
    w.rmatch = w.used + (m + 1);
    o += align16((size_t)(m + 1) * 2);
    w.scal = reinterpret_cast<int*>(base + o);
    return w;
}

__device__ __forceinline__ int scaled_cost(const float* g, int e, float sign, int shift) {
    return __float2int_rn(scalbnf(sign * g[e], shift));
}

// Exact assignment on the integer costs round(sign*g*2^shift) over the
// Birkhoff polytope restricted by the edge codes (and the face of x when
// `face` is given). One warp. Leaves the row->column map in w.pi and keeps
// column potentials / matching for the next call. Returns a warp-uniform flag.
static __device__ bool int_hungarian_warp(const IHW& w, int m, const float* g, float sign, int shift,
                                   const uint8_t* code, const uint8_t* face) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    for (int i = lane; i < m; i += 32) { w.fcol[i] = -1; w.frow[i] = -1; }
    __syncwarp();
    bool ok = true;
    const int nn = m * m;
    for (int e = lane; e < nn; e += 32) {
        const uint8_t c = code[e];
        if (c & kBad) ok = false;
        const bool forced = (c & kForced) || (face && (face[e] & kFaceOne));
        if (forced) {
            const int r = e / m, col = e - r * m;
            if (!(c & kAllowed)) ok = false;
            if (atomicCAS(&w.fcol[r], -1, col) != -1) ok = false;
            if (atomicCAS(&w.frow[col], -1, r) != -1) ok = false;
        }
    }
    ok = __all_sync(kFull, ok);
    __syncwarp();
    if (!ok) return false;
    int k = 0, kc = 0;
    for (int base = 0; base < m; base += 32) {
        const int i = base + lane;
        const bool fr = i < m && w.fcol[i] < 0;
        const bool fc = i < m && w.frow[i] < 0;
        const unsigned mr = __ballot_sync(kFull, fr), mc = __ballot_sync(kFull, fc);
        if (fr) { w.rows[k + __popc(mr & lt)] = i; }
        if (i < m) w.rowpos[i] = fr ? k + __popc(mr & lt) + 1 : 0;
        if (fc) w.cols[kc + __popc(mc & lt)] = i;
        k += __popc(mr);
        kc += __popc(mc);
    }
    if (k != kc) return false;
    __syncwarp();
    const bool warm = w.scal[0] != 0;
    const int old_shift = w.scal[1];
    // column potentials: kept (rescaled to this call's cost scale) or zero
    for (int j = lane + 1; j <= k; j += 32) {
        int v = 0;
        if (warm) {
            long long t = w.colpot[w.cols[j - 1]];
            const int d = shift - old_shift;
            if (d > 0) t = d >= 24 ? 0 : t * (1ll << d);
            else if (d < 0) t = -d >= 40 ? 0 : (t >> (-d));
            v = (int)max(-kPotLimit, min(kPotLimit, t));
        }
        w.pv[j] = v;
        w.p[j] = 0;
        w.way[j] = 0;
    }
    if (lane == 0) { w.pv[0] = 0; w.p[0] = 0; }
    __syncwarp();
    // row potentials u_i = min_j (c_ij - v_j): dual feasible for the new costs
    for (int i = 1; i <= k; ++i) {
        const int rb = w.rows[i - 1] * m;
        int best = kIntInf;
        for (int j = lane + 1; j <= k; j += 32) {
            const int e = rb + w.cols[j - 1];
            if ((code[e] & kAllowed) && (!face || (face[e] & kFaceIn))) {
                const int r = scaled_cost(g, e, sign, shift) - w.pv[j];
                best = r < best ? r : best;
            }
        }
        best = __reduce_min_sync(kFull, best);
        if (best >= kIntInf) return false;
        if (lane == 0) { w.u[i] = best; w.rmatch[i] = 0; }
    }
    __syncwarp();
    // keep the previous matching where its edge is still allowed and tight
    if (warm) {
        for (int j = lane + 1; j <= k; j += 32) {
            const int c = w.cols[j - 1];
            const int r = w.match[c];
            if (r < 0 || r >= m) continue;
            const int i = w.rowpos[r];
            if (i <= 0) continue;
            const int e = r * m + c;
            if ((code[e] & kAllowed) && (!face || (face[e] & kFaceIn))
                    && scaled_cost(g, e, sign, shift) - w.u[i] - w.pv[j] == 0) {
                w.p[j] = i;
                w.rmatch[i] = 1;
            }
        }
    }
    __syncwarp();
    // augment every unmatched row along a shortest path
    for (int i = 1; i <= k; ++i) {
        if (w.rmatch[i]) continue;
        for (int j = lane; j <= k; j += 32) { w.minv[j] = kIntInf; w.used[j] = 0; }
        if (lane == 0) w.p[0] = i;
        __syncwarp();
        int j0 = 0;
        int step = 0;
        for (; step <= k; ++step) {
            if (lane == 0) w.used[j0] = 1;
            __syncwarp();
            const int i0 = w.p[j0];
            const int ui0 = w.u[i0];
            const int rb = w.rows[i0 - 1] * m;
            int bv = kIntInf, bj = 0x7fffffff;
            for (int j = lane + 1; j <= k; j += 32) {
                if (w.used[j]) continue;
                const int e = rb + w.cols[j - 1];
                int mv = w.minv[j];
                if ((code[e] & kAllowed) && (!face || (face[e] & kFaceIn))) {
                    const int cur = scaled_cost(g, e, sign, shift) - ui0 - w.pv[j];
                    if (cur < mv) { mv = cur; w.minv[j] = cur; w.way[j] = j0; }
                }
                if (mv < bv) { bv = mv; bj = j; }
            }
            const int gmin = __reduce_min_sync(kFull, bv);
            if (gmin >= kIntInf) return false;
            const int j1 = __reduce_min_sync(kFull, bv == gmin ? bj : 0x7fffffff);
            __syncwarp();
            for (int j = lane; j <= k; j += 32) {
                if (w.used[j]) { w.u[w.p[j]] += gmin; w.pv[j] -= gmin; }
                else if (w.minv[j] < kIntInf) w.minv[j] -= gmin;
            }
            __syncwarp();
            j0 = j1;
            if (w.p[j0] == 0) break;
        }
        if (w.p[j0] != 0) return false;
        if (lane == 0) {
            int jj = j0;
            for (int guard = 0; guard <= k && jj != 0; ++guard) {
                const int jp = w.way[jj];
                w.p[jj] = w.p[jp];
                jj = jp;
            }
        }
        __syncwarp();
    }
    // outputs and the warm state for the next call (original indices)
    for (int i = lane; i < m; i += 32) {
        if (w.fcol[i] >= 0) { w.pi[i] = w.fcol[i]; w.match[w.fcol[i]] = i; }
    }
    for (int j = lane + 1; j <= k; j += 32) {
        const int r = w.rows[w.p[j] - 1], c = w.cols[j - 1];
        w.pi[r] = c;
        w.match[c] = r;
        w.colpot[c] = w.pv[j];
    }
    __syncwarp();
    int lo = kIntInf;
    for (int j = lane + 1; j <= k; j += 32) lo = min(lo, w.pv[j]);
    lo = __reduce_min_sync(kFull, lo);
    if (lo >= kIntInf) lo = 0;
    bool sane = true;
    for (int j = lane + 1; j <= k; j += 32) {
        const int v = w.colpot[w.cols[j - 1]] - lo;
        w.colpot[w.cols[j - 1]] = v;
        sane = sane && v <= kPotLimit;
    }
    sane = __all_sync(kFull, sane);
    if (lane == 0) { w.scal[0] = sane ? 1 : 0; w.scal[1] = shift; }
    __syncwarp();
    return true;
}

// Block-wide max of |v| over n floats (broadcast).
static __device__ float bmax_abs(const float* v, int n, double* red) {
    float mx = 0.f;
    for (int e = threadIdx.x; e < n; e += kThreads) mx = fmaxf(mx, fabsf(v[e]));
    for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_down_sync(kFull, mx, off));
    __syncthreads();
    float* r = reinterpret_cast<float*>(red);
    if ((threadIdx.x & 31) == 0) r[threadIdx.x >> 5] = mx;
    __syncthreads();
    float out = 0.f;
    for (int w = 0; w < kWarps; ++w) out = fmaxf(out, r[w]);
    __syncthreads();
    return out;
}

// FP32 gradient g = 2s(A'R - RB') with R = AX - XB; A, B, Bt given in FP32.
static __device__ void grad_f32(int m, float two_s, const float* A, const float* B, const float* Bt, const float* X,
                         float* R, float* G) {
    const int n = m * m;
    for (int e = threadIdx.x; e < n; e += kThreads) {
        const int i = e / m, j = e - (e / m) * m;
        float r = 0.f;
        for (int k = 0; k < m; ++k) {
            r = fmaf(A[i * m + k], X[k * m + j], r);
            r = fmaf(-X[i * m + k], B[k * m + j], r);
        }
        R[e] = r;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n; e += kThreads) {
        const int p = e / m, q = e - (e / m) * m;
        float acc = 0.f;
        for (int r = 0; r < m; ++r) acc = fmaf(A[r * m + p], R[r * m + q], acc);
        for (int c = 0; c < m; ++c) acc = fmaf(-R[p * m + c], Bt[c * m + q], acc);
        G[e] = two_s * acc;
    }
    __syncthreads();
}

}  // namespace gbx
