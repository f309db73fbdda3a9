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
// the iterate's face, in the same byte (DICG in-face oracle)
constexpr uint8_t kFaceIn = 32;    // x > 1e-9
constexpr uint8_t kFaceOne = 64;   // x >= 1 - 1e-9
constexpr uint8_t kFaceBits = kFaceIn | kFaceOne;

// Packed costs (large orders): one array serves both oracles of an
// iteration, (cost << 1) | face bit for an allowed edge, kIntInf otherwise.
// FACE 3 reads it as the forward costs, FACE 4 as the in-face costs (the
// negated cost on the iterate's face, kIntInf elsewhere) -- the values FACE 0
// and FACE 1 read from two separate arrays, so the assignments are identical.
__device__ __forceinline__ int packed_forward(int v) { return v >= kIntInf ? kIntInf : (v >> 1); }
__device__ __forceinline__ int packed_inface(int v) { return (v < kIntInf && (v & 1)) ? -(v >> 1) : kIntInf; }
__device__ __forceinline__ int pack_cost(int ci, bool allowed, bool face) {
    return allowed ? (int)(((unsigned)ci << 1) | (face ? 1u : 0u)) : kIntInf;
}

struct IHW {
    int *u, *rowb, *pvs;                         // [m+1] row potentials, row offsets r*m, column potentials
    int *rows, *cols, *rowpos, *fcol, *frow, *pi, *colpot, *match, *pinv;  // [m]
    uint8_t* rmatch;                             // [m+1]
    int* scal;   // [0] warm state valid, [1] shift of the stored potentials, [2] k+1 of the cached restriction (0: none)
};

__device__ inline IHW ihw_at(unsigned char* base, int m) {
    IHW w;
    size_t o = 0;
    w.u = reinterpret_cast<int*>(base);
    w.rowb = w.u + (m + 1);
    w.pvs = w.rowb + (m + 1);
    o += align16(3 * (size_t)(m + 1) * sizeof(int));
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
    w.rmatch = base + o;
    o += align16((size_t)(m + 1));
    w.scal = reinterpret_cast<int*>(base + o);
    return w;
}

template <int CPL>
__device__ __forceinline__ int lane_slot(const int (&a)[CPL], int slot) {
    int v = 0;
#pragma unroll
    for (int t = 0; t < CPL; ++t)
        if (t == slot) v = a[t];
    return v;
}

// Slacks below this bound travel as one packed 32-bit key (slack << 10 | column)
// through a single warp min-reduction; larger ones take the two-reduction path.
constexpr int kPackLimit = 1 << 21;

// Exact assignment on integer costs over the Birkhoff polytope. `costs` holds
// round(g*2^shift) for allowed edges and kIntInf for excluded ones; the
// in-face oracle (FACE 1: `costs` already holds its negated face costs; FACE
// 2: it negates the forward costs on the iterate's face -- edge code bit
// kFaceIn -- and excludes every other edge) also forces the face's unit
// entries (kFaceOne). The
// forced / face-forced pre-pass reads the edge codes and is skipped when
// `restrict_same` says the restrictions equal those of the previous call. One
// warp; lane l owns the compacted columns l+1, l+33, ... and keeps, per column,
// its potential, slack, predecessor, matched row and that row's potential and
// offset in registers (CPL columns per lane: the compacted order k must not
// exceed 32*CPL). Shortest augmenting paths use lazy potentials: slacks are
// stored offset by the running path length D, a column remembers the D at
// which it joined the tree, and potentials are applied once per path; the
// reached row's potential is still its value from the path's start when it is
// relaxed, so the integer arithmetic equals the eager update exactly. Column
// potentials and the matching persist in `w`. Ties go to the lowest column.
// Returns a warp-uniform success flag; the row->column map is left in w.pi.
template <int CPL, int FACE>
__device__ bool int_hungarian_warp(const IHW& w, int m, const int* costs, int shift, const uint8_t* code,
                                   bool restrict_same) {
    const int lane = threadIdx.x & 31;
    auto cost_at = [&](int e) -> int {
        const int c0 = costs[e];
        if constexpr (FACE == 2) return (c0 < kIntInf && (code[e] & kFaceIn)) ? -c0 : kIntInf;
        else if constexpr (FACE == 3) return packed_forward(c0);
        else if constexpr (FACE == 4) return packed_inface(c0);
        else return c0;
    };
    const unsigned lt = (1u << lane) - 1u;
    int k;
    if (restrict_same && w.scal[2] > 0) {
        k = w.scal[2] - 1;
    } else {
        for (int i = lane; i < m; i += 32) { w.fcol[i] = -1; w.frow[i] = -1; }
        __syncwarp();
        bool ok = true;
        const int nn = m * m;
        for (int e = lane; e < nn; e += 32) {
            const uint8_t c = code[e];
            if (c & kBad) ok = false;
            const bool forced = (c & kForced) || (FACE != 0 && FACE != 3 && (c & kFaceOne));
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
        k = 0;
        int kc = 0;
        for (int base = 0; base < m; base += 32) {
            const int i = base + lane;
            const bool fr = i < m && w.fcol[i] < 0;
            const bool fc = i < m && w.frow[i] < 0;
            const unsigned mr = __ballot_sync(kFull, fr), mc = __ballot_sync(kFull, fc);
            if (fr) w.rows[k + __popc(mr & lt)] = i;
            if (i < m) w.rowpos[i] = fr ? k + __popc(mr & lt) + 1 : 0;
            if (fc) w.cols[kc + __popc(mc & lt)] = i;
            k += __popc(mr);
            kc += __popc(mc);
        }
        if (k != kc || k > 32 * CPL) return false;
        for (int i = lane + 1; i <= k; i += 32) w.rowb[i] = w.rows[i - 1] * m;
        if (lane == 0) w.scal[2] = k + 1;
        __syncwarp();
    }
    const bool warm = w.scal[0] != 0;
    const int dshift = shift - w.scal[1];
    int colE[CPL], pv[CPL], mraw[CPL], way[CPL], pj[CPL], usedAt[CPL], ur[CPL], rbr[CPL];
    bool valid[CPL];
#pragma unroll
    for (int t = 0; t < CPL; ++t) {
        const int j = lane + 1 + 32 * t;
        valid[t] = j <= k;
        colE[t] = valid[t] ? w.cols[j - 1] : 0;
        long long v = 0;
        if (valid[t] && warm) {
            v = w.colpot[colE[t]];
            if (dshift > 0) v = dshift >= 24 ? 0 : v * (1ll << dshift);
            else if (dshift < 0) v = -dshift >= 40 ? 0 : (v >> (-dshift));
            v = max(-kPotLimit, min(kPotLimit, v));
        }
        pv[t] = (int)v;
        pj[t] = 0;
        ur[t] = 0;
        rbr[t] = 0;
        if (valid[t]) w.pvs[j] = pv[t];
    }
    __syncwarp();
    // row potentials u_i = min_j (c_ij - v_j), one row per lane
    bool rows_ok = true;
    for (int i = lane + 1; i <= k; i += 32) {
        const int rb = w.rowb[i];
        int best = kIntInf, barg = 0;
        int j = 1;
        // eight columns' costs in flight at a time, compared in column order
        for (; j + 7 <= k; j += 8) {
            int cc[8], pp[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) { cc[q] = cost_at(rb + w.cols[j - 1 + q]); pp[q] = w.pvs[j + q]; }
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (cc[q] < kIntInf && cc[q] - pp[q] < best) { best = cc[q] - pp[q]; barg = j + q; }
        }
        for (; j <= k; ++j) {
            const int c = cost_at(rb + w.cols[j - 1]);
            if (c < kIntInf && c - w.pvs[j] < best) { best = c - w.pvs[j]; barg = j; }
        }
        if (best >= kIntInf) rows_ok = false;
        w.u[i] = best;
        w.pinv[i - 1] = barg;   // a tight column of row i (pinv is free during the call)
        w.rmatch[i] = 0;
    }
    if (!__all_sync(kFull, rows_ok)) return false;
    __syncwarp();
    // keep the previous matching where its edge is still allowed and tight
    if (warm) {
#pragma unroll
        for (int t = 0; t < CPL; ++t) {
            if (!valid[t]) continue;
            const int r = w.match[colE[t]];
            if (r < 0 || r >= m) continue;
            const int i = w.rowpos[r];
            if (i <= 0) continue;
            const int c = cost_at(r * m + colE[t]);
            const int ui = w.u[i];
            if (c < kIntInf && c - ui - pv[t] == 0) {
                pj[t] = i;
                ur[t] = ui;
                rbr[t] = w.rowb[i];
                w.rmatch[i] = 1;
            }
        }
    }
    __syncwarp();
    // greedy tight matching: every row still free claims its tight column, the
    // lowest row wins a contested free column (deterministic); the partial
    // matching is consistent with the potentials, so only the losers need paths
    {
        int* claim = w.pi;   // per compacted column; pi is rewritten at the end
#pragma unroll
        for (int t = 0; t < CPL; ++t)
            if (valid[t]) claim[lane + 32 * t] = pj[t] ? 0 : 0x7fffffff;
        __syncwarp();
        for (int i = lane + 1; i <= k; i += 32)
            if (!w.rmatch[i]) atomicMin(&claim[w.pinv[i - 1] - 1], i);
        __syncwarp();
#pragma unroll
        for (int t = 0; t < CPL; ++t) {
            if (!valid[t] || pj[t]) continue;
            const int r = claim[lane + 32 * t];
            if (r != 0x7fffffff) {
                pj[t] = r;
                ur[t] = w.u[r];
                rbr[t] = w.rowb[r];
                w.rmatch[r] = 1;
            }
        }
        __syncwarp();
    }
    bool feasible = true;
    for (int i = 1; i <= k && feasible; ++i) {
        if (w.rmatch[i]) continue;
#pragma unroll
        for (int t = 0; t < CPL; ++t) {
            mraw[t] = kIntInf;
            way[t] = 0;
            usedAt[t] = -1;
        }
        int j0 = 0, D = 0;
        int ui0 = w.u[i], rb = w.rowb[i];
        bool augmented = false;
        for (int step = 0; step <= k; ++step) {
            int bv = kIntInf, bj = 0x7fffffff;
            if constexpr (CPL >= 8) {
                // large orders read their costs from L2: all of this lane's costs
                // of the row at once (invalid slots read column 0 of the same row),
                // then the scan -- one memory latency per step instead of CPL
                int cv[CPL];
#pragma unroll
                for (int t = 0; t < CPL; ++t) cv[t] = cost_at(rb + colE[t]);
#pragma unroll
                for (int t = 0; t < CPL; ++t) {
                    const bool live = valid[t] && usedAt[t] < 0;
                    const int c = cv[t];
                    const int cur = c < kIntInf ? c - ui0 - pv[t] + D : kIntInf;
                    if (live && c < kIntInf && cur < mraw[t]) { mraw[t] = cur; way[t] = j0; }
                    if (live && mraw[t] < bv) { bv = mraw[t]; bj = lane + 1 + 32 * t; }
                }
            } else {
#pragma unroll
                for (int t = 0; t < CPL; ++t) {
                    if (!valid[t] || usedAt[t] >= 0) continue;
                    const int c = cost_at(rb + colE[t]);
                    if (c < kIntInf) {
                        const int cur = c - ui0 - pv[t] + D;
                        if (cur < mraw[t]) { mraw[t] = cur; way[t] = j0; }
                    }
                    if (mraw[t] < bv) { bv = mraw[t]; bj = lane + 1 + 32 * t; }
                }
            }
            int gmin, j1;
            const int key = bv < kPackLimit ? (bv << 10) | bj : 0x7fffffff;
            const int kmin = __reduce_min_sync(kFull, key);
            if (kmin != 0x7fffffff) {
                gmin = kmin >> 10;
                j1 = kmin & 1023;
            } else {
                gmin = __reduce_min_sync(kFull, bv);
                if (gmin >= kIntInf) { feasible = false; break; }
                j1 = __reduce_min_sync(kFull, bv == gmin ? bj : 0x7fffffff);
            }
            D = gmin;
            const int owner = (j1 - 1) & 31, slot = (j1 - 1) >> 5;
            const int pnext = __shfl_sync(kFull, lane_slot<CPL>(pj, slot), owner);
            const int unext = __shfl_sync(kFull, lane_slot<CPL>(ur, slot), owner);
            const int rnext = __shfl_sync(kFull, lane_slot<CPL>(rbr, slot), owner);
            if (lane == owner) {
#pragma unroll
                for (int t = 0; t < CPL; ++t)
                    if (t == slot) usedAt[t] = D;
            }
            j0 = j1;
            if (pnext == 0) { augmented = true; break; }
            ui0 = unext;
            rb = rnext;
        }
        if (!feasible || !augmented) { feasible = false; break; }
        // apply the potentials of this path (before the matching flips)
        const int uroot = w.u[i] + D;
#pragma unroll
        for (int t = 0; t < CPL; ++t) {
            if (usedAt[t] < 0) continue;
            const int d = D - usedAt[t];
            pv[t] -= d;
            ur[t] += d;
        }
        // flip the path: column j takes the row (and its potential / offset) of way[j]
        int j = j0;
        for (int guard = 0; guard <= k && j != 0; ++guard) {
            const int owner = (j - 1) & 31, slot = (j - 1) >> 5;
            const int jp = __shfl_sync(kFull, lane_slot<CPL>(way, slot), owner);
            int np = i, nu = uroot, nr = w.rowb[i];
            if (jp != 0) {
                const int po = (jp - 1) & 31, ps = (jp - 1) >> 5;
                np = __shfl_sync(kFull, lane_slot<CPL>(pj, ps), po);
                nu = __shfl_sync(kFull, lane_slot<CPL>(ur, ps), po);
                nr = __shfl_sync(kFull, lane_slot<CPL>(rbr, ps), po);
            }
            if (lane == owner) {
#pragma unroll
                for (int t = 0; t < CPL; ++t)
                    if (t == slot) { pj[t] = np; ur[t] = nu; rbr[t] = nr; }
            }
            j = jp;
        }
        __syncwarp();
    }
    if (!__all_sync(kFull, feasible)) return false;
    // outputs and the warm state for the next call (original indices)
    for (int i = lane; i < m; i += 32)
        if (w.fcol[i] >= 0) { w.pi[i] = w.fcol[i]; w.match[w.fcol[i]] = i; }
    int lo = kIntInf;
#pragma unroll
    for (int t = 0; t < CPL; ++t) {
        if (!valid[t]) continue;
        const int r = w.rows[pj[t] - 1];
        w.pi[r] = colE[t];
        w.match[colE[t]] = r;
        lo = min(lo, pv[t]);
    }
    lo = __reduce_min_sync(kFull, lo);
    if (lo >= kIntInf) lo = 0;
    bool sane = true;
#pragma unroll
    for (int t = 0; t < CPL; ++t) {
        if (!valid[t]) continue;
        const int v = pv[t] - lo;
        w.colpot[colE[t]] = v;
        sane = sane && v <= kPotLimit;
    }
    sane = __all_sync(kFull, sane);
    if (lane == 0) { w.scal[0] = sane ? 1 : 0; w.scal[1] = shift; }
    __syncwarp();
    return true;
}

// int_hungarian_warp with the per-column state (potential, slack, predecessor,
// matched row with its potential and offset, the D at which a column joined
// the tree) in shared memory `cs` (colstate_bytes(CPL) bytes, one warp): the
// same shortest-augmenting-path steps, ties and results, in about 40
// registers instead of ~9*CPL, so that two large-order nodes fit on an SM.
// The owner of the step's column is read straight from shared memory instead
// of being shuffled from its lane.
template <int CPL, int FACE>
__device__ bool int_hungarian_warp_cs(const IHW& w, int* cs, int m, const int* costs, int shift,
                                      const uint8_t* code, bool restrict_same) {
    const int lane = threadIdx.x & 31;
    auto S = [&](int a, int t) -> int& { return cs[(a * CPL + t) * 32 + lane]; };
    auto O = [&](int a, int t, int l) -> int { return cs[(a * CPL + t) * 32 + l]; };
    auto cost_at = [&](int e) -> int {
        const int c0 = costs[e];
        if constexpr (FACE == 2) return (c0 < kIntInf && (code[e] & kFaceIn)) ? -c0 : kIntInf;
        else if constexpr (FACE == 3) return packed_forward(c0);
        else if constexpr (FACE == 4) return packed_inface(c0);
        else return c0;
    };
    const unsigned lt = (1u << lane) - 1u;
    int k;
    if (restrict_same && w.scal[2] > 0) {
        k = w.scal[2] - 1;
    } else {
        for (int i = lane; i < m; i += 32) { w.fcol[i] = -1; w.frow[i] = -1; }
        __syncwarp();
        bool ok = true;
        const int nn = m * m;
        for (int e = lane; e < nn; e += 32) {
            const uint8_t c = code[e];
            if (c & kBad) ok = false;
            const bool forced = (c & kForced) || (FACE != 0 && FACE != 3 && (c & kFaceOne));
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
        k = 0;
        int kc = 0;
        for (int base = 0; base < m; base += 32) {
            const int i = base + lane;
            const bool fr = i < m && w.fcol[i] < 0;
            const bool fc = i < m && w.frow[i] < 0;
            const unsigned mr = __ballot_sync(kFull, fr), mc = __ballot_sync(kFull, fc);
            if (fr) w.rows[k + __popc(mr & lt)] = i;
            if (i < m) w.rowpos[i] = fr ? k + __popc(mr & lt) + 1 : 0;
            if (fc) w.cols[kc + __popc(mc & lt)] = i;
            k += __popc(mr);
            kc += __popc(mc);
        }
        if (k != kc || k > 32 * CPL) return false;
        for (int i = lane + 1; i <= k; i += 32) w.rowb[i] = w.rows[i - 1] * m;
        if (lane == 0) w.scal[2] = k + 1;
        __syncwarp();
    }
    const bool warm = w.scal[0] != 0;
    const int dshift = shift - w.scal[1];
    for (int t = 0; t < CPL; ++t) {
        const int j = lane + 1 + 32 * t;
        const bool valid = j <= k;
        const int col = valid ? w.cols[j - 1] : 0;
        long long v = 0;
        if (valid && warm) {
            v = w.colpot[col];
            if (dshift > 0) v = dshift >= 24 ? 0 : v * (1ll << dshift);
            else if (dshift < 0) v = -dshift >= 40 ? 0 : (v >> (-dshift));
            v = max(-kPotLimit, min(kPotLimit, v));
        }
        S(CS_COL, t) = col;
        S(CS_PV, t) = (int)v;
        S(CS_PJ, t) = 0;
        S(CS_UR, t) = 0;
        S(CS_RBR, t) = 0;
        if (valid) w.pvs[j] = (int)v;
    }
    __syncwarp();
    // row potentials u_i = min_j (c_ij - v_j), one row per lane
    bool rows_ok = true;
    for (int i = lane + 1; i <= k; i += 32) {
        const int rb = w.rowb[i];
        int best = kIntInf, barg = 0;
        int j = 1;
        for (; j + 7 <= k; j += 8) {
            int cc[8], pp[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) { cc[q] = cost_at(rb + w.cols[j - 1 + q]); pp[q] = w.pvs[j + q]; }
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (cc[q] < kIntInf && cc[q] - pp[q] < best) { best = cc[q] - pp[q]; barg = j + q; }
        }
        for (; j <= k; ++j) {
            const int c = cost_at(rb + w.cols[j - 1]);
            if (c < kIntInf && c - w.pvs[j] < best) { best = c - w.pvs[j]; barg = j; }
        }
        if (best >= kIntInf) rows_ok = false;
        w.u[i] = best;
        w.pinv[i - 1] = barg;   // a tight column of row i (pinv is free during the call)
        w.rmatch[i] = 0;
    }
    if (!__all_sync(kFull, rows_ok)) return false;
    __syncwarp();
    // keep the previous matching where its edge is still allowed and tight
    if (warm) {
        for (int t = 0; t < CPL; ++t) {
            if (lane + 1 + 32 * t > k) continue;
            const int col = S(CS_COL, t);
            const int r = w.match[col];
            if (r < 0 || r >= m) continue;
            const int i = w.rowpos[r];
            if (i <= 0) continue;
            const int c = cost_at(r * m + col);
            const int ui = w.u[i];
            if (c < kIntInf && c - ui - S(CS_PV, t) == 0) {
                S(CS_PJ, t) = i;
                S(CS_UR, t) = ui;
                S(CS_RBR, t) = w.rowb[i];
                w.rmatch[i] = 1;
            }
        }
    }
    __syncwarp();
    // greedy tight matching: every free row claims its tight column, the lowest
    // row wins a contested free column
    {
        int* claim = w.pi;   // per compacted column; pi is rewritten at the end
        for (int t = 0; t < CPL; ++t)
            if (lane + 1 + 32 * t <= k) claim[lane + 32 * t] = S(CS_PJ, t) ? 0 : 0x7fffffff;
        __syncwarp();
        for (int i = lane + 1; i <= k; i += 32)
            if (!w.rmatch[i]) atomicMin(&claim[w.pinv[i - 1] - 1], i);
        __syncwarp();
        for (int t = 0; t < CPL; ++t) {
            if (lane + 1 + 32 * t > k || S(CS_PJ, t)) continue;
            const int r = claim[lane + 32 * t];
            if (r != 0x7fffffff) {
                S(CS_PJ, t) = r;
                S(CS_UR, t) = w.u[r];
                S(CS_RBR, t) = w.rowb[r];
                w.rmatch[r] = 1;
            }
        }
        __syncwarp();
    }
    bool feasible = true;
    for (int i = 1; i <= k && feasible; ++i) {
        if (w.rmatch[i]) continue;
        for (int t = 0; t < CPL; ++t) {
            S(CS_MRAW, t) = kIntInf;
            S(CS_WAY, t) = 0;
            S(CS_USED, t) = -1;
        }
        int j0 = 0, D = 0;
        int ui0 = w.u[i], rb = w.rowb[i];
        bool augmented = false;
        for (int step = 0; step <= k; ++step) {
            int bv = kIntInf, bj = 0x7fffffff;
            // all of this lane's costs of the row at once (invalid slots read
            // column 0 of the same row), then the scan
            int cv[CPL];
#pragma unroll
            for (int t = 0; t < CPL; ++t) cv[t] = cost_at(rb + S(CS_COL, t));
#pragma unroll
            for (int t = 0; t < CPL; ++t) {
                const bool live = lane + 1 + 32 * t <= k && S(CS_USED, t) < 0;
                const int c = cv[t];
                int mr = S(CS_MRAW, t);
                if (live && c < kIntInf) {
                    const int cur = c - ui0 - S(CS_PV, t) + D;
                    if (cur < mr) { mr = cur; S(CS_MRAW, t) = cur; S(CS_WAY, t) = j0; }
                }
                if (live && mr < bv) { bv = mr; bj = lane + 1 + 32 * t; }
            }
            int gmin, j1;
            const int key = bv < kPackLimit ? (bv << 10) | bj : 0x7fffffff;
            const int kmin = __reduce_min_sync(kFull, key);
            if (kmin != 0x7fffffff) {
                gmin = kmin >> 10;
                j1 = kmin & 1023;
            } else {
                gmin = __reduce_min_sync(kFull, bv);
                if (gmin >= kIntInf) { feasible = false; break; }
                j1 = __reduce_min_sync(kFull, bv == gmin ? bj : 0x7fffffff);
            }
            D = gmin;
            const int owner = (j1 - 1) & 31, slot = (j1 - 1) >> 5;
            const int pnext = O(CS_PJ, slot, owner);
            const int unext = O(CS_UR, slot, owner);
            const int rnext = O(CS_RBR, slot, owner);
            if (lane == owner) S(CS_USED, slot) = D;
            j0 = j1;
            if (pnext == 0) { augmented = true; break; }
            ui0 = unext;
            rb = rnext;
        }
        if (!feasible || !augmented) { feasible = false; break; }
        // apply the potentials of this path (before the matching flips)
        const int uroot = w.u[i] + D;
        for (int t = 0; t < CPL; ++t) {
            const int ua = S(CS_USED, t);
            if (ua < 0) continue;
            const int d = D - ua;
            S(CS_PV, t) -= d;
            S(CS_UR, t) += d;
        }
        __syncwarp();
        // flip the path: column j takes the row (and its potential / offset) of way[j]
        int j = j0;
        for (int guard = 0; guard <= k && j != 0; ++guard) {
            const int owner = (j - 1) & 31, slot = (j - 1) >> 5;
            const int jp = O(CS_WAY, slot, owner);
            int np = i, nu = uroot, nr = w.rowb[i];
            if (jp != 0) {
                const int po = (jp - 1) & 31, ps = (jp - 1) >> 5;
                np = O(CS_PJ, ps, po);
                nu = O(CS_UR, ps, po);
                nr = O(CS_RBR, ps, po);
            }
            __syncwarp();
            if (lane == owner) { S(CS_PJ, slot) = np; S(CS_UR, slot) = nu; S(CS_RBR, slot) = nr; }
            __syncwarp();
            j = jp;
        }
        __syncwarp();
    }
    if (!__all_sync(kFull, feasible)) return false;
    // outputs and the warm state for the next call (original indices)
    for (int i = lane; i < m; i += 32)
        if (w.fcol[i] >= 0) { w.pi[i] = w.fcol[i]; w.match[w.fcol[i]] = i; }
    int lo = kIntInf;
    for (int t = 0; t < CPL; ++t) {
        if (lane + 1 + 32 * t > k) continue;
        const int col = S(CS_COL, t);
        const int r = w.rows[S(CS_PJ, t) - 1];
        w.pi[r] = col;
        w.match[col] = r;
        lo = min(lo, S(CS_PV, t));
    }
    lo = __reduce_min_sync(kFull, lo);
    if (lo >= kIntInf) lo = 0;
    bool sane = true;
    for (int t = 0; t < CPL; ++t) {
        if (lane + 1 + 32 * t > k) continue;
        const int v = S(CS_PV, t) - lo;
        w.colpot[S(CS_COL, t)] = v;
        sane = sane && v <= kPotLimit;
    }
    sane = __all_sync(kFull, sane);
    if (lane == 0) { w.scal[0] = sane ? 1 : 0; w.scal[1] = shift; }
    __syncwarp();
    return true;
}
// ---- the same integer Hungarian on a group of four warps (large orders).
// At orders above 128 the costs come from L2 and a Dijkstra step of one warp
// scans up to 16 columns per lane; on four warps (one per SM sub-partition)
// a lane scans a quarter of them, and the four warps' best keys meet in
// shared memory behind one named barrier per step. Group g is threads
// [128g, 128g+128) with named barrier 1+g; thread gt of the group owns the
// compacted columns gt+1, gt+129, ... (CPL per thread, k <= 128*CPL), its
// column state at cs[(a*CPL + t)*128 + gt] (colstate_bytes(4*CPL) bytes, the
// single-warp layout of 4*CPL columns per lane). The steps, the tie rule
// (lowest column) and the warm state are those of int_hungarian_warp_cs, so
// the assignment, the kept potentials and the matching are identical; every
// early return is group-uniform. All 128 threads of the group call it.
__device__ __forceinline__ void oracle_group_bar(int g) {
    asm volatile("bar.sync %0, 128;" :: "r"(1 + g) : "memory");
}

template <int CPL, int FACE>
__device__ bool int_hungarian_group_cs(const IHW& w, int* cs, int m, const int* costs, int shift,
                                       const uint8_t* code, bool restrict_same, int g) {
    constexpr int GT = 128, GW = 4;
    __shared__ int s_key[2][2][GW];   // [group][step parity][warp]: packed (slack, column) keys
    __shared__ int s_fbv[2][2][GW];   // the two-reduction path: slack and column per warp
    __shared__ int s_fbj[2][2][GW];
    __shared__ int s_red[2][GW];      // group min / and
    __shared__ int s_k[2];
    const int gt = (int)threadIdx.x - GT * g, lane = gt & 31, gw = gt >> 5;
    auto S = [&](int a, int t) -> int& { return cs[(a * CPL + t) * GT + gt]; };
    auto O = [&](int a, int t, int o) -> int& { return cs[(a * CPL + t) * GT + o]; };
    auto cost_at = [&](int e) -> int {
        const int c0 = costs[e];
        if constexpr (FACE == 2) return (c0 < kIntInf && (code[e] & kFaceIn)) ? -c0 : kIntInf;
        else if constexpr (FACE == 3) return packed_forward(c0);
        else if constexpr (FACE == 4) return packed_inface(c0);
        else return c0;
    };
    auto group_min = [&](int v) -> int {
        v = __reduce_min_sync(kFull, v);
        if (lane == 0) s_red[g][gw] = v;
        oracle_group_bar(g);
        int r = s_red[g][0];
#pragma unroll
        for (int q = 1; q < GW; ++q) r = min(r, s_red[g][q]);
        oracle_group_bar(g);
        return r;
    };
    auto group_all = [&](bool b) -> bool { return group_min(b ? 1 : 0) != 0; };
    int k;
    if (restrict_same && w.scal[2] > 0) {
        k = w.scal[2] - 1;
    } else {
        for (int i = gt; i < m; i += GT) { w.fcol[i] = -1; w.frow[i] = -1; }
        oracle_group_bar(g);
        bool ok = true;
        const int nn = m * m;
        for (int e = gt; e < nn; e += GT) {
            const uint8_t c = code[e];
            if (c & kBad) ok = false;
            const bool forced = (c & kForced) || (FACE != 0 && FACE != 3 && (c & kFaceOne));
            if (forced) {
                const int r = e / m, col = e - r * m;
                if (!(c & kAllowed)) ok = false;
                if (atomicCAS(&w.fcol[r], -1, col) != -1) ok = false;
                if (atomicCAS(&w.frow[col], -1, r) != -1) ok = false;
            }
        }
        if (!group_all(ok)) return false;
        if (gw == 0) {   // compaction in index order on the first warp
            const unsigned lt = (1u << lane) - 1u;
            int kr = 0, kc = 0;
            for (int base = 0; base < m; base += 32) {
                const int i = base + lane;
                const bool fr = i < m && w.fcol[i] < 0;
                const bool fc = i < m && w.frow[i] < 0;
                const unsigned mr = __ballot_sync(kFull, fr), mc = __ballot_sync(kFull, fc);
                if (fr) w.rows[kr + __popc(mr & lt)] = i;
                if (i < m) w.rowpos[i] = fr ? kr + __popc(mr & lt) + 1 : 0;
                if (fc) w.cols[kc + __popc(mc & lt)] = i;
                kr += __popc(mr);
                kc += __popc(mc);
            }
            if (lane == 0) s_k[g] = (kr != kc || kr > GT * CPL) ? -1 : kr;
        }
        oracle_group_bar(g);
        k = s_k[g];
        if (k < 0) return false;
        for (int i = gt + 1; i <= k; i += GT) w.rowb[i] = w.rows[i - 1] * m;
        if (gt == 0) w.scal[2] = k + 1;
        oracle_group_bar(g);
    }
    const bool warm = w.scal[0] != 0;
    const int dshift = shift - w.scal[1];
    for (int t = 0; t < CPL; ++t) {
        const int j = gt + 1 + GT * t;
        const bool valid = j <= k;
        const int col = valid ? w.cols[j - 1] : 0;
        long long v = 0;
        if (valid && warm) {
            v = w.colpot[col];
            if (dshift > 0) v = dshift >= 24 ? 0 : v * (1ll << dshift);
            else if (dshift < 0) v = -dshift >= 40 ? 0 : (v >> (-dshift));
            v = max(-kPotLimit, min(kPotLimit, v));
        }
        S(CS_COL, t) = col;
        S(CS_PV, t) = (int)v;
        S(CS_PJ, t) = 0;
        S(CS_UR, t) = 0;
        S(CS_RBR, t) = 0;
        if (valid) w.pvs[j] = (int)v;
    }
    oracle_group_bar(g);
    // row potentials u_i = min_j (c_ij - v_j), one row per thread
    bool rows_ok = true;
    for (int i = gt + 1; i <= k; i += GT) {
        const int rb = w.rowb[i];
        int best = kIntInf, barg = 0;
        int j = 1;
        for (; j + 7 <= k; j += 8) {
            int cc[8], pp[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) { cc[q] = cost_at(rb + w.cols[j - 1 + q]); pp[q] = w.pvs[j + q]; }
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (cc[q] < kIntInf && cc[q] - pp[q] < best) { best = cc[q] - pp[q]; barg = j + q; }
        }
        for (; j <= k; ++j) {
            const int c = cost_at(rb + w.cols[j - 1]);
            if (c < kIntInf && c - w.pvs[j] < best) { best = c - w.pvs[j]; barg = j; }
        }
        if (best >= kIntInf) rows_ok = false;
        w.u[i] = best;
        w.pinv[i - 1] = barg;   // a tight column of row i (pinv is free during the call)
        w.rmatch[i] = 0;
    }
    if (!group_all(rows_ok)) return false;
    // keep the previous matching where its edge is still allowed and tight
    if (warm) {
        for (int t = 0; t < CPL; ++t) {
            if (gt + 1 + GT * t > k) continue;
            const int col = S(CS_COL, t);
            const int r = w.match[col];
            if (r < 0 || r >= m) continue;
            const int i = w.rowpos[r];
            if (i <= 0) continue;
            const int c = cost_at(r * m + col);
            const int ui = w.u[i];
            if (c < kIntInf && c - ui - S(CS_PV, t) == 0) {
                S(CS_PJ, t) = i;
                S(CS_UR, t) = ui;
                S(CS_RBR, t) = w.rowb[i];
                w.rmatch[i] = 1;
            }
        }
    }
    oracle_group_bar(g);
    // greedy tight matching: every free row claims its tight column, the lowest
    // row wins a contested free column
    {
        int* claim = w.pi;   // per compacted column; pi is rewritten at the end
        for (int t = 0; t < CPL; ++t)
            if (gt + 1 + GT * t <= k) claim[gt + GT * t] = S(CS_PJ, t) ? 0 : 0x7fffffff;
        oracle_group_bar(g);
        for (int i = gt + 1; i <= k; i += GT)
            if (!w.rmatch[i]) atomicMin(&claim[w.pinv[i - 1] - 1], i);
        oracle_group_bar(g);
        for (int t = 0; t < CPL; ++t) {
            if (gt + 1 + GT * t > k || S(CS_PJ, t)) continue;
            const int r = claim[gt + GT * t];
            if (r != 0x7fffffff) {
                S(CS_PJ, t) = r;
                S(CS_UR, t) = w.u[r];
                S(CS_RBR, t) = w.rowb[r];
                w.rmatch[r] = 1;
            }
        }
        oracle_group_bar(g);
    }
    bool feasible = true;
    int par = 0;
    for (int i = 1; i <= k && feasible; ++i) {
        if (w.rmatch[i]) continue;
        for (int t = 0; t < CPL; ++t) {
            S(CS_MRAW, t) = kIntInf;
            S(CS_WAY, t) = 0;
            S(CS_USED, t) = -1;
        }
        int j0 = 0, D = 0;
        int ui0 = w.u[i], rb = w.rowb[i];
        bool augmented = false;
        for (int step = 0; step <= k; ++step) {
            int bv = kIntInf, bj = 0x7fffffff;
            int cv[CPL];
#pragma unroll
            for (int t = 0; t < CPL; ++t) cv[t] = cost_at(rb + S(CS_COL, t));
#pragma unroll
            for (int t = 0; t < CPL; ++t) {
                const bool live = gt + 1 + GT * t <= k && S(CS_USED, t) < 0;
                const int c = cv[t];
                int mr = S(CS_MRAW, t);
                if (live && c < kIntInf) {
                    const int cur = c - ui0 - S(CS_PV, t) + D;
                    if (cur < mr) { mr = cur; S(CS_MRAW, t) = cur; S(CS_WAY, t) = j0; }
                }
                if (live && mr < bv) { bv = mr; bj = gt + 1 + GT * t; }
            }
            const int key = bv < kPackLimit ? (bv << 10) | bj : 0x7fffffff;
            const int wk = __reduce_min_sync(kFull, key);
            if (lane == 0) s_key[g][par][gw] = wk;
            // the warp's candidate column's matched row holds the next step's
            // costs if the candidate wins: start bringing it toward the SM (one
            // 128-byte line per lane) while the warps meet
            if (wk != 0x7fffffff) {
                const int wj = wk & 1023;
                const int wo = (wj - 1) & (GT - 1), ws = (wj - 1) >> 7;
                if (O(CS_PJ, ws, wo) != 0 && lane * 32 < m)
                    asm volatile("prefetch.global.L1 [%0];" :: "l"(costs + O(CS_RBR, ws, wo) + lane * 32));
            }
            oracle_group_bar(g);
            int kmin = s_key[g][par][0];
#pragma unroll
            for (int q = 1; q < GW; ++q) kmin = min(kmin, s_key[g][par][q]);
            int gmin, j1;
            if (kmin != 0x7fffffff) {
                gmin = kmin >> 10;
                j1 = kmin & 1023;
            } else {
                // every slack is large: minimum slack, then the lowest column at it
                const int wb = __reduce_min_sync(kFull, bv);
                const int wj = __reduce_min_sync(kFull, bv == wb ? bj : 0x7fffffff);
                if (lane == 0) { s_fbv[g][par][gw] = wb; s_fbj[g][par][gw] = wj; }
                oracle_group_bar(g);
                gmin = s_fbv[g][par][0];
                j1 = s_fbj[g][par][0];
#pragma unroll
                for (int q = 1; q < GW; ++q) {
                    const int vq = s_fbv[g][par][q], jq = s_fbj[g][par][q];
                    if (vq < gmin || (vq == gmin && jq < j1)) { gmin = vq; j1 = jq; }
                }
                if (gmin >= kIntInf) { feasible = false; break; }
            }
            par ^= 1;
            D = gmin;
            const int owner = (j1 - 1) & (GT - 1), slot = (j1 - 1) >> 7;
            const int pnext = O(CS_PJ, slot, owner);
            const int unext = O(CS_UR, slot, owner);
            const int rnext = O(CS_RBR, slot, owner);
            if (gt == owner) S(CS_USED, slot) = D;
            j0 = j1;
            if (pnext == 0) { augmented = true; break; }
            ui0 = unext;
            rb = rnext;
        }
        if (!feasible || !augmented) { feasible = false; break; }
        // apply the potentials of this path (before the matching flips)
        const int uroot = w.u[i] + D;
        for (int t = 0; t < CPL; ++t) {
            const int ua = S(CS_USED, t);
            if (ua < 0) continue;
            const int d = D - ua;
            S(CS_PV, t) -= d;
            S(CS_UR, t) += d;
        }
        oracle_group_bar(g);
        // flip the path on one thread: column j takes the row (and its
        // potential / offset) of way[j], from the path's end back to its root
        if (gt == 0) {
            int j = j0;
            for (int guard = 0; guard <= k && j != 0; ++guard) {
                const int owner = (j - 1) & (GT - 1), slot = (j - 1) >> 7;
                const int jp = O(CS_WAY, slot, owner);
                int np = i, nu = uroot, nr = w.rowb[i];
                if (jp != 0) {
                    const int po = (jp - 1) & (GT - 1), ps = (jp - 1) >> 7;
                    np = O(CS_PJ, ps, po);
                    nu = O(CS_UR, ps, po);
                    nr = O(CS_RBR, ps, po);
                }
                O(CS_PJ, slot, owner) = np;
                O(CS_UR, slot, owner) = nu;
                O(CS_RBR, slot, owner) = nr;
                j = jp;
            }
        }
        oracle_group_bar(g);
    }
    if (!feasible) return false;
    // outputs and the warm state for the next call (original indices)
    for (int i = gt; i < m; i += GT)
        if (w.fcol[i] >= 0) { w.pi[i] = w.fcol[i]; w.match[w.fcol[i]] = i; }
    int lo = kIntInf;
    for (int t = 0; t < CPL; ++t) {
        if (gt + 1 + GT * t > k) continue;
        const int col = S(CS_COL, t);
        const int r = w.rows[S(CS_PJ, t) - 1];
        w.pi[r] = col;
        w.match[col] = r;
        lo = min(lo, S(CS_PV, t));
    }
    lo = group_min(lo);
    if (lo >= kIntInf) lo = 0;
    bool sane = true;
    for (int t = 0; t < CPL; ++t) {
        if (gt + 1 + GT * t > k) continue;
        const int v = S(CS_PV, t) - lo;
        w.colpot[S(CS_COL, t)] = v;
        sane = sane && v <= kPotLimit;
    }
    sane = group_all(sane);
    if (gt == 0) { w.scal[0] = sane ? 1 : 0; w.scal[1] = shift; }
    oracle_group_bar(g);
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
// For m % 4 == 0 every thread computes strips of four consecutive outputs: one
// scalar and one float4 load per operand pair feed four FMAs (rows of m floats
// stay 16-byte aligned).
static __device__ void grad_f32(int m, float two_s, const float* A, const float* B, const float* Bt, const float* X,
                         float* R, float* G) {
    const int n = m * m;
    if ((m & 3) == 0) {
        const int strips = n >> 2, sm = m >> 2;
        for (int s = threadIdx.x; s < strips; s += kThreads) {
            const int i = s / sm, j = (s - (s / sm) * sm) << 2;
            float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int k = 0; k < m; ++k) {
                const float a = A[i * m + k], xi = -X[i * m + k];
                const float4 xk = *reinterpret_cast<const float4*>(X + k * m + j);
                const float4 bk = *reinterpret_cast<const float4*>(B + k * m + j);
                r.x = fmaf(xi, bk.x, fmaf(a, xk.x, r.x));
                r.y = fmaf(xi, bk.y, fmaf(a, xk.y, r.y));
                r.z = fmaf(xi, bk.z, fmaf(a, xk.z, r.z));
                r.w = fmaf(xi, bk.w, fmaf(a, xk.w, r.w));
            }
            *reinterpret_cast<float4*>(R + i * m + j) = r;
        }
        __syncthreads();
        for (int s = threadIdx.x; s < strips; s += kThreads) {
            const int p = s / sm, q = (s - (s / sm) * sm) << 2;
            float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int r = 0; r < m; ++r) {
                const float a = A[r * m + p];
                const float4 rr = *reinterpret_cast<const float4*>(R + r * m + q);
                g.x = fmaf(a, rr.x, g.x);
                g.y = fmaf(a, rr.y, g.y);
                g.z = fmaf(a, rr.z, g.z);
                g.w = fmaf(a, rr.w, g.w);
            }
            for (int c = 0; c < m; ++c) {
                const float rp = -R[p * m + c];
                const float4 bt = *reinterpret_cast<const float4*>(Bt + c * m + q);
                g.x = fmaf(rp, bt.x, g.x);
                g.y = fmaf(rp, bt.y, g.y);
                g.z = fmaf(rp, bt.z, g.z);
                g.w = fmaf(rp, bt.w, g.w);
            }
            *reinterpret_cast<float4*>(G + p * m + q) =
                make_float4(two_s * g.x, two_s * g.y, two_s * g.z, two_s * g.w);
        }
        __syncthreads();
        return;
    }
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
