// cluster.cuh -- the large-order mixed relaxation on a thread-block cluster:
// four CTAs per node, each holding a slice of the integer oracle costs in its
// own shared memory, the Dijkstra steps of the assignment oracles split across
// the four and reduced through distributed shared memory. Included by
// relax_impl.cuh.
//
// Why. At Birkhoff orders above ~256 one CTA cannot hold the m x m integer
// costs (640 KB at order 400); the one-CTA kernel reads a cost row from L2 at
// every Dijkstra step, a dependent chain of ~2,700 cycles per step. Four CTAs
// hold 100 columns each (160 KB of shared memory apiece), so a step scans
// 4 columns per lane from shared memory and exchanges one 32-byte record per
// CTA. This replaces the reference's MultiBlock backend (K CTAs per node
// under a cooperative launch with device-scope atomic barriers,
// include/gpuboscia/multiblock.cuh:36-103, device_resident_solver.cuh:662-757):
// here the node's CTAs are a hardware cluster, talk through DSMEM stores and
// mbarriers with cluster scope, and every wait is bounded.
//
// Roles. CTA 0 of the cluster (the leader) runs the node's relaxation as the
// one-CTA kernel does, except that the two integer oracles run on warp 0
// (forward) and warp 1 (in-face) of every CTA of the cluster at once. Before
// an oracle call the leader posts a command (cost scale, restriction flags)
// in its shared memory and arrives on each helper's "go" barrier; every CTA
// then scales its slice of the FP32 gradient into packed integer costs
// (2c + face bit) and runs its share of the oracles. After the last iteration
// the leader posts an exit; the helpers acknowledge it on the leader's "done"
// barrier and return, and the leader computes the FP64 certificate alone.
//
// The split oracle computes exactly what int_hungarian_warp_cs computes on
// one warp: the same compacted rows and columns, warm-started potentials,
// greedy tight matching (lowest row wins a column), shortest augmenting paths
// with ties to the lowest compacted column, and the same normalised warm
// state, so the two launch shapes give bit-identical relaxations.
#pragma once

namespace gbx {

constexpr long kClSpin = 1l << 22;      // try_wait rounds of an exchange / phase wait
constexpr long kClSpinGo = 1l << 24;    // rounds (each with a short sleep) of a helper waiting for a command

// ---- PTX helpers ----------------------------------------------------------
__device__ __forceinline__ unsigned cl_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cl_saddr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
// the address of this CTA's object p in CTA `rank`'s shared memory (same layout in every CTA)
__device__ __forceinline__ unsigned cl_map(const void* p, unsigned rank) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(cl_saddr(p)), "r"(rank));
    return r;
}
__device__ __forceinline__ void cl_st(unsigned a, int v) {
    asm volatile("st.shared::cluster.s32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void cl_st_u8(unsigned a, int v) {
    asm volatile("st.shared::cluster.u8 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void cl_st4(unsigned a, int x, int y, int z, int w) {
    asm volatile("st.shared::cluster.v4.s32 [%0], {%1, %2, %3, %4};" ::"r"(a), "r"(x), "r"(y), "r"(z), "r"(w)
                 : "memory");
}
__device__ __forceinline__ int cl_ld(unsigned a) {
    int v;
    asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
    return v;
}
__device__ __forceinline__ void cl_atom_min(unsigned a, int v) {
    asm volatile("red.shared::cluster.min.s32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void cl_fence() { asm volatile("fence.acq_rel.cluster;" ::: "memory"); }
// release store of an event counter into another CTA's shared memory
__device__ __forceinline__ void cl_st_release(unsigned a, int v) {
    asm volatile("st.release.cluster.shared::cluster.s32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ int cl_ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.cluster.shared::cta.s32 %0, [%1];" : "=r"(v) : "r"(cl_saddr(p)) : "memory");
    return v;
}
__device__ __forceinline__ void cl_bar_init(uint64_t* b, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(cl_saddr(b)), "r"(count) : "memory");
}
// arrive (release, cluster scope) on the barrier at cluster address a
__device__ __forceinline__ void cl_arrive(unsigned a) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(a) : "memory");
}
// bounded wait (acquire, cluster scope) for the phase of parity `par` of a local barrier
__device__ __forceinline__ bool cl_wait(uint64_t* b, unsigned par, long limit, bool sleep) {
    const unsigned a = cl_saddr(b);
    for (long i = 0; i < limit; ++i) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(par)
            : "memory");
        if (done) return true;
        if (sleep) __nanosleep(256);
    }
    return false;
}
__device__ __forceinline__ void cl_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// ---- the per-oracle workspace of one CTA -----------------------------------
// column state of the CTA's slice: [CS_COUNT][kClCpl][32]; CS_RBR holds the
// matched row's index (the cost slice is addressed by row)
struct CHW {
    int *u, *rows, *rowpos, *fcol, *frow, *lmin, *larg, *logpos;   // [m + 1]
    int *lw, *lp, *lu, *lr, *ld;                                   // per-step log [m + 1]
    int *claim, *colpot, *match;                                   // [128], by slice position
    int* jst;                                                      // [16]: first compacted column of each CTA
    int* cs;                                                       // column state
    int* rec;                                                      // [2][kClCtas][8] exchange records
    int* scal;                                                     // [16]
    int* flg;                                                      // [2][kClCtas] event counters per sender
    uint8_t* rmatch;                                               // [m + 1]
};
__device__ inline CHW chw_at(unsigned char* base, int m) {
    CHW w;
    int* p = reinterpret_cast<int*>(base);
    const int M = m + 1;
    w.u = p; w.rows = p + M; w.rowpos = p + 2 * M; w.fcol = p + 3 * M; w.frow = p + 4 * M; w.lmin = p + 5 * M;
    w.larg = p + 6 * M; w.logpos = p + 7 * M; w.lw = p + 8 * M; w.lp = p + 9 * M; w.lu = p + 10 * M;
    w.lr = p + 11 * M; w.ld = p + 12 * M;
    size_t o = align16((size_t)13 * M * sizeof(int));
    w.claim = reinterpret_cast<int*>(base + o);
    w.colpot = w.claim + 128;
    w.match = w.claim + 256;
    o += align16(3 * 128 * sizeof(int));
    w.jst = reinterpret_cast<int*>(base + o);
    o += 16 * sizeof(int);
    w.cs = reinterpret_cast<int*>(base + o);
    o += align16((size_t)CS_COUNT * kClCpl * 32 * sizeof(int));
    w.rec = reinterpret_cast<int*>(base + o);
    o += align16(2 * kClCtas * 8 * sizeof(int));
    w.scal = reinterpret_cast<int*>(base + o);
    o += 16 * sizeof(int);
    w.flg = reinterpret_cast<int*>(base + o);
    o += 2 * kClCtas * sizeof(int);
    w.rmatch = base + o;
    return w;
}

// Per node, before the cluster barrier that opens the launch (thread 0 of each
// CTA): barriers and a cold warm state.
__device__ inline void chw_reset(const CHW& w) {
    for (int i = 0; i < 16; ++i) w.scal[i] = 0;
    for (int q = 0; q < 128; ++q) { w.colpot[q] = 0; w.match[q] = -1; }
    for (int q = 0; q < 2 * kClCtas; ++q) w.flg[q] = 0;
}

// The CTA's slice of packed integer costs (all threads): for original columns
// base .. base+S-1, 2 * round(g * 2^shift) + (edge on the iterate's face) for
// allowed edges, kIntInf otherwise -- the forward costs of the one-CTA kernel,
// and (face bit) its in-face costs.
__device__ inline void cl_stage(int* slice, int S, int base, int m, const float* gf, const uint8_t* code,
                                int shift) {
    const int total = m * S;
    for (int e = threadIdx.x; e < total; e += kThreads) {
        const int r = e / S, c = base + (e - r * S);
        int v = kIntInf;
        if (c < m) {
            const uint8_t cd = code[r * m + c];
            if (cd & kAllowed) {
                const int ci = __float2int_rn(scalbnf(gf[r * m + c], shift));
                v = 2 * ci + ((cd & kFaceIn) ? 1 : 0);
            }
        }
        slice[e] = v;
    }
}

// One oracle on one warp of every CTA of the cluster (FACE 0: forward costs;
// FACE 2: in-face costs -- negated forward costs on the iterate's face --
// and the face's unit entries forced). Writes the row->column map into the
// leader's `pi` (the same offset in every CTA's shared memory). Returns a
// warp-uniform success flag, equal in every CTA unless a wait gave up (*err).
template <int FACE>
__device__ bool cl_hungarian(const CHW& w, const int* slice, int S, int m, int shift, const uint8_t* code,
                             bool restrict_same, int* pi, int* err) {
    constexpr int CPL = kClCpl;
    constexpr int C = kClCtas;
    const int lane = threadIdx.x & 31;
    const unsigned rank = cl_rank();
    const int base = (int)rank * S;
    auto SS = [&](int a, int t) -> int& { return w.cs[(a * CPL + t) * 32 + lane]; };
    auto OO = [&](int a, int q) -> int { return w.cs[(a * CPL + (q >> 5)) * 32 + (q & 31)]; };
    auto cost_at = [&](int row, int col) -> int {
        const int v = slice[row * S + (col - base)];
        if (v >= kIntInf) return kIntInf;
        if constexpr (FACE == 2) return (v & 1) ? -(v >> 1) : kIntInf;
        else return v >> 1;
    };
    if (*err) return false;
    // Events between the CTAs' oracle warps: the sender release-stores its
    // event count (kind 0: step exchange, kind 1: phase) into every CTA's slot
    // for it; a receiver waits (bounded) until every sender's count reached
    // the event. Counts only grow, so a late store never miscounts.
    auto signal = [&](int kind, int e) {
        if (lane == 0)
            for (int r = 0; r < C; ++r) cl_st_release(cl_map(&w.flg[kind * C + (int)rank], r), e);
    };
    auto await = [&](int kind, int e) -> bool {
        bool ok = true;
        for (int r = 0; r < C && ok; ++r) {
            const int* f = &w.flg[kind * C + r];
            for (long it = 0; cl_ld_acquire(f) < e; ++it)
                if (it >= kClSpin) { ok = false; break; }
        }
        ok = __all_sync(kFull, ok);
        if (!ok && lane == 0) *err = 1;
        __syncwarp();
        return ok;
    };
    // all CTAs' oracle warps meet: stores before it are visible after it
    auto phase = [&]() -> bool {
        cl_fence();
        __syncwarp();
        const int e = w.scal[5] + 1;
        __syncwarp();
        if (lane == 0) w.scal[5] = e;
        signal(1, e);
        return await(1, e);
    };
    const unsigned lt = (1u << lane) - 1u;
    int k, jlo, kl;
    if (restrict_same && w.scal[2] > 0) {
        k = w.scal[2] - 1;
        jlo = w.scal[3];
        kl = w.scal[4];
    } else {
        for (int i = lane; i < m; i += 32) { w.fcol[i] = -1; w.frow[i] = -1; }
        __syncwarp();
        bool ok = true;
        const int nn = m * m;
        for (int e = lane; e < nn; e += 32) {
            const uint8_t c = code[e];
            if (c & kBad) ok = false;
            const bool forced = (c & kForced) || (FACE != 0 && (c & kFaceOne));
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
        // compacted rows (all) and columns; this CTA's columns are the free
        // columns of its slice, a contiguous range of compacted indices
        k = 0;
        int kc = 0;
        jlo = 0;
        kl = 0;
        for (int b0 = 0; b0 < m; b0 += 32) {
            const int i = b0 + lane;
            const bool fr = i < m && w.fcol[i] < 0;
            const bool fc = i < m && w.frow[i] < 0;
            const unsigned mr = __ballot_sync(kFull, fr), mc = __ballot_sync(kFull, fc);
            const int jbefore = kc + __popc(mc & lt);   // free columns before i
            if (fr) w.rows[k + __popc(mr & lt)] = i;
            if (i < m) w.rowpos[i] = fr ? k + __popc(mr & lt) + 1 : 0;
            if (i < m && i % S == 0 && i / S < C) w.jst[i / S] = jbefore + 1;
            k += __popc(mr);
            kc += __popc(mc);
        }
        if (k != kc) return false;
        if (lane == 0)
            for (int r = 0; r < C; ++r)
                if (r * S >= m) w.jst[r] = kc + 1;
        if (lane == 0) w.jst[C] = kc + 1;
        __syncwarp();
        jlo = w.jst[rank];
        kl = w.jst[rank + 1] - jlo;
        if (kl < 0 || kl > 32 * CPL) return false;   // equal in every CTA: slices are at most 128 columns
        // this slice's free columns in order: slot q holds compacted column jlo + q
        {
            int q0 = 0;
            for (int b0 = base; b0 < base + S && b0 < m; b0 += 32) {
                const int i = b0 + lane;
                const bool fc = i < m && i < base + S && w.frow[i] < 0;
                const unsigned mc = __ballot_sync(kFull, fc);
                if (fc) {
                    const int q = q0 + __popc(mc & lt);
                    w.cs[(CS_COL * CPL + (q >> 5)) * 32 + (q & 31)] = i;
                }
                q0 += __popc(mc);
            }
        }
        if (lane == 0) { w.scal[2] = k + 1; w.scal[3] = jlo; w.scal[4] = kl; }
        __syncwarp();
    }
    const bool warm = w.scal[0] != 0;
    const int dshift = shift - w.scal[1];
    for (int t = 0; t < CPL; ++t) {
        const int q = lane + 32 * t;
        const bool valid = q < kl;
        if (!valid) SS(CS_COL, t) = base;   // a column of the slice: its cost loads stay in bounds
        const int col = SS(CS_COL, t);
        long long v = 0;
        if (valid && warm) {
            v = w.colpot[col - base];
            if (dshift > 0) v = dshift >= 24 ? 0 : v * (1ll << dshift);
            else if (dshift < 0) v = -dshift >= 40 ? 0 : (v >> (-dshift));
            v = max(-kPotLimit, min(kPotLimit, v));
        }
        SS(CS_PV, t) = (int)v;
        SS(CS_PJ, t) = 0;
        SS(CS_UR, t) = 0;
        SS(CS_RBR, t) = 0;
    }
    __syncwarp();
    // row potentials u_i = min_j (c_ij - v_j): this slice's minima, then the cluster's
    for (int i = lane + 1; i <= k; i += 32) {
        const int row = w.rows[i - 1];
        int best = kIntInf, barg = 0;
        for (int q = 0; q < kl; ++q) {
            const int c = cost_at(row, OO(CS_COL, q));
            const int p = OO(CS_PV, q);
            if (c < kIntInf && c - p < best) { best = c - p; barg = jlo + q; }
        }
        w.lmin[i] = best;
        w.larg[i] = barg;
        w.rmatch[i] = 0;
    }
    if (!phase()) return false;
    bool rows_ok = true;
    for (int i = lane + 1; i <= k; i += 32) {
        int best = kIntInf, bj = 0x7fffffff;
        for (int r = 0; r < C; ++r) {
            const int v = cl_ld(cl_map(&w.lmin[i], r));
            const int j = cl_ld(cl_map(&w.larg[i], r));
            if (v < best || (v == best && v < kIntInf && j < bj)) { best = v; bj = j; }
        }
        if (best >= kIntInf) rows_ok = false;
        w.u[i] = best;
        w.logpos[i] = bj;   // a tight column of row i (the log is free until the paths)
    }
    if (!__all_sync(kFull, rows_ok)) return false;
    __syncwarp();
    // keep the previous matching where its edge is still allowed and tight
    if (warm) {
        for (int t = 0; t < CPL; ++t) {
            if (lane + 32 * t >= kl) continue;
            const int col = SS(CS_COL, t);
            const int r = w.match[col - base];
            if (r < 0 || r >= m) continue;
            const int i = w.rowpos[r];
            if (i <= 0) continue;
            const int c = cost_at(r, col);
            const int ui = w.u[i];
            if (c < kIntInf && c - ui - SS(CS_PV, t) == 0) {
                SS(CS_PJ, t) = i;
                SS(CS_UR, t) = ui;
                SS(CS_RBR, t) = r;
                for (int rr = 0; rr < C; ++rr) cl_st_u8(cl_map(&w.rmatch[i], rr), 1);
            }
        }
    }
    for (int t = 0; t < CPL; ++t)
        if (lane + 32 * t < kl) w.claim[lane + 32 * t] = SS(CS_PJ, t) ? 0 : 0x7fffffff;
    if (!phase()) return false;
    // greedy tight matching: every free row claims its tight column at the
    // column's CTA, the lowest row wins (rows split among the CTAs)
    for (int i = lane + 1; i <= k; i += 32) {
        if ((i - 1) % C != (int)rank || w.rmatch[i]) continue;
        const int j = w.logpos[i];
        int owner = 0;
        for (int r = 1; r < C; ++r)
            if (w.jst[r] <= j) owner = r;
        cl_atom_min(cl_map(&w.claim[j - w.jst[owner]], owner), i);
    }
    if (!phase()) return false;
    for (int t = 0; t < CPL; ++t) {
        if (lane + 32 * t >= kl || SS(CS_PJ, t)) continue;
        const int r = w.claim[lane + 32 * t];
        if (r != 0x7fffffff) {
            SS(CS_PJ, t) = r;
            SS(CS_UR, t) = w.u[r];
            SS(CS_RBR, t) = w.rows[r - 1];
            for (int rr = 0; rr < C; ++rr) cl_st_u8(cl_map(&w.rmatch[r], rr), 1);
        }
    }
    if (!phase()) return false;
    // shortest augmenting paths, one exchange of the CTAs' best slacks per step
    // (event e of kind 0 carries records in buffer e & 1)
    bool feasible = true;
    for (int i = 1; i <= k && feasible; ++i) {
        if (w.rmatch[i]) continue;
        for (int t = 0; t < CPL; ++t) {
            SS(CS_MRAW, t) = kIntInf;
            SS(CS_WAY, t) = 0;
            SS(CS_USED, t) = -1;
        }
        int j0 = 0, D = 0;
        int ui0 = w.u[i], row = w.rows[i - 1];
        bool augmented = false;
        for (int step = 0; step <= k; ++step) {
            int cv[CPL];
#pragma unroll
            for (int t = 0; t < CPL; ++t) cv[t] = cost_at(row, SS(CS_COL, t));
            int bv = kIntInf, bq = 0x7fffffff;
#pragma unroll
            for (int t = 0; t < CPL; ++t) {
                const int q = lane + 32 * t;
                const bool live = q < kl && SS(CS_USED, t) < 0;
                const int c = cv[t];
                int mr = SS(CS_MRAW, t);
                if (live && c < kIntInf) {
                    const int cur = c - ui0 - SS(CS_PV, t) + D;
                    if (cur < mr) { mr = cur; SS(CS_MRAW, t) = cur; SS(CS_WAY, t) = j0; }
                }
                if (live && mr < bv) { bv = mr; bq = q; }
            }
            __syncwarp();   // the scan's slack / predecessor writes, before lane 0 reads the winner's
            const int gl = __reduce_min_sync(kFull, bv);
            const int qm = __reduce_min_sync(kFull, bv == gl ? bq : 0x7fffffff);
            const int e = w.scal[6] + 1;
            const int p = e & 1;
            __syncwarp();
            if (lane == 0) w.scal[6] = e;
            if (lane == 0) {
                int jc = 0x7fffffff, pn = 0, un = 0, rn = 0, wn = 0;
                if (gl < kIntInf && qm < kl) {
                    jc = jlo + qm;
                    pn = OO(CS_PJ, qm);
                    un = OO(CS_UR, qm);
                    rn = OO(CS_RBR, qm);
                    wn = OO(CS_WAY, qm);
                }
                int* my = w.rec + (p * C + (int)rank) * 8;
                for (int r = 0; r < C; ++r) {
                    cl_st4(cl_map(my, r), gl, jc, pn, un);
                    cl_st4(cl_map(my + 4, r), rn, wn, 0, 0);
                }
            }
            signal(0, e);   // (lane 0: its record stores precede the release)
            if (!await(0, e)) return false;
            int gmin = kIntInf, j1 = 0x7fffffff, ob = 0;
            for (int r = 0; r < C; ++r) {
                const int* rc = w.rec + (p * C + r) * 8;
                const int v = rc[0], j = rc[1];
                if (v < gmin || (v == gmin && j < j1)) { gmin = v; j1 = j; ob = r; }
            }
            if (gmin >= kIntInf) { feasible = false; break; }
            const int* rw = w.rec + (p * C + ob) * 8;
            const int pnext = rw[2], unext = rw[3], rnext = rw[4], wnext = rw[5];
            __syncwarp();
            D = gmin;
            if (ob == (int)rank) {
                const int q1 = j1 - jlo;
                if (lane == (q1 & 31)) SS(CS_USED, q1 >> 5) = D;
            }
            if (lane == 0) {
                w.lw[step] = wnext;
                w.lp[step] = pnext;
                w.lu[step] = unext;
                w.lr[step] = rnext;
                w.ld[step] = D;
                w.logpos[j1] = step;
            }
            __syncwarp();
            j0 = j1;
            if (pnext == 0) { augmented = true; break; }
            ui0 = unext;
            row = rnext;
        }
        if (!feasible || !augmented) { feasible = false; break; }
        // potentials of this path (before the matching flips)
        const int uroot = w.u[i] + D;
        for (int t = 0; t < CPL; ++t) {
            const int ua = SS(CS_USED, t);
            if (ua < 0) continue;
            const int d = D - ua;
            SS(CS_PV, t) -= d;
            SS(CS_UR, t) += d;
        }
        __syncwarp();
        // flip the path from the step log: column j takes the row (potential
        // after this path's update, index) its predecessor held when it was reached
        int j = j0;
        for (int guard = 0; guard <= k && j != 0; ++guard) {
            const int s = w.logpos[j];
            const int jp = w.lw[s];
            int np = i, nu = uroot, nr = w.rows[i - 1];
            if (jp != 0) {
                const int sp = w.logpos[jp];
                np = w.lp[sp];
                nu = w.lu[sp] + (D - w.ld[sp]);
                nr = w.lr[sp];
            }
            if (j >= jlo && j < jlo + kl) {
                const int q = j - jlo;
                if (lane == (q & 31)) {
                    SS(CS_PJ, q >> 5) = np;
                    SS(CS_UR, q >> 5) = nu;
                    SS(CS_RBR, q >> 5) = nr;
                }
            }
            j = jp;
        }
        __syncwarp();
    }
    if (!__all_sync(kFull, feasible)) return false;
    // outputs: the leader's row->column map; the warm state of this slice
    for (int c = base + lane; c < base + S && c < m; c += 32) w.match[c - base] = -1;
    __syncwarp();
    for (int i = lane; i < m; i += 32) {
        const int fc = w.fcol[i];
        if (fc < 0) continue;
        if (rank == 0) pi[i] = fc;
        if (fc >= base && fc < base + S) w.match[fc - base] = i;
    }
    int lo = kIntInf;
    for (int t = 0; t < CPL; ++t) {
        if (lane + 32 * t >= kl) continue;
        const int col = SS(CS_COL, t);
        const int r = w.rows[SS(CS_PJ, t) - 1];
        cl_st(cl_map(&pi[r], 0), col);
        w.match[col - base] = r;
        lo = min(lo, SS(CS_PV, t));
    }
    lo = __reduce_min_sync(kFull, lo);
    if (lane == 0)
        for (int r = 0; r < C; ++r) cl_st(cl_map(&w.scal[8 + (int)rank], r), lo);
    if (!phase()) return false;
    int glo = kIntInf;
    for (int r = 0; r < C; ++r) glo = min(glo, w.scal[8 + r]);
    if (glo >= kIntInf) glo = 0;
    bool sane = true;
    for (int t = 0; t < CPL; ++t) {
        if (lane + 32 * t >= kl) continue;
        const int v = SS(CS_PV, t) - glo;
        w.colpot[SS(CS_COL, t) - base] = v;
        sane = sane && v <= kPotLimit;
    }
    sane = __all_sync(kFull, sane);
    if (lane == 0)
        for (int r = 0; r < C; ++r) cl_st(cl_map(&w.scal[12 + (int)rank], r), sane ? 1 : 0);
    if (!phase()) return false;
    bool all_sane = true;
    for (int r = 0; r < C; ++r) all_sane = all_sane && w.scal[12 + r] != 0;
    if (lane == 0) { w.scal[0] = all_sane ? 1 : 0; w.scal[1] = shift; }
    __syncwarp();
    return true;
}

// The leader's exit command (all threads of the leader CTA; idempotent): the
// helpers acknowledge it on the leader's done barrier and return, after which
// no CTA of the cluster touches another's shared memory.
__device__ inline void cl_release(ClCtl* ctl) {
    __syncthreads();
    if (threadIdx.x == 0 && !ctl->released) {
        ctl->cmd[0] = CL_EXIT;
        cl_fence();
        for (int r = 1; r < kClCtas; ++r) cl_arrive(cl_map(&ctl->bar_go, (unsigned)r));
        if (!cl_wait(&ctl->bar_done, 0, kClSpinGo, true)) ctl->err = 1;
        ctl->released = 1;
    }
    __syncthreads();
}

// A helper CTA of node `node`: waits for the leader's commands, stages its
// slice of the costs and runs its share of the oracles, until the exit.
__device__ inline void cl_helper(const Params& P, int node, unsigned char* dsm) {
    const Layout& L = P.L;
    const int m = P.obj.order, n = P.obj.n, S = L.cl_cols;
    ClCtl* ctl = reinterpret_cast<ClCtl*>(dsm + L.sm_cl);
    int* slice = reinterpret_cast<int*>(dsm + L.sm_slice);
    int* lpi = reinterpret_cast<int*>(dsm + L.sm_lpi);
    unsigned char* mx = P.mixed + (size_t)node * L.mixed_node_bytes;
    const float* gf = reinterpret_cast<const float*>(mx) + n;
    const uint8_t* code = mx + L.mx_code_off;
    const int base = (int)cl_rank() * S;
    __shared__ int s_cmd[4];
    unsigned par = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            const bool ok = cl_wait(&ctl->bar_go, par, kClSpinGo, true);
            par ^= 1u;
            if (ok) {
                for (int q = 0; q < 4; ++q) s_cmd[q] = cl_ld(cl_map(&ctl->cmd[q], 0));
            } else {
                s_cmd[0] = CL_EXIT;
                ctl->err = 1;
            }
        }
        __syncthreads();
        if (s_cmd[0] != CL_ORACLE) {
            if (threadIdx.x == 0) {
                cl_fence();
                cl_arrive(cl_map(&ctl->bar_done, 0));
            }
            return;
        }
        const int shift = s_cmd[1];
        cl_stage(slice, S, base, m, gf, code, shift);
        __syncthreads();
        const int wid = threadIdx.x >> 5;
        if (wid == 0)
            cl_hungarian<0>(chw_at(dsm + L.sm_chw, m), slice, S, m, shift, code, true, lpi, &ctl->err);
        else if (wid == 1 && s_cmd[3])
            cl_hungarian<2>(chw_at(dsm + L.sm_chw + L.chw_bytes, m), slice, S, m, shift, code, s_cmd[2] != 0,
                            lpi + 2 * m, &ctl->err);
        __syncthreads();
    }
}

}  // namespace gbx
