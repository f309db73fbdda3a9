// user_relax.cuh -- node relaxations for user-written device objectives.
//
// The precompiled library relaxes the built-in objective kinds. A program
// whose objective is its own device struct -- the reference's extension point
// (include/gpuboscia/device_resident_solver.cuh:8-34: n_vars, block_threads,
// shared_bytes, prepare_block, grad, value_local, and optionally
// supports_quadratic_exact with quadratic_curvature_local), such as the graph
// isomorphism objective of examples/main.cu:131-181 -- includes this header
// in a translation unit compiled by nvcc. The relaxation then runs as a
// template kernel compiled in that unit, over the built-in LMO kinds (box,
// bounded and equality simplex, Birkhoff), with the same iteration as the
// library's FP64 kernel: the start vertex of the direction -1 - j/(n+1), FW or
// DICG steps, the five line searches, vertex scoring, the incumbent cutoff,
// and the FP64 certificate and rounding heuristic at the returned iterate
// (drs_fw_relax_node, device_resident_solver.cuh:337-629).
//
// Layout: one CTA per node of min(round32(n), block_threads) threads (the
// reference's launch shape, device_resident_solver.cuh:1366-1393); the
// node's working vectors, the objective's workspace (shared_bytes, as in the
// reference a per-node global buffer) and the LMO's scratch live in the
// batch workspace. The sequential parts of the simplex and Birkhoff oracles
// run on one thread. This path is the general fallback; the built-in kinds
// stay on the library's tuned kernels.
#pragma once

#ifndef __CUDACC__
#error "gpuboscia/user_relax.cuh compiles device code: include it from a file compiled by nvcc"
#endif

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "device_resident_solver.h"

namespace gpuboscia {
namespace user_detail {

constexpr double kNone = 1e300;   // "no candidate"
constexpr int kVecs = 7;          // g, v, a, tx, tg, cand, sorting scratch

__device__ inline double block_sum(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    for (int i = 0; i < nw; ++i) s += red[i];
    __syncthreads();
    return s;
}
__device__ inline double block_min(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[w] = v;
    __syncthreads();
    double s = red[0];
    for (int i = 1; i < nw; ++i) s = fmin(s, red[i]);
    __syncthreads();
    return s;
}
__device__ inline bool block_and(bool b, int* flag) {
    __syncthreads();
    if (threadIdx.x == 0) *flag = 1;
    __syncthreads();
    if (!b) *flag = 0;
    __syncthreads();
    const bool r = *flag != 0;
    __syncthreads();
    return r;
}

// Birkhoff scratch per node (global): potentials and paths of a k x k problem
struct HungWs {
    double *u, *v, *minv;
    int *p, *way, *fcol, *frow, *rows, *cols;
    unsigned char* used;
};
__host__ __device__ inline size_t hung_bytes(int m) {
    return (size_t)3 * (m + 1) * sizeof(double) + (size_t)6 * (m + 1) * sizeof(int) + (size_t)(m + 1) + 16;
}
__device__ inline HungWs hung_at(unsigned char* base, int m) {
    HungWs h;
    double* d = reinterpret_cast<double*>(base);
    h.u = d; h.v = d + (m + 1); h.minv = d + 2 * (m + 1);
    int* i = reinterpret_cast<int*>(d + 3 * (m + 1));
    h.p = i; h.way = i + (m + 1); h.fcol = i + 2 * (m + 1); h.frow = i + 3 * (m + 1); h.rows = i + 4 * (m + 1);
    h.cols = i + 5 * (m + 1);
    h.used = reinterpret_cast<unsigned char*>(i + 6 * (m + 1));
    return h;
}

// The built-in LMO kinds on the device (the library's semantics: lmo.cuh's
// BoxLMO, UnitSimplexLMO / EqualitySimplexLMO greedy, BirkhoffLMO's
// shortest-augmenting-path Hungarian with lowest-index ties).
struct DevLMO {
    gbx_lmo l;
    int n;
    __device__ bool simplex() const { return l.kind == GBX_LMO_SIMPLEX || l.kind == GBX_LMO_EQUALITY_SIMPLEX; }
    __device__ bool eq() const { return l.kind == GBX_LMO_EQUALITY_SIMPLEX; }
    __device__ bool isint(int j) const { return l.is_int && l.is_int[j]; }

    // simplex greedy (thread 0): eligible coordinates in order of (g, index)
    // take min(cap, remaining - caps of those before) (lmo.cuh:529-618)
    __device__ void greedy(const double* g, const double* ub, double* out, const unsigned char* fixed,
                           double remaining, bool force_full, bool floor_int, int* order) const {
        int cnt = 0;
        for (int j = 0; j < n; ++j) {
            if ((fixed && fixed[j]) || !(force_full || g[j] <= 0.0)) continue;
            int pos = cnt++;
            while (pos > 0) {   // insertion by (g, index)
                const int q = order[pos - 1];
                if (g[q] < g[j] || (g[q] == g[j] && q < j)) break;
                order[pos] = q;
                --pos;
            }
            order[pos] = j;
        }
        double before = 0.0;
        for (int t = 0; t < cnt; ++t) {
            const int j = order[t];
            const double cap = isint(j) ? fmax(ub[j] - out[j], 0.0) : remaining;
            double add = fmin(fmax(remaining - before, 0.0), cap);
            before += cap;
            if (floor_int && isint(j)) add = floor(add + (eq() ? 1e-9 : 0.0));
            out[j] += add;
        }
    }

    // min-cost permutation under the branch bounds (and the face of x when
    // given); thread 0; false when none exists
    __device__ bool hungarian(const double* cost, const double* lb, const double* ub, double* out,
                              const double* face, const HungWs& h) const {
        const int m = l.order;
        for (int i = 0; i < m; ++i) { h.fcol[i] = -1; h.frow[i] = -1; }
        for (int r = 0; r < m; ++r)
            for (int c = 0; c < m; ++c) {
                const int e = r * m + c;
                if (lb[e] > ub[e] + 1e-9) return false;
                const bool ff = face && face[e] >= 1.0 - 1e-9;
                if (lb[e] > 0.5 || ff) {
                    if (ub[e] < 0.5 || h.fcol[r] >= 0 || h.frow[c] >= 0) return false;
                    h.fcol[r] = c;
                    h.frow[c] = r;
                    out[e] = 1.0;
                }
            }
        int k = 0, kc = 0;
        for (int i = 0; i < m; ++i) {
            if (h.fcol[i] < 0) h.rows[k++] = i;
            if (h.frow[i] < 0) h.cols[kc++] = i;
        }
        if (k != kc) return false;
        for (int j = 0; j <= k; ++j) { h.u[j] = 0.0; h.v[j] = 0.0; h.p[j] = 0; h.way[j] = 0; }
        for (int i = 1; i <= k; ++i) {
            h.p[0] = i;
            int j0 = 0;
            for (int j = 0; j <= k; ++j) { h.minv[j] = kNone; h.used[j] = 0; }
            for (int guard = 0; guard <= k + 1; ++guard) {
                h.used[j0] = 1;
                const int i0 = h.p[j0];
                for (int j = 1; j <= k; ++j) {
                    if (h.used[j]) continue;
                    const int e = h.rows[i0 - 1] * m + h.cols[j - 1];
                    if (ub[e] >= 0.5 && (!face || face[e] > 1e-9)) {
                        const double cur = cost[e] - h.u[i0] - h.v[j];
                        if (cur < h.minv[j]) { h.minv[j] = cur; h.way[j] = j0; }
                    }
                }
                double delta = kNone;
                int j1 = -1;
                for (int j = 1; j <= k; ++j) {
                    if (h.used[j] || !(h.minv[j] < kNone)) continue;
                    if (j1 < 0 || h.minv[j] < delta) { delta = h.minv[j]; j1 = j; }
                }
                if (j1 < 0 || !isfinite(delta)) return false;
                for (int j = 0; j <= k; ++j) {
                    if (h.used[j]) { h.u[h.p[j]] += delta; h.v[j] -= delta; }
                    else h.minv[j] -= delta;
                }
                j0 = j1;
                if (h.p[j0] == 0) break;
            }
            if (h.p[j0] != 0) return false;
            for (int guard = 0; guard <= k && j0 != 0; ++guard) {
                const int j1 = h.way[j0];
                h.p[j0] = h.p[j1];
                j0 = j1;
            }
        }
        for (int j = 1; j <= k; ++j) out[h.rows[h.p[j] - 1] * m + h.cols[j - 1]] = 1.0;
        return true;
    }

    // all threads; out, fixed, order, h: the node's scratch
    __device__ void forward(const double* g, const double* lb, const double* ub, double* out, double* red,
                            int* order, const HungWs& h) const {
        const int tid = threadIdx.x;
        if (l.kind == GBX_LMO_BOX) {
            for (int j = tid; j < n; j += blockDim.x) out[j] = g[j] > 0.0 ? lb[j] : ub[j];
            __syncthreads();
            return;
        }
        if (simplex()) {
            double loc = 0.0;
            for (int j = tid; j < n; j += blockDim.x) {
                out[j] = isint(j) ? lb[j] : 0.0;
                loc += out[j];
            }
            const double mass = block_sum(loc, red);
            if (tid == 0) greedy(g, ub, out, nullptr, l.right_side - mass, eq(), eq(), order);
            __syncthreads();
            return;
        }
        for (int j = tid; j < n; j += blockDim.x) out[j] = 0.0;
        __syncthreads();
        if (tid == 0 && n == l.order * l.order) hungarian(g, lb, ub, out, nullptr, h);
        __syncthreads();
    }

    __device__ void inface(const double* g, const double* x, const double* lb, const double* ub, double* out,
                           double* red, int* order, unsigned char* fixed, const HungWs& h) const {
        const int tid = threadIdx.x;
        const double atol = 1e-6, rtol = 1e-4;
        if (l.kind == GBX_LMO_BOX) {
            for (int j = tid; j < n; j += blockDim.x) {
                const double ut = atol + rtol * fabs(ub[j]), lt = atol + rtol * fabs(lb[j]);
                if (fabs(x[j] - ub[j]) <= ut) out[j] = ub[j];
                else if (fabs(x[j] - lb[j]) <= lt) out[j] = lb[j];
                else out[j] = g[j] > 0.0 ? lb[j] : ub[j];
            }
            __syncthreads();
            return;
        }
        if (simplex()) {
            double lm = 0.0, lx = 0.0;
            for (int j = tid; j < n; j += blockDim.x) {
                fixed[j] = 0;
                const double lower = isint(j) ? lb[j] : 0.0;
                out[j] = lower;
                if (fabs(x[j] - lower) <= atol + rtol * fmax(fabs(x[j]), fabs(lower))) {
                    fixed[j] = 1;
                } else if (isint(j) && fabs(x[j] - ub[j]) <= atol + rtol * fmax(fabs(x[j]), fabs(ub[j]))) {
                    fixed[j] = 1;
                    out[j] = ub[j];
                }
                lm += out[j];
                lx += x[j];
            }
            const double mass = block_sum(lm, red), xmass = block_sum(lx, red);
            const bool force = eq() || fabs(xmass - l.right_side)
                                           <= atol + rtol * fmax(fabs(xmass), fabs(l.right_side));
            if (tid == 0) greedy(g, ub, out, fixed, l.right_side - mass, force, true, order);
            __syncthreads();
            return;
        }
        for (int j = tid; j < n; j += blockDim.x) out[j] = 0.0;
        __syncthreads();
        if (tid == 0 && n == l.order * l.order) hungarian(g, lb, ub, out, x, h);
        __syncthreads();
    }

    // largest step of x - gamma * d inside the node's set, in [0, 1]
    __device__ double max_step(const double* d, const double* x, const double* lb, const double* ub,
                               double* red) const {
        double res = 1.0, sx = 0.0, sd = 0.0;
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            const double dj = d[j];
            if (simplex()) {
                const double tol = 1e-6;
                if (dj > tol) res = fmin(res, (x[j] - (isint(j) ? lb[j] : 0.0)) / dj);
                else if (dj < -tol) res = fmin(res, ((isint(j) ? ub[j] : l.right_side) - x[j]) / -dj);
                sx += x[j];
                sd += dj;
            } else {
                if (dj > 0.0) res = fmin(res, (x[j] - lb[j]) / dj);
                else if (dj < 0.0) res = fmin(res, (ub[j] - x[j]) / -dj);
            }
        }
        const double coord = block_min(res, red);
        double agg = 1.0;
        if (simplex()) {
            const double sum_x = block_sum(sx, red), sum_d = block_sum(sd, red);
            if (eq() && fabs(sum_d) > 1e-9) agg = 0.0;
            else agg = sum_d < 0.0 ? fmin(1.0, (sum_x - l.right_side) / sum_d) : 1.0;
        }
        return fmax(0.0, fmin(coord, agg));
    }

    __device__ bool feasible(const double* lb, const double* ub, const uint8_t* flags, double* red, int* flag,
                             double* out, const HungWs& h) const {
        if (l.kind == GBX_LMO_BOX) return true;
        if (simplex()) {
            bool valid = true, cont = false;
            double mand = 0.0, cap = 0.0;
            for (int j = threadIdx.x; j < n; j += blockDim.x) {
                const bool integer = flags ? flags[j] != 0 : isint(j);
                const double lo = integer ? ceil(fmax(0.0, lb[j])) : fmax(0.0, lb[j]);
                const double hi = integer ? floor(ub[j]) : ub[j];
                valid = valid && lo <= hi;
                mand += lo;
                cap += hi;
                cont = cont || !integer;
            }
            const double ms = block_sum(mand, red), cs = block_sum(cap, red);
            valid = block_and(valid, flag);
            const bool anycont = !block_and(!cont, flag);
            bool ok = valid && ms <= l.right_side + 1e-9;
            if (eq())
                ok = ok && cs >= l.right_side - 1e-9
                     && (anycont || fabs(l.right_side - round(l.right_side)) <= 1e-9);
            return ok;
        }
        (void)out;
        (void)h;
        return true;   // (Birkhoff nodes are checked by the kernel: a permutation inside the bounds)
    }

    __device__ bool rounded_feasible(const double* x, double tol, double* red, int* flag) const {
        if (l.kind == GBX_LMO_BOX) return true;
        bool valid = true;
        if (simplex()) {
            double s = 0.0;
            for (int j = threadIdx.x; j < n; j += blockDim.x) {
                valid = valid && x[j] >= -tol;
                s += x[j];
            }
            const double sum = block_sum(s, red);
            valid = block_and(valid, flag);
            return valid && (eq() ? fabs(sum - l.right_side) <= tol : sum <= l.right_side + tol);
        }
        const int m = l.order;
        if (n != m * m) return false;
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            double row = 0.0, col = 0.0;
            for (int j = 0; j < m; ++j) {
                if (x[i * m + j] < -tol) valid = false;
                row += x[i * m + j];
                col += x[j * m + i];
            }
            if (fabs(row - 1.0) > tol || fabs(col - 1.0) > tol) valid = false;
        }
        return block_and(valid, flag);
    }
};

template <class Obj>
__device__ double full_value(const Obj& obj, const double* x, unsigned char* ows, double* red) {
    return block_sum(obj.value_local(threadIdx.x, x, ows), red);
}

template <class Obj, class = void>
struct HasCurvature : std::false_type {};
template <class Obj>
struct HasCurvature<Obj, std::enable_if_t<Obj::supports_quadratic_exact>> : std::true_type {};

template <class Obj>
__device__ double curvature(const Obj& obj, const double* d, unsigned char* ows, double* red) {
    if constexpr (HasCurvature<Obj>::value) return block_sum(obj.quadratic_curvature_local(threadIdx.x, d, ows), red);
    else return 0.0;
}

// bytes of one node's scratch in the workspace
inline size_t node_bytes(int n, int order, int obj_bytes) {
    size_t b = (size_t)kVecs * n * sizeof(double);
    b += ((size_t)obj_bytes + 15) / 16 * 16;
    b += (hung_bytes(order) + 15) / 16 * 16;
    b += ((size_t)n + 15) / 16 * 16;   // in-face fixed flags
    return (b + 255) / 256 * 256;
}

// One CTA per node: the FW / DICG loop of the library's FP64 kernel over a
// user objective.
template <class Obj>
__global__ void user_relax_kernel(const Obj obj, const gbx_lmo lmo, const gbx_algorithm alg, const gbx_node_batch b,
                                  unsigned char* ws, size_t stride) {
    __shared__ double red[32];
    __shared__ int sflag[2];
    const int node = blockIdx.x;
    const int tid = threadIdx.x, n = Obj::n_vars;
    const DevLMO L{lmo, n};
    unsigned char* base = ws + (size_t)node * stride;
    double* g = reinterpret_cast<double*>(base);
    double* v = g + n;
    double* a = v + n;
    double* tx = a + n;
    double* tg = tx + n;
    double* cand = tg + n;
    int* order = reinterpret_cast<int*>(cand + n);
    unsigned char* ows = base + (size_t)kVecs * n * sizeof(double);
    unsigned char* hb = ows + ((size_t)Obj::shared_bytes + 15) / 16 * 16;
    const HungWs H = hung_at(hb, lmo.kind == GBX_LMO_BIRKHOFF ? lmo.order : 0);
    unsigned char* fixed = hb + (hung_bytes(lmo.kind == GBX_LMO_BIRKHOFF ? lmo.order : 0) + 15) / 16 * 16;
    const size_t off = (size_t)node * n;
    double* x = b.x + off;
    const double* lb = b.lb + off;
    const double* ub = b.ub + off;
    double* best = b.best_vertex + off;
    const uint8_t* flags = b.integer_flags;
    const double tol = b.candidate_tol, eps = b.eps[node];
    const int it0 = b.iterations[node];
    const bool supplied = (b.status[node] & GBX_NODE_INITIAL_POINT_SUPPLIED) != 0;
    obj.prepare_block(tid, ows);
    __syncthreads();
    double best_val = kNone;
    if (tid == 0) { b.best_vertex_val[node] = kNone; b.iterations[node] = it0; }

    // node feasibility (drs_node_feasible)
    bool valid = true;
    for (int j = tid; j < n; j += blockDim.x)
        if (isnan(lb[j]) || isnan(ub[j]) || lb[j] > ub[j] || (flags && flags[j] && ceil(lb[j]) > floor(ub[j])))
            valid = false;
    valid = block_and(valid, sflag);
    if (valid && lmo.kind == GBX_LMO_BIRKHOFF) {
        for (int j = tid; j < n; j += blockDim.x) { v[j] = 0.0; tg[j] = 0.0; }
        __syncthreads();
        if (tid == 0) sflag[1] = L.hungarian(tg, lb, ub, v, nullptr, H) ? 1 : 0;
        __syncthreads();
        valid = sflag[1] != 0;
    } else if (valid) {
        valid = L.feasible(lb, ub, flags, red, sflag, v, H);
    }
    if (!valid) {
        if (tid == 0) {
            b.status[node] = GBX_NODE_INFEASIBLE;
            b.value[node] = INFINITY;
            b.gap[node] = 0.0;
        }
        return;
    }
    if (it0 == 0 && !supplied) {
        for (int j = tid; j < n; j += blockDim.x) g[j] = -1.0 - (double)j / (n + 1.0);
        __syncthreads();
        L.forward(g, lb, ub, v, red, order, H);
        for (int j = tid; j < n; j += blockDim.x) x[j] = v[j];
        __syncthreads();
    }
    auto integer_value = [&](const double* vert) -> double {
        bool ok = true;
        for (int j = tid; j < n; j += blockDim.x)
            if (!isfinite(vert[j]) || vert[j] < lb[j] - tol || vert[j] > ub[j] + tol
                    || (flags && flags[j] && vert[j] != round(vert[j])))
                ok = false;
        ok = block_and(ok, sflag);
        if (!ok) return kNone;
        const double val = full_value(obj, vert, ows, red);
        return isfinite(val) ? val : kNone;
    };
    auto score = [&](const double* vert) {
        const double fv = integer_value(vert);
        if (fv < best_val) {
            best_val = fv;
            if (tid == 0) b.best_vertex_val[node] = fv;
        }
        if (fv < 1e299 && fv == best_val)
            for (int j = tid; j < n; j += blockDim.x) best[j] = vert[j];
        __syncthreads();
    };
    auto dot = [&](const double* u, const double* w2) {
        double loc = 0.0;
        for (int j = tid; j < n; j += blockDim.x) loc = fma(u[j], w2[j], loc);
        return block_sum(loc, red);
    };
    auto gap_of = [&](const double* gr, const double* vv) {
        double loc = 0.0;
        for (int j = tid; j < n; j += blockDim.x) loc = fma(gr[j], x[j] - vv[j], loc);
        return block_sum(loc, red);
    };
    // SecantLS::search (algorithms.cuh:121-258) and QuadraticExactLS
    auto search = [&](double gap, double maxg, const double* dir) -> double {
        if (alg.line_search == GBX_LS_QUADRATIC_EXACT) {
            const double curv = curvature(obj, dir, ows, red);
            if (maxg <= 0.0) return 0.0;
            if (curv > 0.0) return gap <= 0.0 ? 0.0 : fmin(gap / curv, maxg);
            return -gap + 0.5 * curv * maxg < 0.0 ? maxg : 0.0;
        }
        const double stol = alg.secant_tol, deps = alg.secant_denom_eps;
        const double f_base = full_value(obj, x, ows, red);
        double lo = 0.0, hi = maxg, best_f = f_base, best_gamma = 0.0, phi_lo = -gap, phi_hi = 0.0, gamma = 0.0;
        bool done = phi_lo >= -stol;
        const double allow = stol * (1.0 + fabs(f_base));
        auto probe = [&](double gm, double& phi, double& f) {
            for (int j = tid; j < n; j += blockDim.x) tx[j] = fma(gm, dir[j], x[j]);
            __syncthreads();
            obj.grad(tid, tx, tg, ows);
            __syncthreads();
            phi = dot(tg, dir);
            f = full_value(obj, tx, ows, red);
        };
        double f_hi;
        probe(maxg, phi_hi, f_hi);
        if (f_hi < best_f || (best_gamma == 0.0 && f_hi <= f_base + allow)) { best_f = f_hi; best_gamma = maxg; }
        if (!done && phi_hi <= stol && f_hi <= f_base + allow) { gamma = maxg; done = true; }
        for (int it = 0; it < alg.secant_iters && !done; ++it) {
            const double denom = phi_hi - phi_lo;
            double gm = (denom > deps || denom < -deps) ? hi - phi_hi * (hi - lo) / denom : 0.5 * (lo + hi);
            if (!(gm > lo && gm < hi)) gm = 0.5 * (lo + hi);
            gamma = gm;
            double phi, ft;
            probe(gamma, phi, ft);
            if (ft < best_f || (best_gamma == 0.0 && ft <= f_base + allow)) { best_f = ft; best_gamma = gamma; }
            if (phi < 0.0) { lo = gamma; phi_lo = phi; }
            else { hi = gamma; phi_hi = phi; }
            if ((phi <= stol && phi >= -stol) || (hi - lo) <= stol) { gamma = 0.5 * (lo + hi); done = true; }
        }
        if (best_gamma > 0.0 && best_f <= f_base + allow) gamma = best_gamma;
        else if (!done) gamma = 0.0;
        return gamma;
    };
    const bool dicg = alg.kind == GBX_ALG_DICG;
    const bool uses_search = alg.line_search == GBX_LS_SECANT || alg.line_search == GBX_LS_QUADRATIC_EXACT;
    const double cutv = b.cutoff ? *b.cutoff : INFINITY;
    int iters = it0;
    for (int iter = 0; iter < b.max_iters; ++iter) {
        iters = it0 + iter + 1;
        obj.grad(tid, x, g, ows);
        __syncthreads();
        const double fcut = (cutv < INFINITY && iter > 0) ? full_value(obj, x, ows, red) : 0.0;
        L.forward(g, lb, ub, v, red, order, H);
        score(v);
        const double gap = gap_of(g, v);
        if (gap >= 0.0 && gap < eps) break;
        if (cutv < INFINITY && iter > 0 && fcut - gap >= cutv) break;
        if (!dicg) {
            if (uses_search) {
                for (int j = tid; j < n; j += blockDim.x) v[j] -= x[j];
                __syncthreads();
                const double gm = search(gap, 1.0, v);
                for (int j = tid; j < n; j += blockDim.x) x[j] = fma(gm, v[j], x[j]);
            } else {
                const double gm = 2.0 / (double)(it0 + iter + 2);
                for (int j = tid; j < n; j += blockDim.x) x[j] = fma(gm, v[j] - x[j], x[j]);
            }
            __syncthreads();
            continue;
        }
        for (int j = tid; j < n; j += blockDim.x) g[j] = -g[j];
        __syncthreads();
        L.inface(g, x, lb, ub, a, red, order, fixed, H);
        score(a);
        for (int j = tid; j < n; j += blockDim.x) { g[j] = -g[j]; a[j] -= v[j]; }
        __syncthreads();
        const double gmax = L.max_step(a, x, lb, ub, red);
        if (uses_search) {
            for (int j = tid; j < n; j += blockDim.x) a[j] = -a[j];
            __syncthreads();
            double loc = 0.0;
            for (int j = tid; j < n; j += blockDim.x) loc = fma(-g[j], a[j], loc);
            const double pgap = block_sum(loc, red);
            const double gm = search(pgap, gmax, a);
            for (int j = tid; j < n; j += blockDim.x) x[j] = fma(gm, a[j], x[j]);
        } else {
            const double open = 2.0 / (double)(it0 + iter + 2);
            double gm;
            if (alg.line_search == GBX_LS_SAFEGUARDED_SCALED_OPEN_LOOP) gm = gmax <= open ? gmax : gmax * open;
            else if (alg.line_search == GBX_LS_SCALED_OPEN_LOOP) gm = gmax * open;
            else gm = fmin(gmax, open);
            for (int j = tid; j < n; j += blockDim.x) x[j] = fma(-gm, a[j], x[j]);
        }
        __syncthreads();
    }
    // certificate at the returned iterate
    obj.grad(tid, x, g, ows);
    __syncthreads();
    L.forward(g, lb, ub, v, red, order, H);
    score(v);
    const double fgap = gap_of(g, v);
    const double fval = full_value(obj, x, ows, red);
    int st = (fgap >= 0.0 && fgap < eps) ? GBX_NODE_FRACTIONAL_CONVERGED : GBX_NODE_FRACTIONAL_UNCONVERGED;
    if (flags) {
        for (int j = tid; j < n; j += blockDim.x) cand[j] = flags[j] ? round(x[j]) : x[j];
        __syncthreads();
        if (L.rounded_feasible(cand, tol, red, sflag)) {
            const double cv = integer_value(cand);
            if (cv < best_val) {
                for (int j = tid; j < n; j += blockDim.x) best[j] = cand[j];
                if (tid == 0) b.best_vertex_val[node] = cv;
            }
        }
    }
    bool integral = true;
    for (int j = tid; j < n; j += blockDim.x)
        if (!isfinite(x[j]) || (flags && flags[j] && fabs(x[j] - round(x[j])) > tol)) integral = false;
    if (block_and(integral, sflag)) st = st ? GBX_NODE_INTEGRAL_CONVERGED : GBX_NODE_INTEGRAL_UNCONVERGED;
    if (tid == 0) {
        b.value[node] = fval;
        b.gap[node] = fgap;
        b.status[node] = (uint8_t)st;
        b.iterations[node] = iters;
    }
}

}  // namespace user_detail

// The relaxation of user objective type Obj: what the engine calls instead of
// the library's gbx_relax_batch.
template <class Obj>
struct UserRelax<Obj, std::enable_if_t<!HasDescriptor<Obj>::value>> {
    static RelaxHooks hooks(const Obj& obj) {
        static_assert(Obj::block_threads >= 32 && Obj::block_threads % 32 == 0,
                      "block_threads must be a positive multiple of the CUDA warp size");
        static_assert(Obj::shared_bytes >= 0, "negative objective workspace");
        RelaxHooks h;
        h.workspace_bytes = [](const gbx_lmo& l, int nodes) -> size_t {
            return user_detail::node_bytes(Obj::n_vars, l.kind == GBX_LMO_BIRKHOFF ? l.order : 0,
                                           Obj::shared_bytes) * (size_t)(nodes > 0 ? nodes : 1);
        };
        h.launch = [obj](const gbx_lmo& l, const gbx_algorithm& a, const gbx_node_batch& b, void* ws,
                         size_t ws_bytes, cudaStream_t st) -> int {
            if (b.n_nodes <= 0) return GBX_OK;
            if (l.kind != GBX_LMO_BOX && l.kind != GBX_LMO_SIMPLEX && l.kind != GBX_LMO_EQUALITY_SIMPLEX
                    && l.kind != GBX_LMO_BIRKHOFF)
                return GBX_ERR_UNSUPPORTED;
            const size_t stride = user_detail::node_bytes(Obj::n_vars, l.kind == GBX_LMO_BIRKHOFF ? l.order : 0,
                                                          Obj::shared_bytes);
            if (!ws || ws_bytes < stride * (size_t)b.n_nodes) return GBX_ERR_WORKSPACE;
            // min(round32(n), block_threads, 1024) threads (device_resident_solver.cuh:1366-1393)
            int threads = (Obj::n_vars + 31) / 32 * 32;
            if (threads > Obj::block_threads) threads = Obj::block_threads;
            if (threads > 1024) threads = 1024;
            if (threads < 32) threads = 32;
            user_detail::user_relax_kernel<Obj><<<b.n_nodes, threads, 0, st>>>(
                obj, l, a, b, static_cast<unsigned char*>(ws), stride);
            return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
        };
        return h;
    }
};

}  // namespace gpuboscia
