// lmo.h -- the built-in linear minimization oracles (reference: include/gpuboscia/lmo.cuh).
//
// These are host-side descriptors: the oracles themselves run inside the
// GB300 relaxation kernel (libgpuboscia_gb300). Each type keeps the reference
// name, its supports_dicg flag and relaxation_feasible_cpu, and describes
// itself to the C ABI through spec().
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../gpuboscia_gb300.h"
#include "lmo_dicg.h"

namespace gpuboscia {
// What the relaxation kernel needs to know about an LMO (host data).
struct LMOSpec {
    int kind = GBX_LMO_BOX;
    double right_side = 1.0;
    std::vector<uint8_t> is_int;  // simplex integer flags, empty = none
    int order = 0;
    const double* upper = nullptr;  // linked cardinality: device per-asset bounds U_i
};
}  // namespace gpuboscia

// argmin over the box [lb, ub] (lmo.cuh:212-321)
struct BoxLMO {
    static constexpr bool supports_dicg = true;
    bool relaxation_feasible_cpu(const std::vector<double>&, const std::vector<double>&,
                                 const std::vector<double>&, double) const {
        return true;  // the public API checks the box bounds itself
    }
    // host restatements of the kernel's oracles (the reference's *_cpu members)
    void compute_v_cpu(const std::vector<double>& grad, const std::vector<double>& lb,
                       const std::vector<double>& ub, std::vector<double>& v) const {
        for (size_t j = 0; j < grad.size(); ++j) v[j] = grad[j] > 0.0 ? lb[j] : ub[j];
    }
    void compute_inface_v_cpu(const std::vector<double>& grad, const std::vector<double>& x,
                              const std::vector<double>& lb, const std::vector<double>& ub, std::vector<double>& a,
                              double atol = 1e-6, double rtol = 1e-4) const {
        box_inface_lmo_cpu(grad, x, lb, ub, a, atol, rtol);
    }
    double dicg_maximum_step_cpu(const std::vector<double>& direction, const std::vector<double>& x,
                                 const std::vector<double>& lb, const std::vector<double>& ub) const {
        return box_dicg_maximum_step_cpu(direction, x, lb, ub);
    }
    gpuboscia::LMOSpec spec(int) const { return {GBX_LMO_BOX, 1.0, {}, 0}; }
};

// Bounded simplex {x >= 0, sum x <= right_side} (== with RequireEquality),
// integer coordinates capped by their branch interval (lmo.cuh:335-912).
template <int MaxN, bool RequireEquality = false>
struct UnitSimplexLMO {
    static constexpr bool supports_dicg = true;
    double right_side = 1.0;
    unsigned char is_int[MaxN]{};

    UnitSimplexLMO() = default;
    UnitSimplexLMO(double rhs, int n, const std::vector<int>& int_vars) : right_side(rhs) {
        set_integer_vars(n, int_vars);
    }
    void set_integer_vars(int n, const std::vector<int>& int_vars) {
        std::fill(is_int, is_int + MaxN, (unsigned char)0);
        const int capped = std::min(n, MaxN);
        for (int idx : int_vars)
            if (idx >= 0 && idx < capped) is_int[idx] = 1;
    }
    bool relaxation_feasible_cpu(const std::vector<double>& x, const std::vector<double>&,
                                 const std::vector<double>&, double tol) const {
        return dicg_linear_feasible_cpu(x, tol);
    }
    bool dicg_linear_feasible_cpu(const std::vector<double>& v, double tol = 1e-3) const {
        return RequireEquality ? equality_simplex_linear_feasible_cpu(right_side, v, tol)
                               : unit_simplex_linear_feasible_cpu(right_side, v, tol);
    }
    bool dicg_inface_feasible_cpu(const std::vector<double>& a, const std::vector<double>& x, double atol = 1e-6,
                                  double rtol = 1e-4) const {
        return RequireEquality
                   ? equality_simplex_linear_feasible_cpu(right_side, a, atol + rtol * std::abs(right_side))
                   : unit_simplex_inface_feasible_cpu(right_side, a, x, atol, rtol);
    }
    // Forward oracle on the host: integer coordinates start at lb, the rest of
    // the mass goes greedily in (gradient, index) order -- to non-positive
    // gradients only unless the mass is fixed -- integer coordinates up to
    // ub (whole units under the equality), continuous ones taking all of it.
    void compute_v_cpu(const std::vector<double>& grad, const std::vector<double>& lb,
                       const std::vector<double>& ub, std::vector<double>& v) const {
        const int n = (int)grad.size(), m = std::min(n, MaxN);
        double mass = 0.0;
        std::vector<int> order;
        order.reserve(m);
        for (int j = 0; j < n; ++j) {
            v[j] = j < m && is_int[j] ? lb[j] : 0.0;
            if (j < m && is_int[j]) mass += v[j];
            if (j < m && (RequireEquality || !(grad[j] > 0.0))) order.push_back(j);
        }
        std::stable_sort(order.begin(), order.end(), [&](int p, int q) { return grad[p] < grad[q]; });
        double remaining = right_side - mass;
        for (int j : order) {
            if (!(remaining > 0.0)) break;
            double add = remaining;
            if (is_int[j]) {
                const double room = std::max(ub[j] - lb[j], 0.0);
                add = std::min(room, RequireEquality ? std::floor(remaining + 1e-9) : remaining);
            }
            v[j] += add;
            remaining -= add;
        }
    }
    void compute_inface_v_cpu(const std::vector<double>& grad, const std::vector<double>& x,
                              const std::vector<double>& lb, const std::vector<double>& ub, std::vector<double>& a,
                              double atol = 1e-6, double rtol = 1e-4) const {
        const int n = std::min((int)grad.size(), MaxN);
        unit_simplex_inface_lmo_cpu(right_side, std::vector<unsigned char>(is_int, is_int + n), grad, x, lb, ub, a,
                                    atol, rtol, RequireEquality);
    }
    double dicg_maximum_step_cpu(const std::vector<double>& direction, const std::vector<double>& x,
                                 const std::vector<double>& lb, const std::vector<double>& ub,
                                 double tol = 1e-6) const {
        const int n = std::min((int)direction.size(), MaxN);
        return unit_simplex_dicg_maximum_step_cpu(right_side, std::vector<unsigned char>(is_int, is_int + n),
                                                  direction, x, lb, ub, tol, RequireEquality);
    }
    gpuboscia::LMOSpec spec(int n) const {
        gpuboscia::LMOSpec s;
        s.kind = RequireEquality ? GBX_LMO_EQUALITY_SIMPLEX : GBX_LMO_SIMPLEX;
        s.right_side = right_side;
        s.is_int.assign(n, 0);
        for (int j = 0; j < std::min(n, MaxN); ++j) s.is_int[j] = is_int[j];
        return s;
    }
};

template <int MaxN>
using EqualitySimplexLMO = UnitSimplexLMO<MaxN, true>;

// Order x Order Birkhoff polytope, row-major; lb > 1/2 forces an edge,
// ub < 1/2 forbids it; exact Hungarian assignment (lmo.cuh:918-1419).
template <int Order>
struct BirkhoffLMO {
    static_assert(Order > 0, "Birkhoff order must be positive");
    static constexpr bool supports_dicg = true;
    static constexpr int variable_count = Order * Order;
    bool relaxation_feasible_cpu(const std::vector<double>& x, const std::vector<double>&,
                                 const std::vector<double>&, double tol) const {
        if (x.size() != static_cast<size_t>(variable_count)) return false;
        for (double v : x) if (v < -tol || v > 1 + tol) return false;
        for (int i = 0; i < Order; ++i) {
            double row = 0, col = 0;
            for (int j = 0; j < Order; ++j) { row += x[i * Order + j]; col += x[j * Order + i]; }
            if (std::abs(row - 1) > tol || std::abs(col - 1) > tol) return false;
        }
        return true;
    }
    gpuboscia::LMOSpec spec(int) const { return {GBX_LMO_BIRKHOFF, 1.0, {}, Order}; }

    // Host oracles (the reference's *_cpu members): the minimum-cost
    // permutation under the branch bounds (lb > 1/2 forces an edge, ub < 1/2
    // forbids it) -- and, in face mode, the face of x (x_e >= 1 - 1e-9 forced,
    // x_e <= 1e-9 forbidden) -- as the relaxation kernel computes it; all zeros
    // when no permutation exists.
    void compute_v_cpu(const std::vector<double>& grad, const std::vector<double>& lb,
                       const std::vector<double>& ub, std::vector<double>& v) const {
        v.resize(variable_count);
        if (!assign(grad, lb, ub, v, nullptr)) std::fill(v.begin(), v.end(), 0.0);
    }
    void compute_inface_v_cpu(const std::vector<double>& direction, const std::vector<double>& x,
                              const std::vector<double>& lb, const std::vector<double>& ub,
                              std::vector<double>& v) const {
        v.resize(variable_count);
        if (!assign(direction, lb, ub, v, &x)) std::fill(v.begin(), v.end(), 0.0);
    }
    double dicg_maximum_step_cpu(const std::vector<double>& direction, const std::vector<double>& x,
                                 const std::vector<double>& lb, const std::vector<double>& ub) const {
        double gamma = 1.0;
        for (int e = 0; e < variable_count; ++e) {
            const double d = direction[e];
            if (d > 0.0) gamma = std::min(gamma, (x[e] - lb[e]) / d);
            else if (d < 0.0) gamma = std::min(gamma, (ub[e] - x[e]) / -d);
        }
        return std::max(0.0, gamma);
    }

private:
    // Forced edges are placed first; the free rows and columns are then matched
    // by the shortest-augmenting-path Hungarian with row / column potentials
    // (one Dijkstra pass per free row). Reduced costs are (cost - u_row) - v_col;
    // the next column is the unreached one of least slack, the lowest index on
    // ties; columns no allowed edge reaches are never chosen.
    static bool assign(const std::vector<double>& cost, const std::vector<double>& lb,
                       const std::vector<double>& ub, std::vector<double>& out, const std::vector<double>* face) {
        const size_t N = (size_t)variable_count;
        if (cost.size() != N || lb.size() != N || ub.size() != N || (face && face->size() != N)) return false;
        std::fill(out.begin(), out.end(), 0.0);
        std::vector<int> row_of_col(Order, -1), col_of_row(Order, -1);
        for (int r = 0; r < Order; ++r)
            for (int c = 0; c < Order; ++c) {
                const int e = r * Order + c;
                if (lb[e] > ub[e] + 1e-9) return false;
                if (lb[e] > 0.5 || (face && (*face)[e] >= 1.0 - 1e-9)) {
                    if (ub[e] < 0.5 || col_of_row[r] >= 0 || row_of_col[c] >= 0) return false;
                    col_of_row[r] = c;
                    row_of_col[c] = r;
                    out[e] = 1.0;
                }
            }
        std::vector<int> R, C;
        for (int i = 0; i < Order; ++i) {
            if (col_of_row[i] < 0) R.push_back(i);
            if (row_of_col[i] < 0) C.push_back(i);
        }
        if (R.size() != C.size()) return false;
        const int k = (int)R.size();
        const double none = 1e300;   // slack of a column no allowed edge has reached
        // index 0 is the virtual column of the row being inserted
        std::vector<double> pot_r(k + 1, 0.0), pot_c(k + 1, 0.0), slack(k + 1);
        std::vector<int> match(k + 1, 0), prev(k + 1, 0);
        std::vector<char> done(k + 1);
        for (int row = 1; row <= k; ++row) {
            match[0] = row;
            std::fill(slack.begin(), slack.end(), none);
            std::fill(done.begin(), done.end(), 0);
            int col = 0;
            while (true) {
                done[col] = 1;
                const int r = match[col];
                for (int j = 1; j <= k; ++j) {
                    if (done[j]) continue;
                    const int e = R[r - 1] * Order + C[j - 1];
                    if (!(ub[e] >= 0.5) || (face && !((*face)[e] > 1e-9))) continue;
                    const double red = cost[e] - pot_r[r] - pot_c[j];
                    if (red < slack[j]) { slack[j] = red; prev[j] = col; }
                }
                int next = -1;
                for (int j = 1; j <= k; ++j)
                    if (!done[j] && slack[j] < none && (next < 0 || slack[j] < slack[next])) next = j;
                if (next < 0 || !std::isfinite(slack[next])) return false;
                const double delta = slack[next];
                for (int j = 0; j <= k; ++j) {
                    if (done[j]) { pot_r[match[j]] += delta; pot_c[j] -= delta; }
                    else slack[j] -= delta;
                }
                col = next;
                if (match[col] == 0) break;
            }
            for (int j = col; j != 0;) {   // flip the augmenting path
                const int pj = prev[j];
                match[j] = match[pj];
                j = pj;
            }
        }
        for (int j = 1; j <= k; ++j) out[R[match[j] - 1] * Order + C[j - 1]] = 1.0;
        return true;
    }
};

// Cardinality-constrained simplex over x = (w, z), n = 2*Assets:
// sum w = 1, 0 <= w <= z, sum z <= cardinality, 0 <= z <= 1. Branching fixes z;
// Frank-Wolfe only (no in-face oracle). No counterpart in the reference (its
// LinkedCardinalityLMO, below, lacks sum w = 1).
template <int Assets>
struct SimplexCardinalityLMO {
    static_assert(Assets > 0, "asset count must be positive");
    static constexpr bool supports_dicg = false;
    static constexpr int variable_count = 2 * Assets;
    int cardinality = 1;
    bool relaxation_feasible_cpu(const std::vector<double>& x, const std::vector<double>&,
                                 const std::vector<double>&, double tol) const {
        if (x.size() != static_cast<size_t>(variable_count)) return false;
        double sw = 0, sz = 0;
        for (int j = 0; j < Assets; ++j) {
            const double w = x[j], z = x[Assets + j];
            if (w < -tol || z < -tol || z > 1 + tol || w > z + tol) return false;
            sw += w;
            sz += z;
        }
        return std::abs(sw - 1) <= tol && sz <= cardinality + tol;
    }
    gpuboscia::LMOSpec spec(int) const { return {GBX_LMO_CARDINALITY, double(cardinality), {}, 0}; }
};

// The reference's sparse-Sharpe oracle (examples/sparse_sharpe.cu:266-546),
// same members in the same order so `LinkedCardinalityLMO lmo{assets, m, d_U,
// d_H, d_mu}` compiles unchanged: D = {(v, y): 0 <= v_i <= U_i y_i, 1'y <= m}
// with x = (v, y), y at offset n_vars / 2 (the example's MaxAssets), the first
// `assets` coordinates of each half active. Frank-Wolfe and DICG. The rounding
// candidate scales along the objective (a dense quadratic whose v-block is H
// and whose linear term is -mu), so device_H / device_mu are not read.
struct LinkedCardinalityLMO {
    static constexpr bool supports_dicg = true;
    int assets = 0;
    int cardinality = 1;
    const double* device_upper_bounds = nullptr;
    const double* device_H = nullptr;
    const double* device_mu = nullptr;
    gpuboscia::LMOSpec spec(int n) const {
        gpuboscia::LMOSpec s{GBX_LMO_LINKED_CARDINALITY, double(cardinality), {}, assets};
        (void)n;
        s.upper = device_upper_bounds;
        return s;
    }
};
