// lmo_dicg.h -- host-side DICG primitives of the box and simplex oracles
// (reference: include/gpuboscia/lmo_dicg.h). Same functions, arguments,
// defaults and results, so host code and tests that call them keep working;
// the relaxation kernel computes the same vertices and steps on the GPU.
//
// In-face oracle: coordinates that sit on a bound define the minimal face of
// x and stay there; the rest are chosen as by the forward oracle. Maximum
// step: the largest gamma <= 1 with x - gamma * direction still feasible.
#pragma once
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

// |a - b| <= atol + rtol * max(|a|, |b|): the face tolerance.
inline bool dicg_isapprox(double a, double b, double atol = 1e-6, double rtol = 1e-4) {
    const double scale = std::max(std::abs(a), std::abs(b));
    return std::abs(a - b) <= atol + rtol * scale;
}

// Box [lb, ub]: a coordinate at a bound keeps it; the others take lb where the
// gradient is positive and ub otherwise.
inline void box_inface_lmo_cpu(const std::vector<double>& grad, const std::vector<double>& x,
                               const std::vector<double>& lb, const std::vector<double>& ub,
                               std::vector<double>& a, double atol = 1e-6, double rtol = 1e-4) {
    for (size_t j = 0; j < grad.size(); ++j) {
        if (dicg_isapprox(x[j], ub[j], atol, rtol)) a[j] = ub[j];
        else if (dicg_isapprox(x[j], lb[j], atol, rtol)) a[j] = lb[j];
        else a[j] = grad[j] > 0.0 ? lb[j] : ub[j];
    }
}

inline double box_dicg_maximum_step_cpu(const std::vector<double>& direction, const std::vector<double>& x,
                                        const std::vector<double>& lb, const std::vector<double>& ub) {
    double gamma = 1.0;
    for (size_t j = 0; j < x.size(); ++j) {
        const double d = direction[j];
        if (d < 0.0) gamma = std::min(gamma, (ub[j] - x[j]) / -d);
        else if (d > 0.0) gamma = std::min(gamma, (x[j] - lb[j]) / d);
    }
    return gamma;
}

// {x >= 0, sum x <= right_side} (== right_side with require_full_mass, or
// when x already carries the full mass); branch bounds apply to integer
// coordinates only. Integer coordinates start at lb (or the bound they sit
// on); continuous ones at 0 (fixed there when x_j ~ 0). The missing mass then
// goes greedily to the free coordinates in (gradient, index) order -- only
// to non-positive gradients unless the full mass is required -- integer ones
// in whole units up to ub. The remaining mass is re-summed after each
// coordinate, and the walk stops once it is ~0.
inline void unit_simplex_inface_lmo_cpu(double right_side, const std::vector<unsigned char>& is_int,
                                        const std::vector<double>& grad, const std::vector<double>& x,
                                        const std::vector<double>& lb, const std::vector<double>& ub,
                                        std::vector<double>& a, double atol = 1e-6, double rtol = 1e-4,
                                        bool require_full_mass = false) {
    const int n = (int)grad.size();
    double x_mass = 0.0;
    for (int j = 0; j < n; ++j) x_mass += x[j];
    const bool full = require_full_mass || dicg_isapprox(x_mass, right_side, atol, rtol);

    std::vector<int> free_coords;
    free_coords.reserve(n);
    double mass = 0.0;
    for (int j = 0; j < n; ++j) {
        bool fixed = false;
        if (is_int[j]) {
            a[j] = lb[j];
            if (dicg_isapprox(x[j], lb[j], atol, rtol)) {
                fixed = true;
            } else if (dicg_isapprox(x[j], ub[j], atol, rtol)) {
                a[j] = ub[j];
                fixed = true;
            }
        } else {
            a[j] = 0.0;
            fixed = dicg_isapprox(x[j], 0.0, atol, rtol);
        }
        mass += a[j];
        if (!fixed && (full || !(grad[j] > 0.0))) free_coords.push_back(j);
    }
    if (dicg_isapprox(mass, right_side, atol, rtol)) return;

    std::stable_sort(free_coords.begin(), free_coords.end(), [&](int p, int q) { return grad[p] < grad[q]; });
    double remaining = right_side - mass;
    for (int j : free_coords) {
        if (!(remaining > 0.0)) break;
        const double add = is_int[j] ? std::min(std::max(ub[j] - a[j], 0.0), std::floor(remaining)) : remaining;
        a[j] += add;
        double total = 0.0;
        for (int i = 0; i < n; ++i) total += a[i];
        remaining = right_side - total;
        if (dicg_isapprox(remaining, 0.0, atol, rtol)) return;
    }
}

inline double unit_simplex_dicg_maximum_step_cpu(double right_side, const std::vector<unsigned char>& is_int,
                                                 const std::vector<double>& direction, const std::vector<double>& x,
                                                 const std::vector<double>& lb, const std::vector<double>& ub,
                                                 double tol = 1e-6, bool require_full_mass = false) {
    double gamma = 1.0, sum_x = 0.0, sum_d = 0.0;
    for (size_t j = 0; j < x.size(); ++j) {
        const double d = direction[j];
        if (d > tol) gamma = std::min(gamma, (x[j] - (is_int[j] ? lb[j] : 0.0)) / d);
        else if (d < -tol) gamma = std::min(gamma, ((is_int[j] ? ub[j] : right_side) - x[j]) / -d);
        if (std::abs(gamma) <= tol) return 0.0;
        sum_x += x[j];
        sum_d += d;
    }
    // with the full mass required the direction must keep sum x
    if (require_full_mass && std::abs(sum_d) > tol) return 0.0;
    if (sum_d < 0.0) gamma = std::min(gamma, (sum_x - right_side) / sum_d);
    return gamma;
}

inline bool equality_simplex_linear_feasible_cpu(double right_side, const std::vector<double>& v,
                                                 double tol = 1e-3) {
    double mass = 0.0;
    for (double e : v) {
        if (e < -tol) return false;
        mass += e;
    }
    return std::isfinite(mass) && std::abs(mass - right_side) <= tol;
}

inline bool unit_simplex_linear_feasible_cpu(double right_side, const std::vector<double>& v, double tol = 1e-3) {
    double mass = 0.0;
    for (double e : v) {
        if (e < 0.0) return false;
        mass += e;
    }
    return mass <= right_side + tol;
}

// An in-face vertex of a point with the full mass must carry the full mass too.
inline bool unit_simplex_inface_feasible_cpu(double right_side, const std::vector<double>& a,
                                             const std::vector<double>& x, double atol = 1e-6,
                                             double rtol = 1e-4) {
    const double mass_a = std::accumulate(a.begin(), a.end(), 0.0);
    const double mass_x = std::accumulate(x.begin(), x.end(), 0.0);
    if (dicg_isapprox(mass_x, right_side, atol, rtol) && !dicg_isapprox(mass_a, right_side, atol, rtol))
        return false;
    return unit_simplex_linear_feasible_cpu(right_side, a);
}
