// tree.h -- validation of a caller-supplied root relaxation point.
//
// Interface of the reference's include/gpuboscia/tree.h:100-148: the names
// RootInitialPointValidator, HasRelaxationPointCheck,
// validate_initial_point_bounds and validate_root_initial_point, their
// arguments, the std::invalid_argument they throw and its messages. A root
// point must have the problem's size, be finite, lie within the bounds up to
// the tolerance, and lie in the LMO's continuous set -- checked by the
// caller's validator when one is given, else by the LMO's
// relaxation_feasible_cpu.
#pragma once
#include <cmath>
#include <cstddef>
#include <functional>
#include <stdexcept>
#include <type_traits>
#include <utility>
#include <vector>

#include "problem.h"

namespace gpuboscia {

using RootInitialPointValidator = std::function<bool(
    const std::vector<double>&, const std::vector<double>&, const std::vector<double>&, double)>;

namespace detail {
// Overload probe: the first candidate exists only for LMOs with a host
// relaxation_feasible_cpu(x, lb, ub, tol).
template <class LMO>
auto probe_relaxation_check(int) -> decltype(std::declval<const LMO&>().relaxation_feasible_cpu(
                                                 std::declval<const std::vector<double>&>(),
                                                 std::declval<const std::vector<double>&>(),
                                                 std::declval<const std::vector<double>&>(), 0.0),
                                             std::true_type{});
template <class LMO>
std::false_type probe_relaxation_check(long);

inline bool point_sizes_ok(const Problem& p, const std::vector<double>& x, double tol) {
    const std::size_t n = x.size();
    return std::isfinite(tol) && tol >= 0 && p.n_vars > 0 && n == static_cast<std::size_t>(p.n_vars)
           && p.lb.size() == n && p.ub.size() == n;
}

inline bool coordinate_ok(double lo, double hi, double v, double tol) {
    if (std::isnan(lo) || std::isnan(hi) || lo > hi || !std::isfinite(v)) return false;
    return v >= lo - tol && v <= hi + tol;
}
}  // namespace detail

template <class LMO>
struct HasRelaxationPointCheck : decltype(detail::probe_relaxation_check<LMO>(0)) {};

inline void validate_initial_point_bounds(const Problem& problem, const std::vector<double>& x,
                                          double tolerance) {
    if (!detail::point_sizes_ok(problem, x, tolerance))
        throw std::invalid_argument("invalid root initial point dimensions or tolerance");
    for (std::size_t j = 0; j < x.size(); ++j)
        if (!detail::coordinate_ok(problem.lb[j], problem.ub[j], x[j], tolerance))
            throw std::invalid_argument("root initial point is nonfinite or violates bounds");
}

// An empty x keeps the deterministic LMO start.
template <class LMO>
void validate_root_initial_point(const Problem& problem, const LMO& lmo, const std::vector<double>& x,
                                 const RootInitialPointValidator& validator = {}, double tolerance = 1e-9) {
    if (x.empty()) return;
    validate_initial_point_bounds(problem, x, tolerance);
    bool inside;
    if (validator) {
        inside = validator(x, problem.lb, problem.ub, tolerance);
    } else if constexpr (HasRelaxationPointCheck<LMO>::value) {
        inside = lmo.relaxation_feasible_cpu(x, problem.lb, problem.ub, tolerance);
    } else {
        throw std::invalid_argument(
            "root initial point requires LMO::relaxation_feasible_cpu or "
            "Settings::root_initial_point_feasible for custom constraints");
    }
    if (!inside) throw std::invalid_argument("root initial point violates the LMO's continuous feasible set");
}

}  // namespace gpuboscia
