// gpuboscia.h -- public entry point (reference: include/gpuboscia/gpuboscia.cuh:19-172).
//
// Same Settings / Result / solve() / solve_with_algorithm() as the reference.
// The node relaxations run in libgpuboscia_gb300 (link -lgpuboscia_gb300
// -lcudart); this header and the scheduler it includes are plain C++17.
#pragma once

#include <chrono>
#include <cmath>
#include <functional>
#include <limits>
#include <stdexcept>
#include <type_traits>
#include <utility>
#include <vector>

#include "algorithms.h"
#include "branching.h"
#include "device_resident_solver.h"
#include "line_search_options.h"
#include "node.h"
#include "problem.h"
#include "tree.h"

namespace gpuboscia {

struct Settings {
    DeviceResidentConfig device{};
    FWAlgorithmKind algorithm = FWAlgorithmKind::DICG;
    LineSearchOptions line_search{};
    BranchStrategy branch;
    std::function<void(int, int, double, double, bool)> progress;
    double time_limit_seconds = std::numeric_limits<double>::infinity();
    double natural_lower_bound = -std::numeric_limits<double>::infinity();
    // Continuous root iterate (not an incumbent); empty selects the LMO start.
    std::vector<double> root_initial_point;
    RootInitialPointValidator root_initial_point_feasible;
};

struct Result {
    double objective = std::numeric_limits<double>::infinity();
    std::vector<double> x;
    double dual_bound = -std::numeric_limits<double>::infinity();
    int nodes_processed = 0;
    double elapsed_seconds = 0.0;
    bool reached_tolerance = false;
    bool reached_time_limit = false;
};

inline Settings create_default_settings() { return Settings{}; }

template <typename LMO, typename = void>
struct lmo_supports_dicg : std::false_type {};
template <typename LMO>
struct lmo_supports_dicg<LMO, std::void_t<decltype(LMO::supports_dicg)>>
    : std::integral_constant<bool, LMO::supports_dicg> {};

template <typename DeviceObjective, typename Algorithm, typename LMO, typename Heuristic = RoundingHeuristic>
Result solve_with_algorithm(const Problem& problem, DeviceObjective objective, LMO lmo, const Settings& settings,
                            Algorithm algorithm, Heuristic heuristic = {}) {
    validate_root_initial_point(problem, lmo, settings.root_initial_point, settings.root_initial_point_feasible);
    BranchStrategy branch = settings.branch;
    if (settings.device.device_frontier && branch)
        throw std::invalid_argument("the device frontier branches with branch_pow2; leave Settings::branch empty");
    if (!branch) {
        const double integer_tol = settings.device.integer_tol;
        branch = [integer_tol](const Node& parent, int& next_id, const std::vector<double>& x,
                               const std::vector<int>& int_vars) {
            return branch_pow2(parent, next_id, x, int_vars, 3, integer_tol);
        };
    }
    DeviceResidentHybridSolver<DeviceObjective, Algorithm, LMO, Heuristic> solver(
        problem, objective, algorithm, branch, settings.device, lmo, settings.time_limit_seconds, heuristic);
    if (settings.progress) solver.set_progress_callback(settings.progress);
    Node root(0, -1, 0, problem.lb, problem.ub);
    if (std::isnan(settings.natural_lower_bound)
            || settings.natural_lower_bound == std::numeric_limits<double>::infinity())
        throw std::invalid_argument("natural lower bound must be finite or negative infinity");
    root.dual_bound = settings.natural_lower_bound;
    root.relaxation_x = settings.root_initial_point;
    solver.push(root);
    const auto started = std::chrono::steady_clock::now();
    solver.solve();
    const double elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - started).count();
    return Result{solver.incumbent_value(), solver.incumbent_x(), solver.dual_bound(), solver.nodes_processed(),
                  elapsed, solver.reached_tolerance(), solver.reached_time_limit()};
}

// Policy dispatch on Settings::algorithm x Settings::line_search (gpuboscia.cuh:108-170).
template <typename DeviceObjective, typename LMO, typename Heuristic = RoundingHeuristic>
Result solve(const Problem& problem, DeviceObjective objective, LMO lmo,
             const Settings& settings = create_default_settings(), Heuristic heuristic = {}) {
    const auto& ls = settings.line_search;
    if (ls.kind == LineSearchKind::QuadraticExact) {
        if constexpr (!SupportsQuadraticExact<DeviceObjective>::value) {
            throw std::invalid_argument("quadratic-exact requires an objective with quadratic curvature support");
        } else {
            if (settings.algorithm == FWAlgorithmKind::DICG) {
                if constexpr (lmo_supports_dicg<LMO>::value)
                    return solve_with_algorithm(problem, objective, lmo, settings, DICGQuadraticExact{}, heuristic);
                else
                    throw std::invalid_argument("the selected LMO does not support DICG");
            }
            return solve_with_algorithm(problem, objective, lmo, settings, FrankWolfeQuadraticExact{}, heuristic);
        }
    }
    if (settings.algorithm == FWAlgorithmKind::DICG) {
        if constexpr (!lmo_supports_dicg<LMO>::value) {
            throw std::invalid_argument("the selected LMO does not support DICG; use Frank-Wolfe");
        } else {
            if (ls.kind == LineSearchKind::Secant)
                return solve_with_algorithm(problem, objective, lmo, settings,
                                            DICGSecant{SecantLS{ls.secant_iters, ls.secant_tol, ls.secant_denom_eps}},
                                            heuristic);
            if (ls.kind == LineSearchKind::ScaledOpenLoop)
                return solve_with_algorithm(problem, objective, lmo, settings, DICGScaledOpenLoop{}, heuristic);
            if (ls.kind == LineSearchKind::SafeguardedScaledOpenLoop)
                return solve_with_algorithm(problem, objective, lmo, settings, DICGSafeguardedScaledOpenLoop{},
                                            heuristic);
            return solve_with_algorithm(problem, objective, lmo, settings, DICGOpenLoop{}, heuristic);
        }
    }
    if (ls.kind == LineSearchKind::ScaledOpenLoop || ls.kind == LineSearchKind::SafeguardedScaledOpenLoop)
        throw std::invalid_argument("scaled open-loop is available only for DICG");
    if (ls.kind == LineSearchKind::Secant)
        return solve_with_algorithm(problem, objective, lmo, settings,
                                    FrankWolfeSecant{SecantLS{ls.secant_iters, ls.secant_tol, ls.secant_denom_eps}},
                                    heuristic);
    return solve_with_algorithm(problem, objective, lmo, settings, FrankWolfeOpenLoop{}, heuristic);
}

}  // namespace gpuboscia
