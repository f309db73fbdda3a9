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
    // DeviceResidentConfig::node_limit stopped the search (no counterpart in the reference)
    bool reached_node_limit = false;
};

inline Settings create_default_settings() { return Settings{}; }

// True for LMOs that declare `static constexpr bool supports_dicg = true`.
template <typename LMO, typename = void>
struct lmo_supports_dicg : std::false_type {};
template <typename LMO>
struct lmo_supports_dicg<LMO, std::enable_if_t<LMO::supports_dicg>> : std::true_type {};

namespace detail {

// The eight (algorithm, line search) policies solve() can run.
enum class PolicyId { FwOpenLoop, FwSecant, FwQuadExact, DicgOpenLoop, DicgScaled, DicgSafeguarded,
                      DicgSecant, DicgQuadExact };

// Picks the policy of Settings::algorithm x Settings::line_search, or throws
// std::invalid_argument for a combination the objective or LMO cannot run.
// Checks go in this order: quadratic-exact needs the objective's curvature,
// DICG needs an LMO with an in-face oracle, scaled open-loop steps need DICG.
template <typename DeviceObjective, typename LMO>
PolicyId choose_policy(const Settings& settings) {
    const LineSearchKind ls = settings.line_search.kind;
    const bool dicg = settings.algorithm == FWAlgorithmKind::DICG;
    if (ls == LineSearchKind::QuadraticExact && !SupportsQuadraticExact<DeviceObjective>::value)
        throw std::invalid_argument("quadratic-exact requires an objective with quadratic curvature support");
    if (dicg && !lmo_supports_dicg<LMO>::value)
        throw std::invalid_argument(ls == LineSearchKind::QuadraticExact
                                        ? "the selected LMO does not support DICG"
                                        : "the selected LMO does not support DICG; use Frank-Wolfe");
    switch (ls) {
    case LineSearchKind::QuadraticExact: return dicg ? PolicyId::DicgQuadExact : PolicyId::FwQuadExact;
    case LineSearchKind::Secant: return dicg ? PolicyId::DicgSecant : PolicyId::FwSecant;
    case LineSearchKind::ScaledOpenLoop:
    case LineSearchKind::SafeguardedScaledOpenLoop:
        if (!dicg) throw std::invalid_argument("scaled open-loop is available only for DICG");
        return ls == LineSearchKind::ScaledOpenLoop ? PolicyId::DicgScaled : PolicyId::DicgSafeguarded;
    default: return dicg ? PolicyId::DicgOpenLoop : PolicyId::FwOpenLoop;
    }
}

// branch_pow2 over three variables, the reference's default branching.
inline BranchStrategy default_branching(double integer_tol) {
    return [integer_tol](const Node& parent, int& next_id, const std::vector<double>& x,
                         const std::vector<int>& int_vars) {
        return branch_pow2(parent, next_id, x, int_vars, 3, integer_tol);
    };
}

// The root node: the problem's bounds, the natural lower bound as its dual
// bound and the caller's start point (empty: the LMO start).
inline Node root_node(const Problem& problem, const Settings& settings) {
    const double nlb = settings.natural_lower_bound;
    if (std::isnan(nlb) || nlb == std::numeric_limits<double>::infinity())
        throw std::invalid_argument("natural lower bound must be finite or negative infinity");
    Node root(0, -1, 0, problem.lb, problem.ub);
    root.dual_bound = nlb;
    root.relaxation_x = settings.root_initial_point;
    return root;
}

}  // namespace detail

// Runs the search with an explicit policy (gpuboscia.cuh:56-104): the root
// point is validated, Settings::branch (or branch_pow2, k = 3) splits nodes,
// and the result carries the incumbent, the final dual bound and the time
// spent inside the search.
template <typename DeviceObjective, typename Algorithm, typename LMO, typename Heuristic = RoundingHeuristic>
Result solve_with_algorithm(const Problem& problem, DeviceObjective objective, LMO lmo, const Settings& settings,
                            Algorithm algorithm, Heuristic heuristic = {}) {
    validate_root_initial_point(problem, lmo, settings.root_initial_point, settings.root_initial_point_feasible);
    if (settings.device.device_frontier && settings.branch)
        throw std::invalid_argument("the device frontier branches with branch_pow2; leave Settings::branch empty");
    const BranchStrategy branch = settings.branch ? settings.branch
                                                  : detail::default_branching(settings.device.integer_tol);
    DeviceResidentHybridSolver<DeviceObjective, Algorithm, LMO, Heuristic> solver(
        problem, objective, algorithm, branch, settings.device, lmo, settings.time_limit_seconds, heuristic);
    if (settings.progress) solver.set_progress_callback(settings.progress);
    solver.push(detail::root_node(problem, settings));

    using clock = std::chrono::steady_clock;
    const clock::time_point t0 = clock::now();
    solver.solve();
    Result r;
    r.elapsed_seconds = std::chrono::duration<double>(clock::now() - t0).count();
    r.objective = solver.incumbent_value();
    r.x = solver.incumbent_x();
    r.dual_bound = solver.dual_bound();
    r.nodes_processed = solver.nodes_processed();
    r.reached_tolerance = solver.reached_tolerance();
    r.reached_time_limit = solver.reached_time_limit();
    r.reached_node_limit = solver.reached_node_limit();
    return r;
}

// The drop-in entry (gpuboscia.cuh:108-170): runs the policy that
// Settings::algorithm and Settings::line_search name. Policies the objective
// or LMO cannot run are never instantiated.
template <typename DeviceObjective, typename LMO, typename Heuristic = RoundingHeuristic>
Result solve(const Problem& problem, DeviceObjective objective, LMO lmo,
             const Settings& settings = create_default_settings(), Heuristic heuristic = {}) {
    constexpr bool has_curvature = SupportsQuadraticExact<DeviceObjective>::value;
    constexpr bool has_inface = lmo_supports_dicg<LMO>::value;
    const LineSearchOptions& o = settings.line_search;
    const SecantLS secant{o.secant_iters, o.secant_tol, o.secant_denom_eps};
    auto run = [&](auto policy) { return solve_with_algorithm(problem, objective, lmo, settings, policy, heuristic); };
    switch (detail::choose_policy<DeviceObjective, LMO>(settings)) {
    case detail::PolicyId::FwOpenLoop: return run(FrankWolfeOpenLoop{});
    case detail::PolicyId::FwSecant: return run(FrankWolfeSecant{secant});
    case detail::PolicyId::FwQuadExact:
        if constexpr (has_curvature) return run(FrankWolfeQuadraticExact{});
        break;
    case detail::PolicyId::DicgOpenLoop:
        if constexpr (has_inface) return run(DICGOpenLoop{});
        break;
    case detail::PolicyId::DicgScaled:
        if constexpr (has_inface) return run(DICGScaledOpenLoop{});
        break;
    case detail::PolicyId::DicgSafeguarded:
        if constexpr (has_inface) return run(DICGSafeguardedScaledOpenLoop{});
        break;
    case detail::PolicyId::DicgSecant:
        if constexpr (has_inface) return run(DICGSecant{secant});
        break;
    case detail::PolicyId::DicgQuadExact:
        if constexpr (has_inface && has_curvature) return run(DICGQuadraticExact{});
        break;
    }
    throw std::logic_error("solve: no policy for this algorithm and line search");
}

}  // namespace gpuboscia
