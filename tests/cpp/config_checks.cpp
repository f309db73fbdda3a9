// The solver's constructor checks on its configuration, which run before any
// CUDA call in both implementations (device_resident_solver.cuh:1197-1218 of
// the reference): one line per case with the exception's type and message,
// for a differential check (the same source compiled against each set of
// headers; no GPU is needed, every case is rejected before the device).
#include <cmath>
#include <cstdio>
#include <functional>
#include <limits>
#include <stdexcept>
#include <vector>

#include <gpuboscia/dense_quadratic_objectives.cuh>
#include <gpuboscia/gpuboscia.cuh>

using Objective = ILSGlobalCachedObjective<2>;

static void attempt(const char* name, std::function<void(DeviceResidentConfig&, Problem&, double&)> change) {
    DeviceResidentConfig cfg;
    Problem prob{2, {0, 0}, {1, 1}, {0, 1}};
    double limit = std::numeric_limits<double>::infinity();
    change(cfg, prob, limit);
    try {
        DeviceResidentHybridSolver<Objective, FrankWolfePolicy> s(
            prob, Objective{}, FrankWolfePolicy{},
            [](const Node& p, int& id, const std::vector<double>& x, const std::vector<int>& iv) {
                return branch_pow2(p, id, x, iv, 3);
            },
            cfg, BoxLMO{}, limit);
        std::printf("%s accepted\n", name);
    } catch (const std::invalid_argument& e) {
        std::printf("%s invalid_argument: %s\n", name, e.what());
    } catch (const std::runtime_error& e) {
        std::printf("%s runtime_error: %s\n", name, e.what());
    }
}

int main() {
    const double nan = std::numeric_limits<double>::quiet_NaN(), inf = std::numeric_limits<double>::infinity();
    attempt("iters0", [](auto& c, auto&, auto&) { c.gpu_max_iters = 0; });
    attempt("batch0", [](auto& c, auto&, auto&) { c.gpu_batch_size = 0; });
    attempt("streams-1", [](auto& c, auto&, auto&) { c.num_streams = -1; });
    attempt("int_var_high", [](auto&, auto& p, auto&) { p.int_vars = {0, 2}; });
    attempt("int_var_negative", [](auto&, auto& p, auto&) { p.int_vars = {-1}; });
    attempt("eps0", [](auto& c, auto&, auto&) { c.gpu_eps = 0.0; });
    attempt("eps_nan", [nan](auto& c, auto&, auto&) { c.gpu_eps = nan; });
    attempt("eps_min_inf", [inf](auto& c, auto&, auto&) { c.gpu_eps_min = inf; });
    attempt("decay_above_1", [](auto& c, auto&, auto&) { c.gpu_eps_decay = 1.5; });
    attempt("decay0", [](auto& c, auto&, auto&) { c.gpu_eps_decay = 0.0; });
    attempt("abs_tol_negative", [](auto& c, auto&, auto&) { c.abs_gap_tol = -1e-9; });
    attempt("rel_tol_nan", [nan](auto& c, auto&, auto&) { c.rel_gap_tol = nan; });
    attempt("occupancy0", [](auto& c, auto&, auto&) { c.dicg_paired_occupancy_fraction = 0.0; });
    attempt("occupancy_above_1", [](auto& c, auto&, auto&) { c.dicg_paired_occupancy_fraction = 1.01; });
    attempt("limit0", [](auto&, auto&, auto& l) { l = 0.0; });
    attempt("limit_nan", [nan](auto&, auto&, auto& l) { l = nan; });
    attempt("limit_negative", [](auto&, auto&, auto& l) { l = -1.0; });
    attempt("n_vars_mismatch", [](auto&, auto& p, auto&) {
        p.n_vars = 3;
        p.lb = {0, 0, 0};
        p.ub = {1, 1, 1};
    });
    attempt("n_vars_mismatch_and_iters0", [](auto& c, auto& p, auto&) {
        c.gpu_max_iters = 0;
        p.n_vars = 3;
        p.lb = {0, 0, 0};
        p.ub = {1, 1, 1};
    });
    attempt("first_of_two", [](auto& c, auto&, auto& l) {   // the first failing check decides
        c.gpu_eps = 0.0;
        l = 0.0;
    });
    return 0;
}
