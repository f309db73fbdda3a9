// Uses every public member of the reference's DeviceResidentHybridSolver
// (device_resident_solver.cuh:1182-1298: constructor forms, push, the two
// callbacks, solve and the accessors) and of its solve entry points, with the
// reference's own types, so that the same source compiled against two
// implementations of the headers checks that the whole surface exists with
// compatible signatures. Compile-only: running it needs a GPU.
#include <cstdio>
#include <vector>

#include <gpuboscia/dense_quadratic_objectives.cuh>
#include <gpuboscia/gpuboscia.cuh>

using Objective = ILSGlobalCachedObjective<16>;

int run(const double* d_Q, const double* d_c) {
    Problem prob{16, std::vector<double>(16, 0.0), std::vector<double>(16, 1.0), {}};
    Objective obj{d_Q, d_c, 4.0};
    DeviceResidentConfig cfg;
    cfg.gpu_batch_size = 4;
    cfg.num_streams = 1;
    cfg.dicg_oracle_parallelism = DeviceResidentConfig::DICGOracleParallelism::Paired;
    BranchStrategy branch = [](const Node& p, int& id, const std::vector<double>& x, const std::vector<int>& iv) {
        return branch_pow2(p, id, x, iv, 3);
    };
    BirkhoffLMO<4> lmo;
    DeviceResidentHybridSolver<Objective, DICGPolicy, BirkhoffLMO<4>> solver(prob, obj, DICGPolicy{}, branch, cfg,
                                                                             lmo);
    DeviceResidentHybridSolver<Objective, FrankWolfePolicy> plain(prob, obj, FrankWolfePolicy{}, branch);
    Node root(0, -1, 0, prob.lb, prob.ub);
    root.dual_bound = -1e300;
    solver.push(root);
    solver.set_progress_callback([](int, int, double, double, bool) {});
    solver.set_scheduling_callback([](const DRSSchedulingEvent& e) { (void)e.slot_id; });
    solver.solve();
    const double v = solver.incumbent_value();
    const std::vector<double> x = solver.incumbent_x();
    const int nodes = solver.nodes_processed();
    const double bound = solver.dual_bound();
    const int it = solver.last_gpu_iterations();
    const double gap = solver.last_gpu_gap();
    const bool conv = solver.last_gpu_converged();
    const bool tol = solver.reached_tolerance();
    const bool tl = solver.reached_time_limit();
    const int b = solver.effective_gpu_batch_size() + solver.effective_num_streams() + solver.paired_gpu_batches();
    (void)plain;

    auto settings = gpuboscia::create_default_settings();
    settings.algorithm = FWAlgorithmKind::DICG;
    settings.line_search.kind = LineSearchKind::QuadraticExact;
    settings.branch = branch;
    settings.root_initial_point = std::vector<double>(16, 0.25);
    const gpuboscia::Result r1 = gpuboscia::solve(prob, obj, BirkhoffLMO<4>{}, settings);
    const gpuboscia::Result r2 = gpuboscia::solve_with_algorithm(prob, obj, BoxLMO{}, settings, FrankWolfePolicy{});
    std::printf("%g %zu %d %g %d %g %d %d %d %d %g %g\n", v, x.size(), nodes, bound, it, gap, conv, tol, tl, b,
                r1.objective, r2.dual_bound);
    return 0;
}

int main(int argc, char**) {
    // never reached in the check (it only compiles and links); argc keeps the call live
    return argc > 99 ? run(nullptr, nullptr) : 0;
}
