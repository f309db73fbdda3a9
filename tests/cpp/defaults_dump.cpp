// Prints the public defaults and names of the solver interface -- Settings,
// Result, DeviceResidentConfig, LineSearchOptions, the enums and their name
// strings, the scheduling event types -- one per line, for a differential
// check of two implementations of gpuboscia.cuh (the same source compiled
// against each). Only the reference's own fields are named, so a field that
// is missing or renamed fails to compile.
#include <cstdio>
#include <string>

#include <gpuboscia/gpuboscia.cuh>

static void line(const char* name, double v) { std::printf("%s %.17g\n", name, v); }

int main() {
    const auto s = gpuboscia::create_default_settings();
    line("settings.algorithm", (double)static_cast<int>(s.algorithm));
    line("settings.line_search.kind", (double)static_cast<int>(s.line_search.kind));
    line("settings.line_search.secant_iters", s.line_search.secant_iters);
    line("settings.line_search.secant_tol", s.line_search.secant_tol);
    line("settings.line_search.secant_denom_eps", s.line_search.secant_denom_eps);
    line("settings.branch_set", s.branch ? 1.0 : 0.0);
    line("settings.progress_set", s.progress ? 1.0 : 0.0);
    line("settings.time_limit_seconds", s.time_limit_seconds);
    line("settings.natural_lower_bound", s.natural_lower_bound);
    line("settings.root_initial_point.size", (double)s.root_initial_point.size());
    line("settings.root_initial_point_feasible_set", s.root_initial_point_feasible ? 1.0 : 0.0);

    const DeviceResidentConfig& d = s.device;
    line("device.gpu_batch_size", d.gpu_batch_size);
    line("device.num_streams", d.num_streams);
    line("device.gpu_block_threads", d.gpu_block_threads);
    line("device.gpu_max_iters", d.gpu_max_iters);
    line("device.gpu_eps", d.gpu_eps);
    line("device.gpu_eps_decay", d.gpu_eps_decay);
    line("device.gpu_eps_min", d.gpu_eps_min);
    line("device.integer_tol", d.integer_tol);
    line("device.abs_gap_tol", d.abs_gap_tol);
    line("device.rel_gap_tol", d.rel_gap_tol);
    line("device.dicg_oracle_parallelism", (double)static_cast<int>(d.dicg_oracle_parallelism));
    line("device.dicg_paired_occupancy_fraction", d.dicg_paired_occupancy_fraction);
    line("device.execution_mode", (double)static_cast<int>(d.execution_mode));
    line("device.blocks_per_node", d.blocks_per_node);
    using P = DeviceResidentConfig::DICGOracleParallelism;
    line("enum.DICGOracleParallelism", static_cast<int>(P::Auto) * 100 + static_cast<int>(P::Serial) * 10
                                           + static_cast<int>(P::Paired));
    line("enum.FWExecutionMode", static_cast<int>(FWExecutionMode::SingleBlock) * 10
                                     + static_cast<int>(FWExecutionMode::MultiBlock));

    const gpuboscia::Result r{};
    line("result.objective", r.objective);
    line("result.x.size", (double)r.x.size());
    line("result.dual_bound", r.dual_bound);
    line("result.nodes_processed", r.nodes_processed);
    line("result.elapsed_seconds", r.elapsed_seconds);
    line("result.reached_tolerance", r.reached_tolerance ? 1.0 : 0.0);
    line("result.reached_time_limit", r.reached_time_limit ? 1.0 : 0.0);

    const LineSearchKind kinds[] = {LineSearchKind::OpenLoop, LineSearchKind::ScaledOpenLoop,
                                    LineSearchKind::SafeguardedScaledOpenLoop, LineSearchKind::Secant,
                                    LineSearchKind::QuadraticExact};
    for (LineSearchKind k : kinds)
        std::printf("line_search %d %s\n", static_cast<int>(k), line_search_name(k));
    for (FWAlgorithmKind a : {FWAlgorithmKind::FrankWolfe, FWAlgorithmKind::DICG})
        std::printf("algorithm %d %s\n", static_cast<int>(a), fw_algorithm_name(a));
    line("enum.DRSSchedulingEventType", static_cast<int>(DRSSchedulingEventType::Dispatched) * 100
                                            + static_cast<int>(DRSSchedulingEventType::CompletionDetached) * 10
                                            + static_cast<int>(DRSSchedulingEventType::PostprocessStarted));
    return 0;
}
