// gpuboscia::solve's argument checks (gpuboscia.cuh:56-170 of the
// reference): algorithm and line-search combinations, the quadratic-exact
// requirement on the objective, the root point, and the solver's own
// configuration checks reached through solve. One line per case: the
// exception type and message ("cuda" for a CUDA failure, whose text names a
// source line). For a differential check, the same source compiled with nvcc
// against each set of headers; without a GPU every case ends before or at
// the first CUDA call.
#include <cstdio>
#include <functional>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include <gpuboscia/dense_quadratic_objectives.cuh>
#include <gpuboscia/gpuboscia.cuh>

// a device objective without curvature support (no quadratic-exact step)
struct PlainObjective {
    static constexpr int n_vars = 2, block_threads = 32, shared_bytes = 0;
    __device__ void prepare_block(int, unsigned char*) const {}
    __device__ void grad(int tid, const double* x, double* g, unsigned char*) const {
        for (int j = tid; j < n_vars; j += blockDim.x) g[j] = 2.0 * (x[j] - 0.5);
        __syncthreads();
    }
    __device__ double value_local(int tid, const double* x, unsigned char*) const {
        double v = 0.0;
        for (int j = tid; j < n_vars; j += blockDim.x) v += (x[j] - 0.5) * (x[j] - 0.5);
        return v;
    }
};

template <class Objective>
static void attempt(const char* name, const Objective& obj,
                    std::function<void(gpuboscia::Settings&, Problem&)> change) {
    Problem prob{2, {0, 0}, {1, 1}, {0, 1}};
    auto s = gpuboscia::create_default_settings();
    change(s, prob);
    try {
        gpuboscia::solve(prob, obj, BoxLMO{}, s);
        std::printf("%s returned\n", name);
    } catch (const std::invalid_argument& e) {
        std::printf("%s invalid_argument: %s\n", name, e.what());
    } catch (const std::runtime_error& e) {
        const std::string m = e.what();
        std::printf("%s runtime_error: %s\n", name, m.rfind("CUDA ", 0) == 0 ? "cuda" : m.c_str());
    }
}

int main() {
    const ILSGlobalCachedObjective<2> ils{};
    attempt("fw_scaled_open_loop", ils, [](auto& s, auto&) {
        s.algorithm = FWAlgorithmKind::FrankWolfe;
        s.line_search.kind = LineSearchKind::ScaledOpenLoop;
    });
    attempt("fw_safeguarded", ils, [](auto& s, auto&) {
        s.algorithm = FWAlgorithmKind::FrankWolfe;
        s.line_search.kind = LineSearchKind::SafeguardedScaledOpenLoop;
    });
    attempt("quadratic_exact_without_curvature", PlainObjective{},
            [](auto& s, auto&) { s.line_search.kind = LineSearchKind::QuadraticExact; });
    attempt("root_point_wrong_size", ils, [](auto& s, auto&) { s.root_initial_point = {0.5}; });
    attempt("root_point_out_of_bounds", ils, [](auto& s, auto&) { s.root_initial_point = {0.5, 1.5}; });
    attempt("root_point_nan", ils, [](auto& s, auto&) {
        s.root_initial_point = {0.5, std::numeric_limits<double>::quiet_NaN()};
    });
    attempt("root_point_rejected_by_validator", ils, [](auto& s, auto&) {
        s.root_initial_point = {0.5, 0.5};
        s.root_initial_point_feasible = [](const std::vector<double>&, const std::vector<double>&,
                                           const std::vector<double>&, double) { return false; };
    });
    attempt("batch0", ils, [](auto& s, auto&) { s.device.gpu_batch_size = 0; });
    attempt("eps_nan", ils, [](auto& s, auto&) { s.device.gpu_eps = std::numeric_limits<double>::quiet_NaN(); });
    attempt("time_limit0", ils, [](auto& s, auto&) { s.time_limit_seconds = 0.0; });
    attempt("int_var_out_of_range", ils, [](auto&, auto& p) { p.int_vars = {0, 5}; });
    attempt("size_mismatch", ils, [](auto&, auto& p) {
        p.n_vars = 3;
        p.lb = {0, 0, 0};
        p.ub = {1, 1, 1};
    });
    attempt("root_point_before_config", ils, [](auto& s, auto&) {   // the root point is checked first
        s.root_initial_point = {0.5};
        s.device.gpu_batch_size = 0;
    });
    attempt("line_search_before_root_point", ils, [](auto& s, auto&) {
        s.algorithm = FWAlgorithmKind::FrankWolfe;
        s.line_search.kind = LineSearchKind::ScaledOpenLoop;
        s.root_initial_point = {0.5};
    });
    return 0;
}
