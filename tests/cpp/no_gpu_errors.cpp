// A CUDA failure surfacing through the C++ drop-in: on a machine where every
// CUDA call fails (no usable GPU), gpuboscia::solve throws std::runtime_error
// with CUDA's message -- on the host and the device frontier -- and a bad
// setting still throws std::invalid_argument first. Prints one line per case.
#include <cstdio>
#include <stdexcept>

#include <gpuboscia/dense_quadratic_objectives.cuh>
#include <gpuboscia/gpuboscia.cuh>
#include <gpuboscia/lmo.cuh>

int main() {
    GlobalCachedDenseQuadraticObjective<2> obj(nullptr, nullptr);
    Problem prob;
    prob.n_vars = 2;
    prob.lb = {0, 0};
    prob.ub = {1, 1};
    prob.int_vars = {0, 1};
    int runtime_errors = 0;
    for (int dev = 0; dev < 2; ++dev) {
        auto s = gpuboscia::create_default_settings();
        s.time_limit_seconds = 5;
        s.device.device_frontier = dev != 0;
        try {
            gpuboscia::solve(prob, obj, BoxLMO{}, s);
            std::printf("frontier=%d returned\n", dev);
        } catch (const std::invalid_argument& e) {
            std::printf("frontier=%d invalid_argument %s\n", dev, e.what());
        } catch (const std::runtime_error& e) {
            std::printf("frontier=%d runtime_error %s\n", dev, e.what());
            ++runtime_errors;
        }
    }
    auto bad = gpuboscia::create_default_settings();
    bad.device.gpu_batch_size = 0;
    try {
        gpuboscia::solve(prob, obj, BoxLMO{}, bad);
        std::printf("bad settings returned\n");
    } catch (const std::invalid_argument&) {
        std::printf("bad settings invalid_argument\n");
    } catch (const std::runtime_error& e) {
        std::printf("bad settings runtime_error %s\n", e.what());
    }
    return runtime_errors == 2 ? 0 : 1;
}
