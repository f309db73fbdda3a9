// Scheduling order of the host branch-and-bound engine through the drop-in
// headers, as the reference's tests assert it (tests/test_pipeline.cu:
// 723-789 and 791-836), and the same optimum afterwards:
//  * a completed slot is refilled with the next full batch before the CPU
//    post-processes the batch it held;
//  * with an empty frontier, a completed batch's children are dispatched
//    before that batch is post-processed, the root is branched once, and the
//    integer optimum 0.5 and a valid bound survive (with the supplied exact
//    lower bound too).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <vector>

#include <gpuboscia/dense_quadratic_objectives.h>
#include <gpuboscia/gpuboscia.h>
#include <gpuboscia/lmo.h>

static int failed = 0;
#define CHECK(c)                                                        \
    do {                                                                \
        if (!(c)) { std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c); ++failed; } \
    } while (0)

static double* upload(const std::vector<double>& h) {
    double* d = nullptr;
    if (cudaMalloc(&d, h.size() * sizeof(double)) != cudaSuccess) throw std::runtime_error("cudaMalloc");
    cudaMemcpy(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice);
    return d;
}

static DeviceResidentConfig config(int batch, int streams) {
    DeviceResidentConfig cfg;
    cfg.gpu_batch_size = batch;
    cfg.num_streams = streams;
    cfg.gpu_max_iters = 50000;
    cfg.gpu_eps = 1e-6;
    return cfg;
}

// first index of an event of this type and generation on the slot (-1: any slot)
static size_t find_event(const std::vector<DRSSchedulingEvent>& ev, DRSSchedulingEventType t, std::uint64_t gen,
                         int slot) {
    for (size_t i = 0; i < ev.size(); ++i)
        if (ev[i].type == t && ev[i].generation == gen && (slot < 0 || ev[i].slot_id == slot)) return i;
    return ev.size();
}

int main() {
    // f(x) = ||x - c||^2 over binaries in two variables (the ILS form, Q = I)
    using Objective = ILSGlobalCachedObjective<2>;
    double* dQ = upload({1, 0, 0, 1});
    {
        const std::vector<double> c = {0.4, 0.6};
        double* dc = upload(c);
        Objective obj{dQ, dc, c[0] * c[0] + c[1] * c[1]};
        Problem prob;
        prob.n_vars = 2;
        prob.lb = {0, 0};
        prob.ub = {1, 1};
        prob.int_vars = {0, 1};
        std::vector<DRSSchedulingEvent> events;
        DeviceResidentHybridSolver<Objective, FrankWolfePolicy> solver(
            prob, obj, FrankWolfePolicy{},
            [](const Node& p, int& id, const std::vector<double>& x, const std::vector<int>& iv) {
                return branch_pow2(p, id, x, iv, 3);
            },
            config(2, 1));
        solver.set_scheduling_callback([&](const DRSSchedulingEvent& e) { events.push_back(e); });
        // four fixed integral nodes: two full batches queued before the solve
        const std::vector<std::vector<double>> points = {{0, 0}, {0, 1}, {1, 0}, {1, 1}};
        for (int i = 0; i < 4; ++i) {
            Node nd(i, -1, 0, points[i], points[i]);
            nd.dual_bound = -1e300;
            solver.push(nd);
        }
        solver.solve();
        const size_t detached = find_event(events, DRSSchedulingEventType::CompletionDetached, 1, 0);
        const size_t refill = find_event(events, DRSSchedulingEventType::Dispatched, 2, 0);
        const size_t post = find_event(events, DRSSchedulingEventType::PostprocessStarted, 1, 0);
        std::printf("refill order: detached %zu dispatched %zu postprocess %zu of %zu events\n", detached, refill,
                    post, events.size());
        CHECK(detached < events.size() && refill < events.size() && post < events.size());
        CHECK(detached < refill && refill < post);
        CHECK(std::fabs(solver.incumbent_value() - 0.32) < 1e-9);   // x = (0, 1): .16 + .16
        cudaFree(dc);
    }
    {
        const std::vector<double> c = {0.5, 0.5};
        double* dc = upload(c);
        Objective obj{dQ, dc, 0.5};
        Problem prob;
        prob.n_vars = 2;
        prob.lb = {0, 0};
        prob.ub = {1, 1};
        prob.int_vars = {0, 1};
        for (double root_bound : {-1e300, 0.5}) {
            std::vector<DRSSchedulingEvent> events;
            int root_branches = 0;
            DeviceResidentHybridSolver<Objective, FrankWolfePolicy> solver(
                prob, obj, FrankWolfePolicy{},
                [&](const Node& p, int& id, const std::vector<double>& x, const std::vector<int>& iv) {
                    if (p.id == 0) ++root_branches;
                    return branch_pow2(p, id, x, iv, 3);
                },
                config(2, 1));
            solver.set_scheduling_callback([&](const DRSSchedulingEvent& e) { events.push_back(e); });
            Node root(0, -1, 0, prob.lb, prob.ub);
            root.dual_bound = root_bound;
            solver.push(root);
            solver.solve();
            const size_t children = find_event(events, DRSSchedulingEventType::Dispatched, 2, -1);
            const size_t post = find_event(events, DRSSchedulingEventType::PostprocessStarted, 1, -1);
            std::printf("root bound %g: children dispatched %zu, root postprocess %zu of %zu events; "
                        "root branched %d time(s); incumbent %.12f, bound %.12f\n",
                        root_bound, children, post, events.size(), root_branches, solver.incumbent_value(),
                        solver.dual_bound());
            CHECK(children < post && post < events.size());
            CHECK(root_branches == 1);
            CHECK(std::fabs(solver.incumbent_value() - 0.5) < 1e-6);
            CHECK(solver.dual_bound() <= solver.incumbent_value() + 1e-6);
        }
        cudaFree(dc);
    }
    cudaFree(dQ);
    std::printf("%d failed\n", failed);
    return failed ? 1 : 0;
}
