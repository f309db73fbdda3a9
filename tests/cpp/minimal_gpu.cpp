// The reference's examples/minimal.cu (min (x0-.3)^2 + (x1-.7)^2 over binaries:
// x = [0, 1], f = .18) through the C++ drop-in headers, once with the host
// frontier and once with the device frontier; and a graph-matching pair of
// order 5 solved both ways to the same certified optimum; a small
// sparse-Sharpe portfolio through the reference's LinkedCardinalityLMO; and
// the weighted-clique example's model over EqualitySimplexLMO.
#include <cuda_runtime.h>

#include <algorithm>
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

template <class T>
static T* upload(const std::vector<T>& h) {
    T* d = nullptr;
    if (cudaMalloc(&d, h.size() * sizeof(T)) != cudaSuccess) throw std::runtime_error("cudaMalloc");
    cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
    return d;
}

int main() {
    double* dQ = upload<double>({2, 0, 0, 2});
    double* dc = upload<double>({-.6, -1.4});
    GlobalCachedDenseQuadraticObjective<2> obj(dQ, dc, 1.0, 1.0, .58);
    Problem prob;
    prob.n_vars = 2;
    prob.lb = {0, 0};
    prob.ub = {1, 1};
    prob.int_vars = {0, 1};
    for (int dev = 0; dev < 2; ++dev) {
        auto s = gpuboscia::create_default_settings();
        s.line_search.kind = LineSearchKind::QuadraticExact;
        s.natural_lower_bound = 0;
        s.time_limit_seconds = 10;
        s.device.device_frontier = dev != 0;
        const auto r = gpuboscia::solve(prob, obj, BoxLMO{}, s);
        std::printf("minimal device_frontier=%d: f=%.12f x=[%g, %g] nodes=%d\n", dev, r.objective,
                    r.x.size() > 0 ? r.x[0] : -1.0, r.x.size() > 1 ? r.x[1] : -1.0, r.nodes_processed);
        CHECK(r.x.size() == 2 && r.x[0] == 0.0 && r.x[1] == 1.0);
        CHECK(std::fabs(r.objective - .18) < 1e-8);
    }
    {
        auto s = gpuboscia::create_default_settings();
        s.device.device_frontier = true;
        s.branch = [](const Node& p, int& id, const std::vector<double>& x, const std::vector<int>& iv) {
            return branch_pow2(p, id, x, iv);
        };
        bool threw = false;
        try {
            gpuboscia::solve(prob, obj, BoxLMO{}, s);
        } catch (const std::invalid_argument&) {
            threw = true;
        }
        CHECK(threw);
    }
    // graph matching: A = path 0-1-2-3-4, B = star around 0 (not isomorphic)
    const int m = 5;
    std::vector<double> A(m * m, 0.0), B(m * m, 0.0);
    for (int i = 0; i + 1 < m; ++i) A[i * m + i + 1] = A[(i + 1) * m + i] = 1;
    for (int i = 1; i < m; ++i) B[i] = B[i * m] = 1;
    double* dA = upload(A);
    double* dB = upload(B);
    GraphMatchingObjective<m> gm(dA, dB, 1.0);
    Problem gp;
    gp.n_vars = m * m;
    gp.lb.assign(m * m, 0.0);
    gp.ub.assign(m * m, 1.0);
    for (int e = 0; e < m * m; ++e) gp.int_vars.push_back(e);
    double obj_val[2] = {0, 0};
    for (int dev = 0; dev < 2; ++dev) {
        auto s = gpuboscia::create_default_settings();
        s.line_search.kind = LineSearchKind::QuadraticExact;
        s.natural_lower_bound = 0;
        s.time_limit_seconds = 30;
        s.device.gpu_batch_size = 16;
        s.device.num_streams = 1;
        s.device.rel_gap_tol = 1e-9;
        s.device.device_frontier = dev != 0;
        const auto r = gpuboscia::solve(gp, gm, BirkhoffLMO<m>{}, s);
        std::printf("graph pair device_frontier=%d: f=%.12f bound=%.12f nodes=%d\n", dev, r.objective,
                    r.dual_bound, r.nodes_processed);
        CHECK(!r.reached_time_limit && r.objective - r.dual_bound <= 1e-6);
        obj_val[dev] = r.objective;
    }
    CHECK(std::fabs(obj_val[0] - obj_val[1]) <= 1e-9);

    // sparse Sharpe (examples/sparse_sharpe.cu): 3 assets padded to 4, at most
    // one; min 0.5 v'Hv - mu'v with H = I, mu = (.5, .3, .1): v = (.5, 0, 0),
    // f = -0.125, y = (1, 0, 0)
    constexpr int MaxAssets = 4, Vars = 2 * MaxAssets;
    std::vector<double> Q(Vars * Vars, 0.0), lin(Vars, 0.0);
    for (int i = 0; i < 3; ++i) Q[i * Vars + i] = 1.0;
    lin[0] = -.5; lin[1] = -.3; lin[2] = -.1;
    double* dQs = upload(Q);
    double* dls = upload(lin);
    double* dU = upload<double>({10.0, 10.0, 10.0});
    GlobalCachedDenseQuadraticObjective<Vars> sharpe(dQs, dls);
    LinkedCardinalityLMO linked{3, 1, dU, nullptr, nullptr};
    Problem sp;
    sp.n_vars = Vars;
    sp.lb.assign(Vars, 0.0);
    sp.ub.assign(Vars, 0.0);
    for (int i = 0; i < 3; ++i) {
        sp.ub[i] = 10.0;
        sp.ub[MaxAssets + i] = 1.0;
        sp.int_vars.push_back(MaxAssets + i);
    }
    for (int dev = 0; dev < 2; ++dev) {
        auto s = gpuboscia::create_default_settings();
        s.line_search.kind = LineSearchKind::QuadraticExact;
        s.natural_lower_bound = -0.5 * (.25 + .09 + .01);
        s.time_limit_seconds = 30;
        s.device.gpu_batch_size = 16;
        s.device.rel_gap_tol = 1e-9;
        s.device.device_frontier = dev != 0;
        const auto r = gpuboscia::solve(sp, sharpe, linked, s);
        std::printf("sparse sharpe device_frontier=%d: f=%.12f y=[%g %g %g] nodes=%d\n", dev, r.objective,
                    r.x.size() == Vars ? r.x[MaxAssets] : -1.0, r.x.size() == Vars ? r.x[MaxAssets + 1] : -1.0,
                    r.x.size() == Vars ? r.x[MaxAssets + 2] : -1.0, r.nodes_processed);
        CHECK(std::fabs(r.objective + 0.125) <= 1e-6);
        CHECK(r.x.size() == Vars && r.x[MaxAssets] == 1.0 && r.x[MaxAssets + 1] == 0.0 && r.x[MaxAssets + 2] == 0.0);
    }

    // weighted clique (examples/weighted_clique.cu): 20 vertices, exactly 5;
    // f = 2 sum_{i<j} (1 - w_ij) x_i x_j + lam sum x_i (x_i - 1), lam = 19,
    // over EqualitySimplexLMO<20> with integer variables, DICG; the optimum is
    // checked against enumeration of all 5-subsets
    constexpr int Vc = 20, Kc = 5;
    std::vector<double> W(Vc * Vc, 0.0), Qc(Vc * Vc, 0.0), lc(Vc, -(Vc - 1.0));
    unsigned long long state = 88172645463325252ull;   // xorshift64 weights in [0, 1)
    for (int i = 0; i < Vc; ++i)
        for (int j = i + 1; j < Vc; ++j) {
            state ^= state << 13; state ^= state >> 7; state ^= state << 17;
            W[i * Vc + j] = W[j * Vc + i] = (double)(state >> 11) * 0x1.0p-53;
        }
    for (int i = 0; i < Vc; ++i)
        for (int j = 0; j < Vc; ++j) Qc[i * Vc + j] = i == j ? 2.0 * (Vc - 1.0) : 2.0 * (1.0 - W[i * Vc + j]);
    double best = 1e300;
    for (int a = 0; a < Vc; ++a) for (int b = a + 1; b < Vc; ++b) for (int c = b + 1; c < Vc; ++c)
        for (int d = c + 1; d < Vc; ++d) for (int e = d + 1; e < Vc; ++e) {
            const int S[Kc] = {a, b, c, d, e};
            double f = 0.0;
            for (int p = 0; p < Kc; ++p)
                for (int q = p + 1; q < Kc; ++q) f += Qc[S[p] * Vc + S[q]];
            best = std::min(best, f);
        }
    double* dQc = upload(Qc);
    double* dlc = upload(lc);
    GlobalCachedDenseQuadraticObjective<Vc, 32> clique(dQc, dlc, 1.0, 1.0, 0.0);
    Problem cp;
    cp.n_vars = Vc;
    cp.lb.assign(Vc, 0.0);
    cp.ub.assign(Vc, 1.0);
    for (int i = 0; i < Vc; ++i) cp.int_vars.push_back(i);
    EqualitySimplexLMO<Vc> card((double)Kc, Vc, cp.int_vars);
    for (int dev = 0; dev < 2; ++dev) {
        auto s = gpuboscia::create_default_settings();
        s.algorithm = FWAlgorithmKind::DICG;
        s.time_limit_seconds = 60;
        s.device.gpu_batch_size = 1024;
        s.device.num_streams = 2;
        s.device.gpu_max_iters = 1000;
        s.device.abs_gap_tol = 1e-7;
        s.device.rel_gap_tol = 1e-3;
        s.device.device_frontier = dev != 0;
        s.natural_lower_bound = (Vc - 1.0) * ((double)Kc * Kc / Vc - Kc);
        const auto r = gpuboscia::solve(cp, clique, card, s);
        double chosen = 0.0;
        for (double v : r.x) chosen += v;
        std::printf("weighted clique device_frontier=%d: f=%.12f enumerated=%.12f bound=%.12f nodes=%d\n", dev,
                    r.objective, best, r.dual_bound, r.nodes_processed);
        CHECK(!r.reached_time_limit && r.x.size() == Vc && chosen == Kc);
        CHECK(r.objective - best <= 1e-3 * std::fabs(best) + 1e-7 && r.dual_bound <= best + 1e-9);
    }
    cudaFree(dQc);
    cudaFree(dlc);
    cudaFree(dQs);
    cudaFree(dls);
    cudaFree(dU);
    cudaFree(dQ);
    cudaFree(dc);
    cudaFree(dA);
    cudaFree(dB);
    std::printf("%d failed\n", failed);
    return failed ? 1 : 0;
}
