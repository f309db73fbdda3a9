// User-written device objectives (the reference's extension point: a device
// struct with n_vars, block_threads, shared_bytes, prepare_block, grad,
// value_local and optionally quadratic_curvature_local) solved through
// gpuboscia::solve, checked against the built-in kinds:
//   * a separable quadratic over BoxLMO (the minimal example's answer x = [0, 1],
//     f = .18), with the default DICG + secant settings and with FW + QE;
//   * graph matching 0.5 ||B X - X A||^2 over BirkhoffLMO, as the reference's
//     graph-isomorphism example writes it, against the built-in
//     GraphMatchingObjective(B, A, 0.5): the same certified optimum on an
//     isomorphic pair (0) and on a non-isomorphic pair;
//   * a quadratic over EqualitySimplexLMO against the built-in dense quadratic.
// Compiled by nvcc: the relaxation kernel of a user objective is a template
// instantiated here (gpuboscia/user_relax.cuh).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <random>
#include <stdexcept>
#include <vector>

#include <gpuboscia/dense_quadratic_objectives.h>
#include <gpuboscia/gpuboscia.h>
#include <gpuboscia/lmo.h>
#include <gpuboscia/user_relax.cuh>

static int failed = 0;
#define CHECK(c)                                                                          \
    do {                                                                                  \
        if (!(c)) { std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c); ++failed; } \
    } while (0)

template <class T>
static T* upload(const std::vector<T>& h) {
    T* d = nullptr;
    if (cudaMalloc(&d, h.size() * sizeof(T)) != cudaSuccess) throw std::runtime_error("cudaMalloc");
    cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
    return d;
}

// sum_j w_j (x_j - t_j)^2, block-stride like any reference objective
struct SeparableQuadratic {
    static constexpr bool supports_quadratic_exact = true;
    static constexpr int n_vars = 2;
    static constexpr int block_threads = 64;
    static constexpr int shared_bytes = 0;
    const double* target;
    __device__ void prepare_block(int, unsigned char*) const {}
    __device__ void grad(int tid, const double* x, double* g, unsigned char*) const {
        for (int j = tid; j < n_vars; j += blockDim.x) g[j] = 2.0 * (x[j] - target[j]);
    }
    __device__ double value_local(int tid, const double* x, unsigned char*) const {
        double s = 0.0;
        for (int j = tid; j < n_vars; j += blockDim.x) s += (x[j] - target[j]) * (x[j] - target[j]);
        return s;
    }
    __device__ double quadratic_curvature_local(int tid, const double* d, unsigned char*) const {
        double s = 0.0;
        for (int j = tid; j < n_vars; j += blockDim.x) s += 2.0 * d[j] * d[j];
        return s;
    }
};

// 0.5 * ||B X - X A||_F^2 over order x order X, the residual kept in the
// per-node objective workspace (shared_bytes), as the example's struct does
template <int Order, int Threads>
struct IsoObjective {
    static constexpr bool supports_quadratic_exact = true;
    static constexpr int n_vars = Order * Order;
    static constexpr int block_threads = Threads;
    static constexpr int shared_bytes = n_vars * (int)sizeof(double);
    const double* A;
    const double* B;
    __device__ double resid(const double* x, int r, int c) const {
        double s = 0.0;
        for (int k = 0; k < Order; ++k) s += B[r * Order + k] * x[k * Order + c] - x[r * Order + k] * A[k * Order + c];
        return s;
    }
    __device__ void prepare_block(int, unsigned char*) const {}
    __device__ void grad(int tid, const double* x, double* g, unsigned char* ws) const {
        double* R = reinterpret_cast<double*>(ws);
        for (int e = tid; e < n_vars; e += blockDim.x) R[e] = resid(x, e / Order, e % Order);
        __syncthreads();
        for (int e = tid; e < n_vars; e += blockDim.x) {
            const int p = e / Order, q = e % Order;
            double s = 0.0;
            for (int r = 0; r < Order; ++r) s += B[r * Order + p] * R[r * Order + q];
            for (int c = 0; c < Order; ++c) s -= R[p * Order + c] * A[q * Order + c];
            g[e] = s;
        }
        __syncthreads();
    }
    __device__ double value_local(int tid, const double* x, unsigned char*) const {
        double s = 0.0;
        for (int e = tid; e < n_vars; e += blockDim.x) {
            const double z = resid(x, e / Order, e % Order);
            s += 0.5 * z * z;
        }
        return s;
    }
    __device__ double quadratic_curvature_local(int tid, const double* d, unsigned char*) const {
        double s = 0.0;
        for (int e = tid; e < n_vars; e += blockDim.x) {
            const double z = resid(d, e / Order, e % Order);
            s += z * z;
        }
        return s;
    }
};

// 0.5 x'Qx + c'x with Q given row-major (device)
template <int N>
struct DenseQuad {
    static constexpr bool supports_quadratic_exact = true;
    static constexpr int n_vars = N;
    static constexpr int block_threads = 64;
    static constexpr int shared_bytes = 16;
    const double* Q;
    const double* c;
    __device__ void prepare_block(int, unsigned char*) const {}
    __device__ void grad(int tid, const double* x, double* g, unsigned char*) const {
        for (int i = tid; i < N; i += blockDim.x) {
            double s = c[i];
            for (int j = 0; j < N; ++j) s += Q[i * N + j] * x[j];
            g[i] = s;
        }
    }
    __device__ double value_local(int tid, const double* x, unsigned char*) const {
        double s = 0.0;
        for (int i = tid; i < N; i += blockDim.x) {
            double qx = 0.0;
            for (int j = 0; j < N; ++j) qx += Q[i * N + j] * x[j];
            s += 0.5 * x[i] * qx + c[i] * x[i];
        }
        return s;
    }
    __device__ double quadratic_curvature_local(int tid, const double* d, unsigned char*) const {
        double s = 0.0;
        for (int i = tid; i < N; i += blockDim.x) {
            double qd = 0.0;
            for (int j = 0; j < N; ++j) qd += Q[i * N + j] * d[j];
            s += d[i] * qd;
        }
        return s;
    }
};

static std::vector<double> random_graph(int m, double p, std::mt19937_64& rng) {
    std::vector<double> A((size_t)m * m, 0.0);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    for (int i = 0; i < m; ++i)
        for (int j = i + 1; j < m; ++j)
            if (U(rng) < p) A[i * m + j] = A[j * m + i] = 1.0;
    return A;
}

template <int M>
static void graph_pair(const char* name, const std::vector<double>& A, const std::vector<double>& B, bool iso) {
    double* dA = upload(A);
    double* dB = upload(B);
    Problem prob;
    prob.n_vars = M * M;
    prob.lb.assign(M * M, 0.0);
    prob.ub.assign(M * M, 1.0);
    for (int j = 0; j < M * M; ++j) prob.int_vars.push_back(j);
    for (int alg = 0; alg < 2; ++alg) {
        auto s = gpuboscia::create_default_settings();
        s.algorithm = alg ? FWAlgorithmKind::DICG : FWAlgorithmKind::FrankWolfe;
        s.line_search.kind = LineSearchKind::QuadraticExact;
        s.natural_lower_bound = 0.0;
        s.time_limit_seconds = 120;
        s.device.gpu_batch_size = 64;
        s.device.num_streams = 1;
        s.device.gpu_max_iters = 500;
        s.device.rel_gap_tol = 1e-6;
        const auto user = gpuboscia::solve(prob, IsoObjective<M, 64>{dA, dB}, BirkhoffLMO<M>{}, s);
        const auto builtin = gpuboscia::solve(prob, GraphMatchingObjective<M>(dB, dA, 0.5), BirkhoffLMO<M>{}, s);
        std::printf("%s alg=%d: user f=%.10g bound=%.10g nodes=%d | built-in f=%.10g bound=%.10g nodes=%d\n", name,
                    alg, user.objective, user.dual_bound, user.nodes_processed, builtin.objective,
                    builtin.dual_bound, builtin.nodes_processed);
        CHECK(!user.reached_time_limit && !builtin.reached_time_limit);
        CHECK(std::fabs(user.objective - builtin.objective) <= 1e-9 * (1.0 + std::fabs(builtin.objective)));
        CHECK(user.dual_bound <= user.objective + 1e-9);
        CHECK(user.x.size() == (size_t)M * M);
        if (iso) CHECK(user.objective == 0.0);
        // the incumbent is a permutation with the reported value
        int ones = 0;
        for (double v : user.x) ones += v == 1.0 ? 1 : 0;
        CHECK(ones == M);
    }
    cudaFree(dA);
    cudaFree(dB);
}

int main() {
    // separable quadratic over the box: x = [0, 1], f = .18 (targets .3, .7)
    double* dt = upload<double>({.3, .7});
    Problem box;
    box.n_vars = 2;
    box.lb = {0, 0};
    box.ub = {1, 1};
    box.int_vars = {0, 1};
    for (int mode = 0; mode < 3; ++mode) {
        auto s = gpuboscia::create_default_settings();   // mode 0: DICG + secant (the defaults)
        if (mode == 1) { s.algorithm = FWAlgorithmKind::FrankWolfe; s.line_search.kind = LineSearchKind::QuadraticExact; }
        if (mode == 2) { s.algorithm = FWAlgorithmKind::DICG; s.line_search.kind = LineSearchKind::OpenLoop; }
        s.natural_lower_bound = 0;
        s.time_limit_seconds = 30;
        const auto r = gpuboscia::solve(box, SeparableQuadratic{dt}, BoxLMO{}, s);
        std::printf("separable mode=%d: f=%.12f x=[%g, %g] nodes=%d\n", mode, r.objective,
                    r.x.size() > 0 ? r.x[0] : -1.0, r.x.size() > 1 ? r.x[1] : -1.0, r.nodes_processed);
        CHECK(r.x.size() == 2 && r.x[0] == 0.0 && r.x[1] == 1.0);
        CHECK(std::fabs(r.objective - .18) < 1e-8);
    }
    // graph matching: an isomorphic pair and a non-isomorphic pair of order 8
    std::mt19937_64 rng(2024);
    constexpr int M = 8;
    const std::vector<double> A = random_graph(M, 0.5, rng);
    std::vector<int> perm(M);
    for (int i = 0; i < M; ++i) perm[i] = (i * 5 + 3) % M;
    std::vector<double> B((size_t)M * M);
    for (int r = 0; r < M; ++r)
        for (int c = 0; c < M; ++c) B[r * M + c] = A[perm[r] * M + perm[c]];
    graph_pair<M>("isomorphic", A, B, true);
    graph_pair<M>("non-isomorphic", A, random_graph(M, 0.5, rng), false);
    // a quadratic over the equality simplex (3 of 6 binaries), against the built-in dense quadratic
    {
        constexpr int N = 6;
        std::vector<double> Q((size_t)N * N), c(N);
        std::uniform_real_distribution<double> U(-1.0, 1.0);
        std::vector<double> Mx((size_t)N * N);
        for (double& v : Mx) v = U(rng);
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
                double s = 0.0;
                for (int k = 0; k < N; ++k) s += Mx[k * N + i] * Mx[k * N + j];
                Q[i * N + j] = s / N + (i == j ? 0.1 : 0.0);
            }
        for (double& v : c) v = U(rng);
        double* dQ = upload(Q);
        double* dc = upload(c);
        Problem p;
        p.n_vars = N;
        p.lb.assign(N, 0.0);
        p.ub.assign(N, 1.0);
        for (int j = 0; j < N; ++j) p.int_vars.push_back(j);
        auto s = gpuboscia::create_default_settings();
        s.line_search.kind = LineSearchKind::QuadraticExact;
        s.time_limit_seconds = 30;
        s.device.rel_gap_tol = 1e-9;
        const EqualitySimplexLMO<N> lmo(3.0, N, p.int_vars);
        const auto user = gpuboscia::solve(p, DenseQuad<N>{dQ, dc}, lmo, s);
        const auto builtin = gpuboscia::solve(p, GlobalCachedDenseQuadraticObjective<N>(dQ, dc), lmo, s);
        std::printf("equality simplex: user f=%.12f nodes=%d | built-in f=%.12f nodes=%d\n", user.objective,
                    user.nodes_processed, builtin.objective, builtin.nodes_processed);
        CHECK(std::fabs(user.objective - builtin.objective) <= 1e-9 * (1.0 + std::fabs(builtin.objective)));
        double sum = 0.0;
        for (double v : user.x) sum += v;
        CHECK(user.x.size() == (size_t)N && std::fabs(sum - 3.0) < 1e-12);
    }
    // the device frontier and mixed precision stay with the built-in kinds
    {
        auto s = gpuboscia::create_default_settings();
        s.device.device_frontier = true;
        bool threw = false;
        try { gpuboscia::solve(box, SeparableQuadratic{dt}, BoxLMO{}, s); } catch (const std::invalid_argument&) { threw = true; }
        CHECK(threw);
    }
    std::printf("%d failed\n", failed);
    return failed ? 1 : 0;
}
