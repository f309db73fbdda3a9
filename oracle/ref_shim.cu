// ref_shim.cu -- TEST INFRASTRUCTURE. Exposes the reference project's own
// CPU functions through a C ABI so the oracle can be pinned against them.
// Built by oracle/build.sh from the reference headers where they lie
// (nothing is copied); the output goes to oracle/_ref/ and is never shipped.
//
// Wrapped reference functions (reference project paths):
//   BoxLMO::compute_v_cpu / compute_inface_v_cpu / dicg_maximum_step_cpu
//       include/gpuboscia/lmo.cuh:225-260
//   UnitSimplexLMO<MaxN,Eq>::compute_v_cpu / compute_inface_v_cpu /
//       dicg_maximum_step_cpu                       lmo.cuh:399-482
//   BirkhoffLMO<Order>::compute_v_cpu / compute_inface_v_cpu / CPU Hungarian
//                                                   lmo.cuh:958-1171
//   unit_simplex_inface_lmo_cpu etc.                include/gpuboscia/lmo_dicg.h
//   certified_fw_lower_bound, gap_*, depth_dependent_tolerance
//                                                   include/gpuboscia/gap_utils.h
//   quadratic_exact_step                            include/gpuboscia/line_search_options.h:53-63
//   top_k_infeasible, branch_pow2                   include/gpuboscia/branching.h
#include <gpuboscia/lmo.cuh>
#include <gpuboscia/gap_utils.h>
#include <gpuboscia/branching.h>
#include <gpuboscia/line_search_options.h>

#include <cstring>
#include <vector>

namespace {
constexpr int kSimplexMax = 512;

template <int Order>
int birkhoff(int mode, const double* cost, const double* x, const double* lb,
             const double* ub, double* out) {
    constexpr int n = Order * Order;
    BirkhoffLMO<Order> lmo;
    std::vector<double> c(cost, cost + n), l(lb, lb + n), u(ub, ub + n), v(n, 0.0);
    if (mode == 0) {
        lmo.compute_v_cpu(c, l, u, v);
    } else {
        std::vector<double> xv(x, x + n);
        lmo.compute_inface_v_cpu(c, xv, l, u, v);
    }
    std::memcpy(out, v.data(), n * sizeof(double));
    return 0;
}

template <bool Eq>
int simplex(int mode, int n, double rhs, const int* int_vars, int n_int,
            const double* grad, const double* x, const double* lb, const double* ub,
            double* out, double* step) {
    if (n > kSimplexMax) return -1;
    UnitSimplexLMO<kSimplexMax, Eq> lmo(rhs, n, std::vector<int>(int_vars, int_vars + n_int));
    std::vector<double> g(grad, grad + n), l(lb, lb + n), u(ub, ub + n), v(n, 0.0);
    if (mode == 0) {
        lmo.compute_v_cpu(g, l, u, v);
    } else {
        std::vector<double> xv(x, x + n);
        lmo.compute_inface_v_cpu(g, xv, l, u, v);
        if (step) {
            // away vertex a of the negated direction's forward oracle pair
            std::vector<double> ng(n), f(n, 0.0), d(n);
            for (int j = 0; j < n; ++j) ng[j] = -g[j];
            lmo.compute_v_cpu(ng, l, u, f);
            for (int j = 0; j < n; ++j) d[j] = v[j] - f[j];
            *step = lmo.dicg_maximum_step_cpu(d, xv, l, u);
        }
    }
    std::memcpy(out, v.data(), n * sizeof(double));
    return 0;
}
}  // namespace

extern "C" {

int ref_birkhoff_lmo(int order, int mode, const double* cost, const double* x,
                     const double* lb, const double* ub, double* out) {
    switch (order) {
    case 1: return birkhoff<1>(mode, cost, x, lb, ub, out);
    case 2: return birkhoff<2>(mode, cost, x, lb, ub, out);
    case 3: return birkhoff<3>(mode, cost, x, lb, ub, out);
    case 4: return birkhoff<4>(mode, cost, x, lb, ub, out);
    case 5: return birkhoff<5>(mode, cost, x, lb, ub, out);
    case 6: return birkhoff<6>(mode, cost, x, lb, ub, out);
    case 7: return birkhoff<7>(mode, cost, x, lb, ub, out);
    case 8: return birkhoff<8>(mode, cost, x, lb, ub, out);
    case 12: return birkhoff<12>(mode, cost, x, lb, ub, out);
    case 16: return birkhoff<16>(mode, cost, x, lb, ub, out);
    case 32: return birkhoff<32>(mode, cost, x, lb, ub, out);
    case 33: return birkhoff<33>(mode, cost, x, lb, ub, out);
    case 36: return birkhoff<36>(mode, cost, x, lb, ub, out);
    case 97: return birkhoff<97>(mode, cost, x, lb, ub, out);
    case 120: return birkhoff<120>(mode, cost, x, lb, ub, out);
    case 129: return birkhoff<129>(mode, cost, x, lb, ub, out);
    case 400: return birkhoff<400>(mode, cost, x, lb, ub, out);
    default: return -1;
    }
}

int ref_simplex_lmo(int equality, int mode, int n, double rhs, const int* int_vars,
                    int n_int, const double* grad, const double* x, const double* lb,
                    const double* ub, double* out, double* step) {
    return equality ? simplex<true>(mode, n, rhs, int_vars, n_int, grad, x, lb, ub, out, step)
                    : simplex<false>(mode, n, rhs, int_vars, n_int, grad, x, lb, ub, out, step);
}

int ref_box_lmo(int mode, int n, const double* grad, const double* x, const double* lb,
                const double* ub, double* out, double* step) {
    BoxLMO lmo;
    std::vector<double> g(grad, grad + n), l(lb, lb + n), u(ub, ub + n), v(n, 0.0);
    if (mode == 0) {
        lmo.compute_v_cpu(g, l, u, v);
    } else {
        std::vector<double> xv(x, x + n);
        lmo.compute_inface_v_cpu(g, xv, l, u, v);
        if (step) {
            std::vector<double> ng(n), f(n, 0.0), d(n);
            for (int j = 0; j < n; ++j) ng[j] = -g[j];
            lmo.compute_v_cpu(ng, l, u, f);
            for (int j = 0; j < n; ++j) d[j] = v[j] - f[j];
            *step = lmo.dicg_maximum_step_cpu(d, xv, l, u);
        }
    }
    std::memcpy(out, v.data(), n * sizeof(double));
    return 0;
}

double ref_certified_fw_lower_bound(double inherited, double primal, double gap) {
    return gpuboscia::certified_fw_lower_bound(inherited, primal, gap);
}
double ref_gap_relative(double b, double i) { return gpuboscia::gap_relative(b, i); }
double ref_gap_absolute(double b, double i) { return gpuboscia::gap_absolute(b, i); }
int ref_gap_within_tolerance(double b, double i, double a, double r) {
    return gpuboscia::gap_within_tolerance(b, i, a, r) ? 1 : 0;
}
double ref_depth_dependent_tolerance(double root, double decay, double mn, int depth) {
    return gpuboscia::depth_dependent_tolerance(root, decay, mn, depth);
}
double ref_quadratic_exact_step(double gap, double curv, double maximum) {
    return quadratic_exact_step(gap, curv, maximum);
}

// branch_pow2: children written as (lb,ub) pairs into out_lb/out_ub [max_children*n]
int ref_branch_pow2(int n, const double* lb, const double* ub, const double* x,
                    const int* int_vars, int n_int, int k, double tol,
                    double* out_lb, double* out_ub) {
    Node parent(0, -1, 0, std::vector<double>(lb, lb + n), std::vector<double>(ub, ub + n));
    int next = 1;
    auto ch = branch_pow2(parent, next, std::vector<double>(x, x + n),
                          std::vector<int>(int_vars, int_vars + n_int), k, tol);
    for (size_t c = 0; c < ch.size(); ++c) {
        std::memcpy(out_lb + c * n, ch[c].lb.data(), n * sizeof(double));
        std::memcpy(out_ub + c * n, ch[c].ub.data(), n * sizeof(double));
    }
    return (int)ch.size();
}

}  // extern "C"
