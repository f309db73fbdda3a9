// The free DICG helpers of lmo_dicg.h (the reference's lmo_dicg.h:8-200) on
// cases read from stdin, one per line, for a differential check (the same
// source compiled against each set of headers):
//   approx a b                                 -> dicg_isapprox
//   feas rhs n v[n]                            -> equality / unit simplex linear feasibility
//   infeas rhs n a[n] x[n]                     -> unit_simplex_inface_feasible_cpu
//   box n g[n] x[n] lb[n] ub[n]                -> box_inface_lmo_cpu, box_dicg_maximum_step_cpu(g, ...)
//   simplex full rhs n ints[n] g[n] x[n] lb[n] ub[n]
//        -> unit_simplex_inface_lmo_cpu, unit_simplex_dicg_maximum_step_cpu(g, ...)
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

#include <gpuboscia/lmo_dicg.h>

static double num() {
    std::string t;
    std::cin >> t;
    return std::strtod(t.c_str(), nullptr);
}

static std::vector<double> nums(int n) {
    std::vector<double> v(n);
    for (double& e : v) e = num();
    return v;
}

static void emit(const std::vector<double>& v) {
    for (double e : v) std::printf(" %.17g", e);
}

int main() {
    std::string op;
    while (std::cin >> op) {
        if (op == "approx") {
            const double a = num(), b = num();
            std::printf("%d\n", dicg_isapprox(a, b) ? 1 : 0);
        } else if (op == "feas") {
            const double rhs = num();
            int n;
            std::cin >> n;
            const auto v = nums(n);
            std::printf("%d %d\n", equality_simplex_linear_feasible_cpu(rhs, v) ? 1 : 0,
                        unit_simplex_linear_feasible_cpu(rhs, v) ? 1 : 0);
        } else if (op == "infeas") {
            const double rhs = num();
            int n;
            std::cin >> n;
            const auto a = nums(n), x = nums(n);
            std::printf("%d\n", unit_simplex_inface_feasible_cpu(rhs, a, x) ? 1 : 0);
        } else if (op == "box") {
            int n;
            std::cin >> n;
            const auto g = nums(n), x = nums(n), lb = nums(n), ub = nums(n);
            std::vector<double> a(n, 0.0);
            box_inface_lmo_cpu(g, x, lb, ub, a);
            emit(a);
            std::printf(" %.17g\n", box_dicg_maximum_step_cpu(g, x, lb, ub));
        } else if (op == "simplex") {
            int full, n;
            std::cin >> full;
            const double rhs = num();
            std::cin >> n;
            std::vector<unsigned char> ints(n);
            for (auto& e : ints) {
                int v;
                std::cin >> v;
                e = (unsigned char)v;
            }
            const auto g = nums(n), x = nums(n), lb = nums(n), ub = nums(n);
            std::vector<double> a(n, 0.0);
            unit_simplex_inface_lmo_cpu(rhs, ints, g, x, lb, ub, a, 1e-6, 1e-4, full != 0);
            emit(a);
            std::printf(" %.17g\n", unit_simplex_dicg_maximum_step_cpu(rhs, ints, g, x, lb, ub, 1e-6, full != 0));
        }
    }
    return 0;
}
