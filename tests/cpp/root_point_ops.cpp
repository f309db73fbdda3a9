// The incumbent, the root-point checks and the node feasibility predicates
// driven by a script on stdin, for a differential check of two
// implementations of atomic_incumbent.h, tree.h's validate_root_initial_point
// and bnb.h (the same source compiled against each):
//   inc value                 -> try_update(value, {value}): result, get(), get_x()
//   root kind n tol lb[n] ub[n] x[m]   (m given first: "root kind n m tol ...")
//        kind: box | simplex rhs | eqsimplex rhs | accept | reject | none
//        -> "ok" or the exception's message
//   intfeas n k tol x[n] ints[k]        -> bnb.h is_integer_feasible
//   nodefeas n k tol lb[n] ub[n] ints[k] -> bnb.h is_node_feasible
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include <gpuboscia/atomic_incumbent.h>
#include <gpuboscia/bnb.h>
#include <gpuboscia/lmo.cuh>
#include <gpuboscia/problem.h>
#include <gpuboscia/tree.h>

struct NoPointCheck {};   // an LMO type without relaxation_feasible_cpu

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

template <class L>
static void check(const Problem& p, const L& lmo, const std::vector<double>& x, double tol,
                  const gpuboscia::RootInitialPointValidator& validator = {}) {
    try {
        gpuboscia::validate_root_initial_point(p, lmo, x, validator, tol);
        std::printf("ok\n");
    } catch (const std::invalid_argument& e) {
        std::printf("err: %s\n", e.what());
    }
}

int main() {
    AtomicIncumbent inc;
    std::string op;
    while (std::cin >> op) {
        if (op == "inc") {
            const double v = num();
            const bool r = inc.try_update(v, {v});
            const auto x = inc.get_x();
            std::printf("%d %.17g %s\n", r ? 1 : 0, inc.get(), x.empty() ? "none" : std::to_string(x[0]).c_str());
        } else if (op == "intfeas" || op == "nodefeas") {
            int n = 0, k = 0;
            std::cin >> n >> k;
            const double tol = num();
            const auto a = nums(n);
            const auto b = op == "nodefeas" ? nums(n) : std::vector<double>{};
            std::vector<int> ints(k);
            for (int& i : ints) std::cin >> i;
            bool r;
            if (op == "intfeas") {
                r = is_integer_feasible(a, ints, tol);
            } else {
                Node nd(0, -1, 0, a, b);
                r = is_node_feasible(nd, ints, tol);
            }
            std::printf("%d\n", r ? 1 : 0);
        } else if (op == "root") {
            std::string kind;
            std::cin >> kind;
            double rhs = 0.0;
            if (kind == "simplex" || kind == "eqsimplex") rhs = num();
            int n = 0, m = 0;
            std::cin >> n >> m;
            const double tol = num();
            Problem p;
            p.n_vars = n;
            p.lb = nums(n);
            p.ub = nums(n);
            const auto x = nums(m);
            if (kind == "box") check(p, BoxLMO{}, x, tol);
            else if (kind == "simplex") check(p, UnitSimplexLMO<64>(rhs, n, {}), x, tol);
            else if (kind == "eqsimplex") check(p, EqualitySimplexLMO<64>(rhs, n, {}), x, tol);
            else if (kind == "none") check(p, NoPointCheck{}, x, tol);
            else {
                const bool answer = kind == "accept";
                check(p, NoPointCheck{}, x, tol,
                      [answer](const std::vector<double>&, const std::vector<double>&, const std::vector<double>&,
                               double) { return answer; });
            }
        }
    }
    return 0;
}
