// Host oracles of the drop-in LMOs (include/gpuboscia/lmo.h, lmo_dicg.h) on
// cases read from stdin, one per line:
//   box n g[n] lb[n] ub[n] x[n]
//   simplex eq rhs n k ints[k] g[n] lb[n] ub[n] x[n]
//   birkhoff order cost[n] lb[n] ub[n] x[n]            (n = order^2)
// For box and simplex: the forward vertex of g, the in-face vertex of g at x,
// and the DICG maximum step along d = inface(g) - forward(-g). For Birkhoff:
// the forward vertex under lb / ub and the in-face vertex at x under the unit
// box. All as %.17g numbers.
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include <gpuboscia/lmo.h>

static std::vector<double> read(int n) {
    std::vector<double> v(n);
    for (double& e : v) std::cin >> e;
    return v;
}

static void emit(const std::vector<double>& v) {
    for (double e : v) std::printf("%.17g ", e);
}

template <class L>
static void run(const L& lmo, const std::vector<double>& g, const std::vector<double>& lb,
                const std::vector<double>& ub, const std::vector<double>& x) {
    const size_t n = g.size();
    std::vector<double> fwd(n), face(n), back(n), ng(n), d(n);
    lmo.compute_v_cpu(g, lb, ub, fwd);
    lmo.compute_inface_v_cpu(g, x, lb, ub, face);
    for (size_t j = 0; j < n; ++j) ng[j] = -g[j];
    lmo.compute_v_cpu(ng, lb, ub, back);
    for (size_t j = 0; j < n; ++j) d[j] = face[j] - back[j];
    emit(fwd);
    emit(face);
    std::printf("%.17g\n", lmo.dicg_maximum_step_cpu(d, x, lb, ub));
}

template <int Order>
static bool birkhoff(int order) {
    if (order != Order) return false;
    constexpr int n = Order * Order;
    auto c = read(n), lb = read(n), ub = read(n), x = read(n);
    BirkhoffLMO<Order> lmo;
    std::vector<double> fwd(n), face(n), zero(n, 0.0), one(n, 1.0);
    lmo.compute_v_cpu(c, lb, ub, fwd);
    lmo.compute_inface_v_cpu(c, x, zero, one, face);
    emit(fwd);
    emit(face);
    std::printf("\n");
    return true;
}

int main() {
    std::string kind;
    while (std::cin >> kind) {
        if (kind == "box") {
            int n;
            std::cin >> n;
            auto g = read(n), lb = read(n), ub = read(n), x = read(n);
            run(BoxLMO{}, g, lb, ub, x);
        } else if (kind == "birkhoff") {
            int order;
            std::cin >> order;
            if (!(birkhoff<3>(order) || birkhoff<4>(order) || birkhoff<5>(order) || birkhoff<6>(order)
                  || birkhoff<7>(order) || birkhoff<8>(order) || birkhoff<12>(order) || birkhoff<16>(order)
                  || birkhoff<36>(order))) {
                std::printf("unsupported order %d\n", order);
                return 1;
            }
        } else {
            int eq, n, k;
            double rhs;
            std::cin >> eq >> rhs >> n >> k;
            std::vector<int> ints(k);
            for (int& i : ints) std::cin >> i;
            auto g = read(n), lb = read(n), ub = read(n), x = read(n);
            if (eq) run(EqualitySimplexLMO<64>(rhs, n, ints), g, lb, ub, x);
            else run(UnitSimplexLMO<64>(rhs, n, ints), g, lb, ub, x);
        }
    }
    return 0;
}
