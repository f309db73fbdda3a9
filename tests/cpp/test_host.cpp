// CPU unit tests of the C++ drop-in headers (include/gpuboscia), mirroring the
// reference's tests/test_cpu.cpp:41-586. Built and run by tests/test_host_cpp.py.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <iostream>
#include <limits>
#include <numeric>
#include <vector>

#include <gpuboscia/bnb.h>
#include <gpuboscia/branching.h>
#include <gpuboscia/concurrent_queue.h>
#include <gpuboscia/gap_utils.h>
#include <gpuboscia/line_search_options.h>
#include <gpuboscia/lmo.h>
#include <gpuboscia/tree.h>

static int g_pass = 0, g_fail = 0;
#define EXPECT(c, m) do { if (c) ++g_pass; else { ++g_fail; std::cerr << "FAIL: " << m << "\n"; } } while (0)
#define NEAR(a, b, t, m) EXPECT(std::abs((a) - (b)) < (t), m)

using namespace gpuboscia;
static const double inf = std::numeric_limits<double>::infinity();
static const double nan_ = std::numeric_limits<double>::quiet_NaN();

static void certified_bound() {
    NEAR(certified_fw_lower_bound(-7, 10, 3), 7.0, 1e-12, "valid certificate advances");
    NEAR(certified_fw_lower_bound(-7, 10, -1e-12), -7.0, 1e-12, "negative gap keeps bound");
    NEAR(certified_fw_lower_bound(-7, 10, nan_), -7.0, 1e-12, "NaN gap keeps bound");
    NEAR(certified_fw_lower_bound(-7, inf, 1), -7.0, 1e-12, "non-finite primal keeps bound");
}

static void gaps() {
    NEAR(gap_absolute(9, 10), 1.0, 1e-12, "abs");
    NEAR(gap_relative(9, 10), 1.0 / 9.0, 1e-12, "rel min denominator");
    NEAR(gap_relative(0.25, 0.75), 2.0, 1e-12, "rel no floor at one");
    NEAR(gap_relative(-10, -9), 1.0 / 9.0, 1e-12, "rel symmetric");
    EXPECT(std::isinf(gap_relative(0, 0)) && std::isinf(gap_relative(0, 1)) && std::isinf(gap_relative(-1, 0)),
           "zero bound -> infinite rel gap");
    EXPECT(gap_within_tolerance(0, 0, 0, 0.01), "closed zero gap via abs");
    EXPECT(!gap_within_tolerance(9, 10, 0, 0.105), "rel uses smaller magnitude");
    EXPECT(!gap_within_tolerance(0, 1, 0.01, 0.01) && !gap_within_tolerance(-1, 0, 0.01, 0.01), "zero bound open");
    for (double bad : {inf, -inf, nan_})
        EXPECT(!gap_within_tolerance(bad, 1, .01, .01) && !gap_within_tolerance(1, bad, .01, .01), "non-finite");
    EXPECT(gap_within_tolerance(9.99, 10, 0.02, 1e-12) && gap_within_tolerance(99, 100, 1e-12, 0.011), "within");
    EXPECT(!gap_within_tolerance(-1, 1, 0.1, 0.1), "opposite signs");
    NEAR(depth_dependent_tolerance(1e-3, 0.8, 1e-6, 0), 1e-3, 1e-15, "root tol");
    NEAR(depth_dependent_tolerance(1e-3, 0.8, 1e-6, 2), 6.4e-4, 1e-15, "decay");
    NEAR(depth_dependent_tolerance(1e-3, 0.8, 1e-6, 1000), 1e-6, 1e-15, "floor");
}

static void feasibility() {
    const std::vector<int> v = {0, 1, 2};
    EXPECT(is_integer_feasible({0, 1, 2}, v) && !is_integer_feasible({0.5, 1, 2}, v), "integer feasible");
    EXPECT(is_integer_feasible({1 + 5e-7, 2}, {0, 1}, 1e-6) && !is_integer_feasible({1 + 5e-5, 2}, {0, 1}, 1e-6),
           "integer tol");
    EXPECT(is_integer_feasible({1.5}, {99}), "out-of-range index skipped");
    EXPECT(is_node_feasible(Node(1, -1, 0, {0, 1}, {3, 2}), {0, 1}), "non-empty box");
    EXPECT(!is_node_feasible(Node(2, -1, 0, {2}, {1}), {0}), "lb > ub");
    EXPECT(!is_node_feasible(Node(3, -1, 0, {1.2}, {1.8}), {0}), "no integer in interval");
    EXPECT(is_node_feasible(Node(4, -1, 0, {1.2}, {1.8}), {}), "continuous interval");
}

static void branching() {
    EXPECT(most_infeasible({1.1, 2.5, 3.9}, {0, 1, 2}) == 1, "most infeasible");
    auto t2 = top_k_infeasible({1.1, 2.5, 3.0}, {0, 1, 2}, 2);
    EXPECT(t2.size() == 2 && t2[0] == 1 && t2[1] == 0, "top-k order");
    EXPECT(top_k_infeasible({1.1, 2.5, 3.0}, {0, 1, 2}, 5).size() == 2, "top-k capped");
    EXPECT(top_k_infeasible({1 + 5e-5}, {0}, 1, 1e-4).empty() && top_k_infeasible({1 + 5e-5}, {0}, 1, 1e-6).size() == 1,
           "top-k tolerance");
    int next = 10;
    Node parent(5, -1, 0, {0, 0, 0}, {5, 5, 5});
    auto ch = branch_pow2(parent, next, {1.5, 2.5, 3.9}, {0, 1, 2}, 3);
    EXPECT(ch.size() == 8 && next == 18, "2^3 children");
    for (auto& c : ch) EXPECT(c.parent_id == 5 && c.depth == 1, "child links");
    int n2 = 1;
    EXPECT(branch_pow2(parent, n2, {1, 2, 3}, {0, 1, 2}, 3).empty(), "integral -> no children");
    auto two = branch_pow2(parent, n2, {1, 2.5, 3}, {0, 1, 2}, 3);
    EXPECT(two.size() == 2 && two[0].ub[1] == 2.0 && two[1].lb[1] == 3.0, "one fractional -> 2 children");
}

static void queue_semantics() {
    ConcurrentQueue q;
    for (int i = 0; i < 4; ++i) {
        Node nd(i, i < 2 ? 10 : 20, 1, {0.0}, {1.0});
        nd.dual_bound = i;
        q.push(nd);
    }
    EXPECT(q.pop_full_batch(3, 1.5).empty(), "full batch refuses cut-off nodes");
    EXPECT(q.size() == 2, "live nodes kept");
    Node other(4, 20, 1, {0.0}, {1.0});
    other.dual_bound = 0.5;
    q.push(other);
    q.discard_children(10);
    auto b = q.pop_batch(3, 1.5);
    EXPECT(b.size() == 1 && b[0].id == 4, "deferred pruning drops only that parent's children");
    Node node(7, 3, 2, {0, 0}, {1, 1});
    node.dual_bound = -0.25;
    node.relaxation_x = {0.2, 0.8};
    node.relaxation_iterations = 17;
    q.push(node);
    auto r = q.pop_batch(1, 1.0);
    EXPECT(r.size() == 1 && r[0].relaxation_x == node.relaxation_x && r[0].relaxation_iterations == 17,
           "queue keeps warm start");
    EXPECT(q.best_bound(1.0) == 1.0, "empty queue bound is the cutoff");
    ConcurrentBoundSet s;
    s.insert(2.0);
    s.insert(1.0);
    s.insert(1.0);
    s.erase_one(1.0);
    EXPECT(s.best_bound(5.0) == 1.0, "multiset erase one");
}

static void root_point() {
    Problem p;
    p.n_vars = 2;
    p.lb = {0, 0};
    p.ub = {1, 1};
    BoxLMO box;
    validate_root_initial_point(p, box, {});
    validate_root_initial_point(p, box, {0.25, 0.75});
    bool threw = false;
    try { validate_root_initial_point(p, box, {1.5, 0}); } catch (const std::invalid_argument&) { threw = true; }
    EXPECT(threw, "out-of-bounds root rejected");
    EqualitySimplexLMO<2> eq(1.0, 2, {});
    threw = false;
    try { validate_root_initial_point(p, eq, {0.5, 0.25}); } catch (const std::invalid_argument&) { threw = true; }
    EXPECT(threw, "root off the simplex rejected");
    validate_root_initial_point(p, eq, {0.5, 0.5});
    bool called = false;
    validate_root_initial_point(p, box, {0.5, 0.5}, [&](const std::vector<double>&, const std::vector<double>&,
                                                        const std::vector<double>&, double) { called = true; return true; });
    EXPECT(called, "custom validator used");
    BirkhoffLMO<2> bk;
    EXPECT(bk.relaxation_feasible_cpu({0.5, 0.5, 0.5, 0.5}, {}, {}, 1e-9), "doubly stochastic accepted");
    EXPECT(!bk.relaxation_feasible_cpu({1, 1, 0, 0}, {}, {}, 1e-9), "column sums checked");
}

static void quad_step() {
    NEAR(quadratic_exact_step(3, 6, 1), 0.5, 1e-14, "interior");
    EXPECT(quadratic_exact_step(3, 2, 0.25) == 0.25, "upper bound");
    EXPECT(quadratic_exact_step(-3, 6, 1) == 0, "uphill");
    EXPECT(quadratic_exact_step(3, 0, 1) == 1, "linear descent");
    EXPECT(quadratic_exact_step(0, 0, 1) == 0, "flat");
    EXPECT(quadratic_exact_step(-1, -4, 1) == 1, "concave endpoints");
    EXPECT(quadratic_exact_step(3, 6, 0) == 0, "zero max");
    NEAR(quadratic_exact_step(3e-100, 6e-100, 1), 0.5, 1e-14, "tiny curvature kept");
}

int main(int argc, char** argv) {
    if (argc > 1) {  // table mode: evaluate the header rules on stdin rows for the fixture checks
        std::string op;
        auto num = [](double& v) { std::string t; if (!(std::cin >> t)) return false; v = std::strtod(t.c_str(), nullptr); return true; };
        while (std::cin >> op) {
            double a = 0, b = 0, c = 0, d = 0;
            if (op == "gap" && num(a) && num(b) && num(c) && num(d)) {
                std::printf("%.17g %.17g %d\n", gap_absolute(a, b), gap_relative(a, b),
                            gap_within_tolerance(a, b, c, d) ? 1 : 0);
            } else if (op == "cert" && num(a) && num(b) && num(c)) {
                std::printf("%.17g\n", certified_fw_lower_bound(a, b, c));
            } else if (op == "depth" && num(a)) {
                std::printf("%.17g\n", depth_dependent_tolerance(1e-3, 0.8, 1e-6, (int)a));
            } else if (op == "quad" && num(a) && num(b) && num(c)) {
                std::printf("%.17g\n", quadratic_exact_step(a, b, c));
            } else if (op == "branch") {   // branch n k tol n_int ints[n_int] lb[n] ub[n] x[n]
                int n = 0, k = 0, n_int = 0;
                double tol = 0;
                std::cin >> n >> k;
                num(tol);
                std::cin >> n_int;
                std::vector<int> ints(n_int);
                for (int& i : ints) std::cin >> i;
                std::vector<double> lb(n), ub(n), x(n);
                for (auto* v : {&lb, &ub, &x})
                    for (double& e : *v) num(e);
                Node parent(0, -1, 0, lb, ub);
                int next = 1;
                const auto ch = branch_pow2(parent, next, x, ints, k, tol);
                std::printf("%d", (int)ch.size());   // then each child's lb and ub
                for (const auto& c2 : ch) {
                    for (double e : c2.lb) std::printf(" %.17g", e);
                    for (double e : c2.ub) std::printf(" %.17g", e);
                }
                std::printf("\n");
            }
        }
        return 0;
    }
    certified_bound();
    gaps();
    feasibility();
    branching();
    queue_semantics();
    root_point();
    quad_step();
    std::printf("%d passed, %d failed\n", g_pass, g_fail);
    return g_fail ? 1 : 0;
}
