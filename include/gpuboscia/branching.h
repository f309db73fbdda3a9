// branching.h -- branching strategies (reference: include/gpuboscia/branching.h:13-118).
#pragma once
#include <algorithm>
#include <cmath>
#include <functional>
#include <vector>

#include "node.h"

using BranchStrategy = std::function<std::vector<Node>(
    const Node& parent, int& next_id, const std::vector<double>& x, const std::vector<int>& int_vars)>;

// The integer variable whose fractional part is closest to 1/2.
inline int most_infeasible(const std::vector<double>& x, const std::vector<int>& int_vars) {
    int best = -1;
    double best_dist = -1.0;
    for (int i : int_vars) {
        const double frac = x[i] - std::floor(x[i]);
        const double dist = std::min(frac, 1.0 - frac);
        if (dist > best_dist) { best_dist = dist; best = i; }
    }
    return best;
}

// Up to k fractional integer variables, most infeasible first.
inline std::vector<int> top_k_infeasible(const std::vector<double>& x, const std::vector<int>& int_vars,
                                         int k, double integer_tol = 1e-6) {
    struct Cand { int idx; double dist; };
    std::vector<Cand> cands;
    cands.reserve(int_vars.size());
    for (int i : int_vars) {
        const double frac = x[i] - std::floor(x[i]);
        const double dist = std::min(frac, 1.0 - frac);
        if (dist > integer_tol) cands.push_back({i, dist});
    }
    std::sort(cands.begin(), cands.end(), [](const Cand& a, const Cand& b) { return a.dist > b.dist; });
    const int m = std::min(k, (int)cands.size());
    std::vector<int> out(m);
    for (int i = 0; i < m; ++i) out[i] = cands[i].idx;
    return out;
}

// 2^k children over the k most infeasible variables: bit b of the child index
// selects lb = ceil(x) (set) or ub = floor(x) (clear) for variable b.
inline std::vector<Node> branch_on_vars(const Node& parent, int& next_id, const std::vector<double>& x,
                                        const std::vector<int>& vars) {
    if (vars.empty()) return {};
    const int k = (int)vars.size();
    std::vector<Node> children;
    children.reserve(size_t(1) << k);
    for (int mask = 0; mask < (1 << k); ++mask) {
        Node child = parent;
        child.id = next_id++;
        child.parent_id = parent.id;
        child.depth = parent.depth + 1;
        child.dual_bound = parent.dual_bound;
        child.status = NodeStatus::Active;
        child.relaxation_x.clear();
        child.relaxation_iterations = 0;
        for (int b = 0; b < k; ++b) {
            const int v = vars[b];
            if (mask & (1 << b)) child.lb[v] = std::ceil(x[v]);
            else child.ub[v] = std::floor(x[v]);
        }
        children.push_back(std::move(child));
    }
    return children;
}

inline std::vector<Node> branch_pow2(const Node& parent, int& next_id, const std::vector<double>& x,
                                     const std::vector<int>& int_vars, int k = 3, double integer_tol = 1e-6) {
    return branch_on_vars(parent, next_id, x, top_k_infeasible(x, int_vars, k, integer_tol));
}
