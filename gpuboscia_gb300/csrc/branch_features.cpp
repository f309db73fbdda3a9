// branch_features.cpp -- per-candidate features of the learned branching
// scorer (host code, shared by the solver and the training-data collection).
#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/gpuboscia_gb300.h"
#include "features.h"

extern "C" void gbx_branch_features(int n, const double* x, const double* lb, const double* ub, int order,
                                    int depth, double gap, double value, int n_cand, const int* vars,
                                    float* out) {
    const int F = GBX_SCORER_FEATURES;
    const bool perm = order > 0 && order * order == n;
    std::vector<double> rmax, cmax;
    std::vector<int> rfrac, cfrac, rfree;
    if (perm) {
        const int m = order;
        rmax.assign(m, 0.0);
        cmax.assign(m, 0.0);
        rfrac.assign(m, 0);
        cfrac.assign(m, 0);
        rfree.assign(m, 0);
        for (int e = 0; e < n; ++e) {
            const int i = e / m, j = e % m;
            const double v = x[e];
            rmax[i] = std::max(rmax[i], v);
            cmax[j] = std::max(cmax[j], v);
            const double fr = v - std::floor(v);
            if (std::min(fr, 1.0 - fr) > 1e-6) { ++rfrac[i]; ++cfrac[j]; }
            if (lb[e] < 0.5 && ub[e] >= 0.5) ++rfree[i];
        }
    }
    const double rel_gap = gbx::feature_rel_gap(gap, value);
    for (int c = 0; c < n_cand; ++c) {
        const int v = vars[c];
        gbx::PermStats p{};
        if (perm) {
            const int i = v / order, j = v % order;
            p.rfrac = rfrac[i];
            p.cfrac = cfrac[j];
            p.rfree = rfree[i];
            p.rmax = rmax[i];
            p.cmax = cmax[j];
        }
        gbx::candidate_features(x[v], depth, rel_gap, perm, order, p, out + (size_t)c * F);
    }
}
