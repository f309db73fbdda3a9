// branch_features.cpp -- per-candidate features of the learned branching
// scorer (host code, shared by the solver and the training-data collection).
#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/gpuboscia_gb300.h"

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
    double rel_gap = std::isfinite(gap) && std::isfinite(value) ? gap / (std::fabs(value) + 1.0) : 1.0;
    rel_gap = std::min(1.0, std::max(0.0, rel_gap));
    for (int c = 0; c < n_cand; ++c) {
        float* f = out + (size_t)c * F;
        std::fill(f, f + F, 0.f);
        const int v = vars[c];
        const double xv = x[v];
        const double fr = xv - std::floor(xv);
        f[0] = (float)std::min(fr, 1.0 - fr);
        f[1] = (float)xv;
        f[2] = (float)fr;
        f[3] = (float)(std::min(depth, 64) / 64.0);
        f[4] = (float)rel_gap;
        f[5] = 1.f;
        if (perm) {
            const int m = order, i = v / m, j = v % m;
            f[6] = (float)rfrac[i] / m;
            f[7] = (float)cfrac[j] / m;
            f[8] = (float)rmax[i];
            f[9] = (float)cmax[j];
            f[10] = xv >= rmax[i] ? 1.f : 0.f;
            f[11] = xv >= cmax[j] ? 1.f : 0.f;
            f[12] = (float)(xv / std::max(rmax[i], 1e-12));
            f[13] = (float)(xv / std::max(cmax[j], 1e-12));
            f[14] = (float)rfree[i] / m;
            f[15] = (float)(std::fabs(xv - 0.5) < 0.25 ? 1.0 : 0.0);
        }
    }
}
