// features.h -- per-candidate features of the learned branching scorer, as
// plain arithmetic usable from host code (gbx_branch_features) and from the
// device frontier's branching kernel, so both give the same floats.
#pragma once

#include <cmath>

#include "../../include/gpuboscia_gb300.h"

#ifdef __CUDACC__
#define GBX_FEAT_HD __host__ __device__
#else
#define GBX_FEAT_HD
#endif

namespace gbx {

// the node's relative gap, clipped to [0, 1] (1 when either number is not finite)
GBX_FEAT_HD inline double feature_rel_gap(double gap, double value) {
    const double r = (std::isfinite(gap) && std::isfinite(value)) ? gap / (std::fabs(value) + 1.0) : 1.0;
    const double lo = (0.0 < r) ? r : 0.0;   // NaN and -0 become +0
    return (lo < 1.0) ? lo : 1.0;
}

// Row statistics of a permutation-matrix iterate (Birkhoff LMO): for the
// candidate's row i and column j, the fractional counts, the maxima and the
// free (unfixed) entries of row i.
struct PermStats {
    int rfrac, cfrac, rfree;
    double rmax, cmax;
};

// features of candidate xv = x[v] (v = i * m + j when perm)
GBX_FEAT_HD inline void candidate_features(double xv, int depth, double rel_gap, bool perm, int m,
                                           const PermStats& p, float* f) {
    for (int q = 0; q < GBX_SCORER_FEATURES; ++q) f[q] = 0.f;
    const double fr = xv - std::floor(xv);
    const double d = (1.0 - fr) < fr ? (1.0 - fr) : fr;
    f[0] = (float)d;
    f[1] = (float)xv;
    f[2] = (float)fr;
    f[3] = (float)((depth < 64 ? depth : 64) / 64.0);
    f[4] = (float)rel_gap;
    f[5] = 1.f;
    if (perm) {
        f[6] = (float)p.rfrac / m;
        f[7] = (float)p.cfrac / m;
        f[8] = (float)p.rmax;
        f[9] = (float)p.cmax;
        f[10] = xv >= p.rmax ? 1.f : 0.f;
        f[11] = xv >= p.cmax ? 1.f : 0.f;
        f[12] = (float)(xv / (p.rmax < 1e-12 ? 1e-12 : p.rmax));
        f[13] = (float)(xv / (p.cmax < 1e-12 ? 1e-12 : p.cmax));
        f[14] = (float)p.rfree / m;
        f[15] = (float)(std::fabs(xv - 0.5) < 0.25 ? 1.0 : 0.0);
    }
}

}  // namespace gbx
