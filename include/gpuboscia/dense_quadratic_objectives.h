// dense_quadratic_objectives.h -- built-in objectives
// (reference: include/gpuboscia/dense_quadratic_objectives.cuh:18-124,
//  examples/main.cu:131-181 for the graph-matching form).
//
// Objectives hold device pointers owned by the caller, as in the reference;
// they are evaluated inside the GB300 relaxation kernel and describe
// themselves to the C ABI through descriptor().
#pragma once
#include <cstddef>

#include "../gpuboscia_gb300.h"

// f(x) = 0.5*s*x'Qx + s*l*c'x + k, with Q stored transposed: d_Qt[k*Vars + j] == Q[j, k].
template <int Vars, int Threads = 64>
struct GlobalCachedDenseQuadraticObjective {
    static constexpr bool supports_quadratic_exact = true;
    static constexpr int n_vars = Vars;
    static constexpr int block_threads = Threads;
    static constexpr int shared_bytes = Vars * (int)sizeof(double) + 16;

    const double* d_Qt;
    const double* d_linear;
    double grad_scale;
    double linear_scale;
    double constant;

    GlobalCachedDenseQuadraticObjective(const double* Q_transposed = nullptr, const double* linear = nullptr,
                                        double grad_scale_ = 1.0, double linear_scale_ = 1.0,
                                        double constant_ = 0.0)
        : d_Qt(Q_transposed), d_linear(linear), grad_scale(grad_scale_), linear_scale(linear_scale_),
          constant(constant_) {}

    const void* l2_window_base() const { return d_Qt; }
    size_t l2_window_bytes() const { return (size_t)Vars * Vars * sizeof(double); }

    gbx_objective descriptor() const {
        gbx_objective o{};
        o.kind = GBX_OBJ_DENSE_QUADRATIC;
        o.n = Vars;
        o.Q = d_Qt;
        o.c = d_linear;
        o.scale = grad_scale;
        o.linear_scale = linear_scale;
        o.constant = constant;
        return o;
    }
};

// ||Ax - b||^2 from A'A (transposed), A'b and b'b: grad_scale 2, linear_scale -1.
template <int Vars, int Threads = 256>
struct ILSGlobalCachedObjective : public GlobalCachedDenseQuadraticObjective<Vars, Threads> {
    using Base = GlobalCachedDenseQuadraticObjective<Vars, Threads>;
    ILSGlobalCachedObjective(const double* d_AtA_transposed = nullptr, const double* d_Atb = nullptr,
                             double btb = 0.0)
        : Base(d_AtA_transposed, d_Atb, 2.0, -1.0, btb) {}
};

// f(X) = scale*||A X - X B||_F^2 over Order x Order matrices (row-major).
// The reference example GraphIsoObjective (0.5*||BX - XA||^2) is scale 0.5
// with the two adjacency matrices swapped.
template <int Order>
struct GraphMatchingObjective {
    static constexpr bool supports_quadratic_exact = true;
    static constexpr int n_vars = Order * Order;
    const double* d_A = nullptr;
    const double* d_B = nullptr;
    double scale = 1.0;

    GraphMatchingObjective() = default;
    GraphMatchingObjective(const double* A, const double* B, double s = 1.0) : d_A(A), d_B(B), scale(s) {}

    gbx_objective descriptor() const {
        gbx_objective o{};
        o.kind = GBX_OBJ_GRAPH_MATCHING;
        o.n = n_vars;
        o.order = Order;
        o.A = d_A;
        o.B = d_B;
        o.scale = scale;
        o.linear_scale = 1.0;
        return o;
    }
};
