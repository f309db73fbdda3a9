// algorithms.h -- FW / DICG policies and line searches (reference: include/gpuboscia/algorithms.cuh).
//
// The policies are compile-time tags, as in the reference; the iteration they
// select runs inside the GB300 relaxation kernel. descriptor() maps a policy
// onto the C ABI.
#pragma once
#include <type_traits>

#include "../gpuboscia_gb300.h"
#include "line_search_options.h"

struct OpenLoopLS {
    static constexpr bool uses_secant_line_search = false;
    static constexpr int kind = GBX_LS_OPEN_LOOP;
};
struct ScaledOpenLoopLS {
    static constexpr bool uses_secant_line_search = false;
    static constexpr int kind = GBX_LS_SCALED_OPEN_LOOP;
};
struct SafeguardedScaledOpenLoopLS {
    static constexpr bool uses_secant_line_search = false;
    static constexpr int kind = GBX_LS_SAFEGUARDED_SCALED_OPEN_LOOP;
};
struct SecantLS {
    static constexpr bool uses_secant_line_search = true;
    static constexpr int kind = GBX_LS_SECANT;
    int max_iters;
    double tolerance;
    double denom_eps;
    SecantLS(int max_iters_ = 8, double tolerance_ = 1e-10, double denom_eps_ = 1e-14)
        : max_iters(max_iters_), tolerance(tolerance_), denom_eps(denom_eps_) {}
};
struct QuadraticExactLS {
    static constexpr bool uses_secant_line_search = true;
    static constexpr int kind = GBX_LS_QUADRATIC_EXACT;
};

template <typename Objective, typename = void>
struct SupportsQuadraticExact : std::false_type {};
template <typename Objective>
struct SupportsQuadraticExact<Objective, std::void_t<decltype(Objective::supports_quadratic_exact)>>
    : std::integral_constant<bool, Objective::supports_quadratic_exact> {};

namespace gpuboscia::detail {
template <class LS>
gbx_algorithm make_algorithm(int kind, const LS& ls) {
    gbx_algorithm a{};
    a.kind = kind;
    a.line_search = LS::kind;
    a.secant_iters = 4;
    a.secant_tol = 1e-10;
    a.secant_denom_eps = 1e-14;
    if constexpr (std::is_same_v<LS, SecantLS>) {
        a.secant_iters = ls.max_iters;
        a.secant_tol = ls.tolerance;
        a.secant_denom_eps = ls.denom_eps;
    }
    a.precision = GBX_PRECISION_FP64;
    return a;
}
}  // namespace gpuboscia::detail

template <typename LS = OpenLoopLS>
struct FrankWolfe {
    static constexpr bool uses_dicg = false;
    static constexpr bool uses_secant_line_search = LS::uses_secant_line_search;
    LS ls{};
    gbx_algorithm descriptor() const { return gpuboscia::detail::make_algorithm(GBX_ALG_FRANK_WOLFE, ls); }
};

template <typename LS = OpenLoopLS>
struct DecompositionInvariantFrankWolfe {
    static constexpr bool uses_dicg = true;
    static constexpr bool uses_secant_line_search = LS::uses_secant_line_search;
    LS ls{};
    gbx_algorithm descriptor() const { return gpuboscia::detail::make_algorithm(GBX_ALG_DICG, ls); }
};

using FrankWolfeOpenLoop = FrankWolfe<OpenLoopLS>;
using FrankWolfeSecant = FrankWolfe<SecantLS>;
using FrankWolfePolicy = FrankWolfeOpenLoop;
using DICGOpenLoop = DecompositionInvariantFrankWolfe<OpenLoopLS>;
using DICGScaledOpenLoop = DecompositionInvariantFrankWolfe<ScaledOpenLoopLS>;
using DICGSafeguardedScaledOpenLoop = DecompositionInvariantFrankWolfe<SafeguardedScaledOpenLoopLS>;
using DICGSecant = DecompositionInvariantFrankWolfe<SecantLS>;
using DICGPolicy = DICGOpenLoop;
using FrankWolfeQuadraticExact = FrankWolfe<QuadraticExactLS>;
using DICGQuadraticExact = DecompositionInvariantFrankWolfe<QuadraticExactLS>;
