// solve.cpp -- gbx_solve / gbx_default_settings: the whole branch and bound
// (gpuboscia::solve, gpuboscia.cuh:56-170) behind the C ABI, driving the same
// scheduler the C++ headers use.
#include <cuda_runtime.h>

#include <cmath>
#include <exception>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gpuboscia/device_resident_solver.h"
#include "../../include/gpuboscia/tree.h"
#include "relax.cuh"

namespace {
// relaxation_feasible_cpu of the built-in LMOs (lmo.cuh:214-217, 484-495, 923-935)
bool relaxation_feasible(const gbx_lmo& l, const std::vector<double>& x, double tol) {
    if (l.kind == GBX_LMO_BOX) return true;
    if (l.kind == GBX_LMO_SIMPLEX || l.kind == GBX_LMO_EQUALITY_SIMPLEX) {
        double mass = 0.0;
        if (l.kind == GBX_LMO_EQUALITY_SIMPLEX) {
            for (double v : x) { if (v < -tol) return false; mass += v; }
            return std::isfinite(mass) && std::abs(mass - l.right_side) <= tol;
        }
        for (double v : x) { if (v < 0.0) return false; mass += v; }
        return mass <= l.right_side + tol;
    }
    const int m = l.order;
    if ((int)x.size() != m * m) return false;
    for (double v : x) if (v < -tol || v > 1 + tol) return false;
    for (int i = 0; i < m; ++i) {
        double row = 0, col = 0;
        for (int j = 0; j < m; ++j) { row += x[i * m + j]; col += x[j * m + i]; }
        if (std::abs(row - 1) > tol || std::abs(col - 1) > tol) return false;
    }
    return true;
}
}  // namespace

extern "C" {

void gbx_default_settings(gbx_settings* s) {
    if (!s) return;
    *s = gbx_settings{};
    s->gpu_batch_size = 1024;
    s->num_streams = 8;
    s->gpu_max_iters = 20000;
    s->gpu_eps = 1e-3;
    s->gpu_eps_decay = 0.8;
    s->gpu_eps_min = 1e-6;
    s->integer_tol = 1e-6;
    s->abs_gap_tol = 1e-6;
    s->rel_gap_tol = 1e-2;
    s->algorithm.kind = GBX_ALG_DICG;
    s->algorithm.line_search = GBX_LS_SECANT;
    s->algorithm.secant_iters = 4;
    s->algorithm.secant_tol = 1e-10;
    s->algorithm.secant_denom_eps = 1e-14;
    s->algorithm.precision = GBX_PRECISION_FP64;
    s->time_limit_seconds = std::numeric_limits<double>::infinity();
    s->natural_lower_bound = -std::numeric_limits<double>::infinity();
    s->root_initial_point = nullptr;
    s->branch_k = 3;
    s->use_cuda_graph = 1;
}

int gbx_solve(const gbx_problem* problem, const gbx_objective* obj, const gbx_lmo* lmo,
              const gbx_settings* s, gbx_result* res) {
    try {
        if (!problem || !obj || !lmo || !s || !res) throw std::invalid_argument("null argument");
        const int n = problem->n_vars;
        if (n <= 0 || !problem->lb || !problem->ub || (problem->n_int > 0 && !problem->int_vars))
            throw std::invalid_argument("invalid problem");
        if (s->algorithm.kind == GBX_ALG_FRANK_WOLFE
                && (s->algorithm.line_search == GBX_LS_SCALED_OPEN_LOOP
                    || s->algorithm.line_search == GBX_LS_SAFEGUARDED_SCALED_OPEN_LOOP))
            throw std::invalid_argument("scaled open-loop is available only for DICG");
        if (s->branch_k < 1 || s->branch_k > 16) throw std::invalid_argument("branch_k must be in [1, 16]");
        Problem prob;
        prob.n_vars = n;
        prob.lb.assign(problem->lb, problem->lb + n);
        prob.ub.assign(problem->ub, problem->ub + n);
        prob.int_vars.assign(problem->int_vars, problem->int_vars + problem->n_int);

        gpuboscia::LMOSpec spec;
        spec.kind = lmo->kind;
        spec.right_side = lmo->right_side;
        spec.order = lmo->order;
        if (lmo->is_int) {
            spec.is_int.resize(n);
            GBX_CUDA_CHECK(cudaMemcpy(spec.is_int.data(), lmo->is_int, n, cudaMemcpyDeviceToHost));
        }
        std::vector<double> root_x;
        if (s->root_initial_point) {
            root_x.assign(s->root_initial_point, s->root_initial_point + n);
            gpuboscia::validate_initial_point_bounds(prob, root_x, 1e-9);
            if (!relaxation_feasible(*lmo, root_x, 1e-9))
                throw std::invalid_argument("root initial point violates the LMO's continuous feasible set");
        }
        if (std::isnan(s->natural_lower_bound) || s->natural_lower_bound == std::numeric_limits<double>::infinity())
            throw std::invalid_argument("natural lower bound must be finite or negative infinity");

        DeviceResidentConfig cfg;
        cfg.gpu_batch_size = s->gpu_batch_size;
        cfg.num_streams = s->num_streams;
        cfg.gpu_max_iters = s->gpu_max_iters;
        cfg.gpu_eps = s->gpu_eps;
        cfg.gpu_eps_decay = s->gpu_eps_decay;
        cfg.gpu_eps_min = s->gpu_eps_min;
        cfg.integer_tol = s->integer_tol;
        cfg.abs_gap_tol = s->abs_gap_tol;
        cfg.rel_gap_tol = s->rel_gap_tol;
        cfg.precision = s->algorithm.precision;

        const double tol = s->integer_tol;
        const int k = s->branch_k;
        BranchStrategy branch = [tol, k](const Node& p, int& id, const std::vector<double>& x,
                                         const std::vector<int>& iv) { return branch_pow2(p, id, x, iv, k, tol); };
        gpuboscia::detail::BnBEngine engine(prob, *obj, spec, s->algorithm, branch, cfg, s->time_limit_seconds);
        engine.set_child_id_stride(std::max(8, 1 << k));
        Node root(0, -1, 0, prob.lb, prob.ub);
        root.dual_bound = s->natural_lower_bound;
        root.relaxation_x = root_x;
        engine.push(root);
        const auto t0 = std::chrono::steady_clock::now();
        engine.solve();
        res->elapsed_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        res->objective = engine.incumbent_value();
        res->dual_bound = engine.dual_bound();
        res->nodes_processed = engine.nodes_processed();
        res->reached_tolerance = engine.reached_tolerance();
        res->reached_time_limit = engine.reached_time_limit();
        const auto x = engine.incumbent_x();
        res->has_incumbent = !x.empty();
        if (res->x && !x.empty()) std::copy(x.begin(), x.end(), res->x);
        return GBX_OK;
    } catch (const std::invalid_argument& e) {
        gbx::set_last_error(e.what());
        return GBX_ERR_INVALID;
    } catch (const std::exception& e) {
        gbx::set_last_error(e.what());
        return GBX_ERR_CUDA;
    }
}

}  // extern "C"
