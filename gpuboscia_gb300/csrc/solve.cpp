// solve.cpp -- gbx_solve / gbx_default_settings: the whole branch and bound
// (gpuboscia::solve, gpuboscia.cuh:56-170) behind the C ABI, driving the same
// scheduler the C++ headers use.
#include <cuda_runtime.h>

#include <cmath>
#include <exception>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
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
    if (l.kind == GBX_LMO_CARDINALITY) {
        const int N = (int)x.size() / 2;
        double sw = 0.0, sz = 0.0;
        for (int j = 0; j < N; ++j) {
            const double w = x[j], z = x[N + j];
            if (w < -tol || z < -tol || z > 1 + tol || w > z + tol) return false;
            sw += w;
            sz += z;
        }
        return std::abs(sw - 1.0) <= tol && sz <= std::floor(l.right_side + 1e-9) + tol;
    }
    if (l.kind == GBX_LMO_LINKED_CARDINALITY) {
        // candidate_feasible_device of the sparse-Sharpe LMO on the host
        const int half = (int)x.size() / 2, assets = l.order > 0 ? l.order : half;
        std::vector<double> U(assets);
        GBX_CUDA_CHECK(cudaMemcpy(U.data(), l.upper, assets * sizeof(double), cudaMemcpyDeviceToHost));
        double sy = 0.0;
        for (int i = 0; i < assets; ++i) {
            const double v = x[i], y = x[half + i];
            if (v < -tol || v > U[i] * y + tol || y < -tol || y > 1 + tol) return false;
            sy += y;
        }
        return sy <= std::floor(l.right_side + 1e-9) + tol;
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
// Learned branching (branch_pow2 over the k candidates the scorer ranks
// highest). Every completed batch is scored in one device call; a node without
// scores (or with a non-finite score) falls back to the k most fractional
// variables, and the FW dual bound alone still decides pruning.
class LearnedBrancher {
public:
    LearnedBrancher(const gbx_scorer* s, int k, double tol, int order, const Problem& prob)
        : s_(s), k_(k), tol_(tol), order_(order), prob_(prob) {
        GBX_CUDA_CHECK(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
    }
    ~LearnedBrancher() {
        if (d_feat_) cudaFree(d_feat_);
        if (d_score_) cudaFree(d_score_);
        if (st_) cudaStreamDestroy(st_);
    }

    void prepare(int N, const Node* nodes, const double* x, const double* gap, const double* value,
                 const uint8_t* status) {
        const int n = prob_.n_vars;
        const int F = GBX_SCORER_FEATURES;
        std::vector<int> who, vars, start;
        for (int i = 0; i < N; ++i) {
            if (status[i] >= GBX_NODE_INTEGRAL_UNCONVERGED || cache_.count(nodes[i].id)) continue;
            const double* xi = x + (size_t)i * n;
            const int b = (int)vars.size();
            for (int v : prob_.int_vars) {
                const double fr = xi[v] - std::floor(xi[v]);
                if (std::isfinite(xi[v]) && std::min(fr, 1.0 - fr) > tol_) vars.push_back(v);
            }
            if ((int)vars.size() == b) continue;
            who.push_back(i);
            start.push_back(b);
        }
        if (vars.empty()) return;
        start.push_back((int)vars.size());
        const size_t R = vars.size();
        h_feat_.resize(R * F);
        for (size_t w = 0; w < who.size(); ++w) {
            const int i = who[w];
            const Node& nd = nodes[i];
            gbx_branch_features(n, x + (size_t)i * n, nd.lb.data(), nd.ub.data(), order_, nd.depth, gap[i],
                                value[i], start[w + 1] - start[w], vars.data() + start[w],
                                h_feat_.data() + (size_t)start[w] * F);
        }
        if (R > cap_) {
            if (d_feat_) cudaFree(d_feat_);
            if (d_score_) cudaFree(d_score_);
            cap_ = R * 2;
            GBX_CUDA_CHECK(cudaMalloc(&d_feat_, cap_ * F * sizeof(float)));
            GBX_CUDA_CHECK(cudaMalloc(&d_score_, cap_ * sizeof(float)));
        }
        gpuboscia::detail::NvtxRange range("gbx.scorer");
        GBX_CUDA_CHECK(cudaMemcpyAsync(d_feat_, h_feat_.data(), R * F * sizeof(float), cudaMemcpyHostToDevice, st_));
        if (gbx_scorer_forward(s_, (int)R, d_feat_, d_score_, s_->params_bf16 ? 1 : 0, st_) != GBX_OK)
            throw std::runtime_error(std::string("scorer: ") + gbx_last_error());
        h_score_.resize(R);
        GBX_CUDA_CHECK(cudaMemcpyAsync(h_score_.data(), d_score_, R * sizeof(float), cudaMemcpyDeviceToHost, st_));
        GBX_CUDA_CHECK(cudaStreamSynchronize(st_));
        for (size_t w = 0; w < who.size(); ++w) {
            auto& c = cache_[nodes[who[w]].id];
            for (int r = start[w]; r < start[w + 1]; ++r) c.push_back({vars[r], h_score_[r]});
        }
    }

    std::vector<Node> branch(const Node& p, int& id, const std::vector<double>& x, const std::vector<int>& iv) {
        std::vector<int> pick;
        auto it = cache_.find(p.id);
        if (it != cache_.end()) {
            auto c = std::move(it->second);
            cache_.erase(it);
            bool finite = true;
            for (auto& e : c) finite = finite && std::isfinite(e.second);
            if (finite && !c.empty()) {
                std::stable_sort(c.begin(), c.end(), [](const std::pair<int, float>& a,
                                                        const std::pair<int, float>& b) { return a.second > b.second; });
                for (int t = 0; t < (int)c.size() && t < k_; ++t) pick.push_back(c[t].first);
            }
        }
        if (pick.empty()) pick = top_k_infeasible(x, iv, k_, tol_);
        return branch_on_vars(p, id, x, pick);
    }

private:
    const gbx_scorer* s_;
    int k_;
    double tol_;
    int order_;
    const Problem& prob_;
    cudaStream_t st_ = nullptr;
    float* d_feat_ = nullptr;
    float* d_score_ = nullptr;
    size_t cap_ = 0;
    std::vector<float> h_feat_, h_score_;
    std::unordered_map<int, std::vector<std::pair<int, float>>> cache_;
};
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
    s->scorer = nullptr;
    s->autotune = 1;
    s->device_frontier = 0;
    s->incumbent_cutoff = 0;
    s->frontier_capacity = 0;
    s->frontier_slots = 2;
    s->node_limit = 0;
    s->trace = nullptr;
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
        if (s->node_limit < 0) throw std::invalid_argument("node_limit must be non-negative");
        res->reached_node_limit = 0;
        res->batches = 0;
        Problem prob;
        prob.n_vars = n;
        prob.lb.assign(problem->lb, problem->lb + n);
        prob.ub.assign(problem->ub, problem->ub + n);
        prob.int_vars.assign(problem->int_vars, problem->int_vars + problem->n_int);

        gpuboscia::LMOSpec spec;
        spec.kind = lmo->kind;
        spec.right_side = lmo->right_side;
        spec.order = lmo->order;
        spec.upper = lmo->upper;
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

        if (s->device_frontier) {
            std::string err;
            const int rc = gbx::solve_device_frontier(*problem, *obj, *lmo, *s, root_x.empty() ? nullptr : root_x.data(),
                                                      res, &err);
            if (rc) gbx::set_last_error(err);
            return rc;
        }

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
        cfg.use_cuda_graph = s->use_cuda_graph != 0;
        cfg.autotune = s->autotune != 0;
        cfg.incumbent_cutoff = s->incumbent_cutoff != 0;
        cfg.node_limit = s->node_limit;

        const double tol = s->integer_tol;
        const int k = s->branch_k;
        BranchStrategy branch = [tol, k](const Node& p, int& id, const std::vector<double>& x,
                                         const std::vector<int>& iv) { return branch_pow2(p, id, x, iv, k, tol); };
        std::unique_ptr<LearnedBrancher> learned;
        if (s->scorer) {
            if (!s->scorer->params || s->scorer->n_features != GBX_SCORER_FEATURES)
                throw std::invalid_argument("scorer: invalid descriptor");
            learned.reset(new LearnedBrancher(s->scorer, k, tol, lmo->kind == GBX_LMO_BIRKHOFF ? lmo->order : 0,
                                              prob));
            LearnedBrancher* lb = learned.get();
            branch = [lb](const Node& p, int& id, const std::vector<double>& x, const std::vector<int>& iv) {
                return lb->branch(p, id, x, iv);
            };
        }
        gpuboscia::detail::BnBEngine engine(prob, *obj, spec, s->algorithm, branch, cfg, s->time_limit_seconds);
        engine.set_child_id_stride(std::max(8, 1 << k));
        if (learned) {
            LearnedBrancher* lb = learned.get();
            engine.set_branch_batch_hook([lb](int N, const Node* nd, const double* x, const double* gap,
                                              const double* val, const uint8_t* st) {
                lb->prepare(N, nd, x, gap, val, st);
            });
        }
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
        res->reached_node_limit = engine.reached_node_limit();
        res->batches = (int)engine.gpu_batches();
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
