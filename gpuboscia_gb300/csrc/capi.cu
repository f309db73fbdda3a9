// capi.cu -- extern "C" entry points of libgpuboscia_gb300 (include/gpuboscia_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>

#include "relax.cuh"

namespace {
thread_local std::string g_err;

int fail(int rc, const std::string& msg) {
    g_err = msg;
    return rc;
}

int validate(const gbx_objective* o, const gbx_lmo* l, const gbx_algorithm* a) {
    if (!o || !l || !a) return fail(GBX_ERR_INVALID, "null descriptor");
    if (o->n <= 0) return fail(GBX_ERR_INVALID, "objective n must be positive");
    if (l->n != o->n) return fail(GBX_ERR_INVALID, "objective and LMO sizes differ");
    if (o->kind == GBX_OBJ_DENSE_QUADRATIC) {
        if (!o->Q) return fail(GBX_ERR_INVALID, "dense quadratic needs Q");
    } else if (o->kind == GBX_OBJ_GRAPH_MATCHING) {
        if (o->order <= 0 || o->order * o->order != o->n || !o->A || !o->B)
            return fail(GBX_ERR_INVALID, "graph matching needs order*order == n and A, B");
    } else {
        return fail(GBX_ERR_UNSUPPORTED, "unknown objective kind");
    }
    if (l->kind == GBX_LMO_BIRKHOFF && l->order * l->order != l->n)
        return fail(GBX_ERR_INVALID, "Birkhoff LMO needs order*order == n");
    if (l->kind < GBX_LMO_BOX || l->kind > GBX_LMO_LINKED_CARDINALITY)
        return fail(GBX_ERR_UNSUPPORTED, "unknown LMO kind");
    if (l->kind == GBX_LMO_LINKED_CARDINALITY) {
        if (l->n % 2 || l->order < 0 || l->order > l->n / 2 || !(l->right_side >= 0.0) || !l->upper)
            return fail(GBX_ERR_INVALID,
                        "linked cardinality LMO needs n = 2 * assets, 0 <= order <= n / 2, a cardinality and upper");
        if (o->kind != GBX_OBJ_DENSE_QUADRATIC)
            return fail(GBX_ERR_UNSUPPORTED, "the linked cardinality LMO needs a dense quadratic objective");
    }
    if (l->kind == GBX_LMO_CARDINALITY) {
        if (l->n % 2 || !(l->right_side >= 1.0))
            return fail(GBX_ERR_INVALID, "cardinality LMO needs n = 2 * assets and a cardinality >= 1");
        if (a->kind == GBX_ALG_DICG)
            return fail(GBX_ERR_UNSUPPORTED, "the cardinality LMO supports Frank-Wolfe only");
    }
    if (a->kind != GBX_ALG_FRANK_WOLFE && a->kind != GBX_ALG_DICG)
        return fail(GBX_ERR_INVALID, "unknown algorithm");
    if (a->line_search < GBX_LS_OPEN_LOOP || a->line_search > GBX_LS_QUADRATIC_EXACT)
        return fail(GBX_ERR_INVALID, "unknown line search");
    if (a->line_search == GBX_LS_SECANT && a->secant_iters < 0)
        return fail(GBX_ERR_INVALID, "secant_iters must be non-negative");
    if (a->precision != GBX_PRECISION_FP64 && a->precision != GBX_PRECISION_MIXED)
        return fail(GBX_ERR_INVALID, "unknown precision");
    return GBX_OK;
}
}  // namespace

namespace gbx {
void set_last_error(const std::string& msg) { g_err = msg; }
}  // namespace gbx

extern "C" {

int gbx_abi_version(void) { return GBX_ABI_VERSION; }

const char* gbx_last_error(void) { return g_err.c_str(); }

size_t gbx_relax_workspace_bytes(const gbx_objective* obj, const gbx_lmo* lmo,
                                 const gbx_algorithm* alg, int n_nodes) {
    if (validate(obj, lmo, alg) != GBX_OK) return 0;
    if (n_nodes < 0) {
        g_err = "n_nodes must be non-negative";
        return 0;
    }
    gbx::Layout L;
    std::string err;
    if (gbx::make_layout(*obj, *lmo, *alg, n_nodes, &L, &err) != GBX_OK) {
        g_err = err;
        return 0;
    }
    return std::max(gbx::workspace_bytes(L, n_nodes), gbx::workspace_bytes_any_variant(*obj, *lmo, *alg, n_nodes));
}

int gbx_relax_batch(const gbx_objective* obj, const gbx_lmo* lmo, const gbx_algorithm* alg,
                    const gbx_node_batch* b, void* workspace, size_t workspace_bytes,
                    void* stream) {
    int rc = validate(obj, lmo, alg);
    if (rc) return rc;
    if (!b || b->n_nodes < 0 || b->max_iters < 0)
        return fail(GBX_ERR_INVALID, "batch: n_nodes and max_iters must be non-negative");
    if (b->n_nodes > 0 && (!b->x || !b->lb || !b->ub || !b->eps || !b->iterations
                           || !b->status || !b->gap || !b->value || !b->best_vertex
                           || !b->best_vertex_val))
        return fail(GBX_ERR_INVALID, "batch: null node buffer");
    if (!(b->candidate_tol >= 0.0)) return fail(GBX_ERR_INVALID, "candidate_tol must be >= 0");
    gbx::Params p{};
    p.obj = *obj;
    p.lmo = *lmo;
    p.alg = *alg;
    p.b = *b;
    std::string err;
    rc = gbx::make_layout(*obj, *lmo, *alg, b->n_nodes, &p.L, &err);
    if (rc) return fail(rc, err);
    const size_t need = gbx::workspace_bytes(p.L, b->n_nodes);
    if ((need > 256 || p.L.persistent) && (!workspace || workspace_bytes < need))
        return fail(GBX_ERR_WORKSPACE, "workspace smaller than gbx_relax_workspace_bytes()");
    p.ws = static_cast<double*>(workspace);
    p.queue = p.L.persistent && b->n_nodes > 0
                  ? reinterpret_cast<int*>(static_cast<unsigned char*>(workspace) + gbx::queue_offset(p.L, b->n_nodes))
                  : nullptr;
    p.mixed = p.L.mixed_node_bytes
                  ? static_cast<unsigned char*>(workspace) + gbx::mixed_region_offset(p.L, b->n_nodes)
                  : nullptr;
    p.sparse = nullptr;
    if (p.L.sparse_bytes && b->n_nodes > 0) {
        p.sparse = static_cast<unsigned char*>(workspace) + gbx::sparse_region_offset(p.L, b->n_nodes);
        rc = gbx::launch_sparse_build(*obj, p.L, p.sparse, static_cast<cudaStream_t>(stream), &err);
        if (rc) return fail(rc, err);
    }
    rc = gbx::launch_relax(p, stream, &err);
    if (rc) return fail(rc, err);
    return GBX_OK;
}

int gbx_relax_autotune(const gbx_objective* obj, const gbx_lmo* lmo, const gbx_algorithm* alg,
                       const gbx_node_batch* b, void* workspace, size_t workspace_bytes, void* stream,
                       int repeats, int* chosen) {
    int rc = validate(obj, lmo, alg);
    if (rc) return rc;
    if (!b || b->n_nodes <= 0 || !b->x || !b->iterations || !b->status)
        return fail(GBX_ERR_INVALID, "autotune needs a non-empty batch");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const std::vector<gbx::Variant> cands = gbx::candidate_variants(*obj, *lmo, *alg);
    const int N = b->n_nodes, n = obj->n;
    const size_t xb = (size_t)N * n * sizeof(double), ib = (size_t)N * sizeof(int), sb = (size_t)N;
    unsigned char* save = nullptr;
    cudaError_t e = cudaMallocAsync(&save, xb + ib + sb, st);
    if (e != cudaSuccess) return fail(GBX_ERR_CUDA, cudaGetErrorString(e));
    auto copy_in = [&](bool restore) {
        const auto k = cudaMemcpyDeviceToDevice;
        if (!restore) {
            cudaMemcpyAsync(save, b->x, xb, k, st);
            cudaMemcpyAsync(save + xb, b->iterations, ib, k, st);
            cudaMemcpyAsync(save + xb + ib, b->status, sb, k, st);
        } else {
            cudaMemcpyAsync(b->x, save, xb, k, st);
            cudaMemcpyAsync(b->iterations, save + xb, ib, k, st);
            cudaMemcpyAsync(b->status, save + xb + ib, sb, k, st);
        }
    };
    copy_in(false);
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    float best_ms = 0.f;
    int best = -1;
    std::string err;
    for (int c = 0; c < (int)cands.size() && rc == GBX_OK; ++c) {
        gbx::Params p{};
        p.obj = *obj;
        p.lmo = *lmo;
        p.alg = *alg;
        p.b = *b;
        if (gbx::make_layout(*obj, *lmo, *alg, N, &p.L, &err, &cands[c]) != GBX_OK) continue;
        if (gbx::workspace_bytes(p.L, N) > workspace_bytes || !workspace) continue;
        p.ws = static_cast<double*>(workspace);
        p.mixed = p.L.mixed_node_bytes ? static_cast<unsigned char*>(workspace) + gbx::mixed_region_offset(p.L, N)
                                       : nullptr;
        p.queue = p.L.persistent ? reinterpret_cast<int*>(static_cast<unsigned char*>(workspace) +
                                                          gbx::queue_offset(p.L, N))
                                 : nullptr;
        p.sparse = nullptr;
        if (p.L.sparse_bytes) {
            p.sparse = static_cast<unsigned char*>(workspace) + gbx::sparse_region_offset(p.L, N);
            rc = gbx::launch_sparse_build(*obj, p.L, p.sparse, st, &err);
            if (rc) break;
        }
        float ms_min = 0.f;
        for (int r = 0; r < std::max(1, repeats); ++r) {
            copy_in(true);
            cudaEventRecord(t0, st);
            rc = gbx::launch_relax(p, st, &err);
            cudaEventRecord(t1, st);
            if (rc) break;
            cudaEventSynchronize(t1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, t0, t1);
            if (r == 0 || ms < ms_min) ms_min = ms;
        }
        if (rc == GBX_OK && (best < 0 || ms_min < best_ms)) { best = c; best_ms = ms_min; }
    }
    copy_in(true);
    cudaFreeAsync(save, st);
    e = cudaStreamSynchronize(st);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (rc) return fail(rc, err);
    if (e != cudaSuccess) return fail(GBX_ERR_CUDA, cudaGetErrorString(e));
    if (best < 0) return fail(GBX_ERR_WORKSPACE, "no launch shape fits the workspace");
    gbx::store_variant(*obj, *lmo, *alg, cands[best]);
    if (chosen) {
        gbx::Layout L;
        gbx::make_layout(*obj, *lmo, *alg, N, &L, &err, &cands[best]);
        chosen[0] = L.tc;
        chosen[1] = L.cluster ? 2 : L.persistent;
    }
    return GBX_OK;
}

int gbx_relax_set_launch_shape(const gbx_objective* obj, const gbx_lmo* lmo, const gbx_algorithm* alg,
                               int tensor_core, int persistent) {
    const int rc = validate(obj, lmo, alg);
    if (rc) return rc;
    if (tensor_core < -1 || tensor_core > 1 || persistent < 0 || persistent > 3)
        return fail(GBX_ERR_INVALID, "launch shape: tensor_core in -1..1, persistent in 0..3");
    gbx::Variant v;
    v.tc = tensor_core;
    v.persistent = persistent;
    gbx::Layout L;
    std::string err;
    const int r = gbx::make_layout(*obj, *lmo, *alg, 1, &L, &err, &v);
    if (r) return fail(r, err);
    gbx::store_variant(*obj, *lmo, *alg, v);
    return GBX_OK;
}

int gbx_relax_set_oracle_warps(const gbx_objective* obj, const gbx_lmo* lmo, const gbx_algorithm* alg, int warps) {
    const int rc = validate(obj, lmo, alg);
    if (rc) return rc;
    if (warps != -1 && warps != 1 && warps != 4) return fail(GBX_ERR_INVALID, "oracle warps: -1, 1 or 4");
    gbx::Variant v = gbx::tuned_variant(*obj, *lmo, *alg);
    v.oracle_warps = warps;
    gbx::Layout L;
    std::string err;
    const int r = gbx::make_layout(*obj, *lmo, *alg, 1, &L, &err, &v);
    if (r) return fail(r, err);
    gbx::store_variant(*obj, *lmo, *alg, v);
    return GBX_OK;
}

int gbx_relax_set_nodes_per_sm(const gbx_objective* obj, const gbx_lmo* lmo, const gbx_algorithm* alg, int per_sm) {
    const int rc = validate(obj, lmo, alg);
    if (rc) return rc;
    if (per_sm != -1 && per_sm != 1 && per_sm != 2) return fail(GBX_ERR_INVALID, "nodes per SM: -1, 1 or 2");
    gbx::Variant v = gbx::tuned_variant(*obj, *lmo, *alg);
    v.per_sm = per_sm;
    gbx::Layout L;
    std::string err;
    const int r = gbx::make_layout(*obj, *lmo, *alg, 1, &L, &err, &v);
    if (r) return fail(r, err);
    gbx::store_variant(*obj, *lmo, *alg, v);
    return GBX_OK;
}

int gbx_lmo_batch(const gbx_lmo* lmo, int cases, int mode, const double* direction,
                  const double* x, const double* lb, const double* ub, double* out,
                  double* out_step, void* stream) {
    if (!lmo || cases < 0 || lmo->n <= 0) return fail(GBX_ERR_INVALID, "lmo batch arguments");
    if (mode != 0 && mode != 1) return fail(GBX_ERR_INVALID, "mode must be 0 or 1");
    if (cases > 0 && (!direction || !lb || !ub || !out || (mode == 1 && !x)))
        return fail(GBX_ERR_INVALID, "null LMO buffer");
    if (lmo->kind == GBX_LMO_BIRKHOFF && lmo->order * lmo->order != lmo->n)
        return fail(GBX_ERR_INVALID, "Birkhoff LMO needs order*order == n");
    if (lmo->kind == GBX_LMO_LINKED_CARDINALITY && !lmo->upper)
        return fail(GBX_ERR_INVALID, "linked cardinality LMO needs upper");
    std::string err;
    const int rc = gbx::launch_lmo_batch(*lmo, cases, mode, direction, x, lb, ub, out,
                                         out_step, stream, &err);
    if (rc) return fail(rc, err);
    return GBX_OK;
}

int gbx_objective_gradient_batch(const gbx_objective* obj, int precision, int cases,
                                 const double* x, double* g, void* stream) {
    if (!obj || cases < 0 || obj->n <= 0) return fail(GBX_ERR_INVALID, "gradient batch arguments");
    if (cases > 0 && (!x || !g)) return fail(GBX_ERR_INVALID, "null gradient buffer");
    if (obj->kind == GBX_OBJ_DENSE_QUADRATIC) {
        if (!obj->Q) return fail(GBX_ERR_INVALID, "dense quadratic needs Q");
    } else if (obj->kind == GBX_OBJ_GRAPH_MATCHING) {
        if (obj->order <= 0 || obj->order * obj->order != obj->n || !obj->A || !obj->B)
            return fail(GBX_ERR_INVALID, "graph matching needs order*order == n and A, B");
    } else {
        return fail(GBX_ERR_UNSUPPORTED, "unknown objective kind");
    }
    if (precision != GBX_PRECISION_FP64 && precision != GBX_PRECISION_MIXED)
        return fail(GBX_ERR_INVALID, "unknown precision");
    if (precision == GBX_PRECISION_MIXED && (obj->kind != GBX_OBJ_GRAPH_MATCHING || obj->order > 128))
        return fail(GBX_ERR_UNSUPPORTED, "the mixed gradient covers graph matching up to order 128");
    std::string err;
    const int rc = gbx::launch_gradient_batch(*obj, precision, cases, x, g,
                                              static_cast<cudaStream_t>(stream), &err);
    if (rc) return fail(rc, err);
    return GBX_OK;
}

int gbx_scorer_param_count(int n_features, int hidden) {
    if (n_features <= 0 || hidden <= 0) return 0;
    return gbx::scorer_param_count(n_features, hidden);
}

int gbx_scorer_forward(const gbx_scorer* s, int rows, const float* features, float* scores, int bf16,
                       void* stream) {
    if (rows < 0 || (rows > 0 && (!features || !scores))) return fail(GBX_ERR_INVALID, "scorer forward arguments");
    std::string err;
    const int rc = gbx::scorer_forward(s, rows, features, scores, bf16, static_cast<cudaStream_t>(stream), &err);
    if (rc) return fail(rc, err);
    return GBX_OK;
}

size_t gbx_scorer_workspace_bytes(const gbx_scorer* s, int rows) { return gbx::scorer_workspace_bytes(s, rows); }

int gbx_scorer_gradient(const gbx_scorer* s, int rows, const float* features, int groups,
                        const int* group_ptr, const float* target, float* grad, float* loss,
                        void* workspace, size_t workspace_bytes, void* stream) {
    std::string err;
    const int rc = gbx::scorer_gradient(s, rows, features, groups, group_ptr, target, grad, loss, workspace,
                                        workspace_bytes, static_cast<cudaStream_t>(stream), &err);
    if (rc) return fail(rc, err);
    return GBX_OK;
}

int gbx_scorer_adam(gbx_scorer* s, const float* grad, float* m, float* v, int step, float lr, void* stream) {
    std::string err;
    const int rc = gbx::scorer_adam(s, grad, m, v, step, lr, static_cast<cudaStream_t>(stream), &err);
    if (rc) return fail(rc, err);
    return GBX_OK;
}

int gbx_objective_gradient_batch_f32(const gbx_objective* obj, int cases, const float* x, float* g,
                                     void* stream) {
    if (!obj || cases < 0 || obj->n <= 0) return fail(GBX_ERR_INVALID, "gradient batch arguments");
    if (cases > 0 && (!x || !g)) return fail(GBX_ERR_INVALID, "null gradient buffer");
    if (obj->kind != GBX_OBJ_GRAPH_MATCHING || obj->order <= 0 || obj->order > 128
            || obj->order * obj->order != obj->n || !obj->A || !obj->B)
        return fail(GBX_ERR_UNSUPPORTED, "the pipelined gradient covers graph matching up to order 128");
    std::string err;
    const int rc = gbx::launch_gradient_batch_f32(*obj, cases, x, g, static_cast<cudaStream_t>(stream), &err);
    if (rc) return fail(rc, err);
    return GBX_OK;
}

int gbx_node_feasible_batch(const gbx_lmo* lmo, int cases, const double* lb,
                            const double* ub, const uint8_t* integer_flags, uint8_t* out,
                            void* stream) {
    if (!lmo || cases < 0 || lmo->n <= 0) return fail(GBX_ERR_INVALID, "feasibility arguments");
    if (cases > 0 && (!lb || !ub || !out)) return fail(GBX_ERR_INVALID, "null buffer");
    if (lmo->kind == GBX_LMO_LINKED_CARDINALITY && !lmo->upper)
        return fail(GBX_ERR_INVALID, "linked cardinality LMO needs upper");
    std::string err;
    const int rc = gbx::launch_node_feasible(*lmo, cases, lb, ub, integer_flags, out, stream, &err);
    if (rc) return fail(rc, err);
    return GBX_OK;
}

}  // extern "C"
