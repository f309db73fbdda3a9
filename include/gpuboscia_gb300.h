/*
 * gpuboscia_gb300.h -- C ABI of the GB300 node-relaxation library.
 *
 * The reference library (GPUBoscia) is header-only C++/CUDA: its hot path is
 * the template kernel drs_fw_relax_batch_kernel<Objective, Algorithm, LMO>
 * (include/gpuboscia/device_resident_solver.cuh:631-660) launched by
 * DeviceResidentHybridSolver::run_slot (device_resident_solver.cuh:1775-1863).
 * This header replaces that launch with plain extern "C" entry points over
 * caller-owned device buffers, so any host language can bind the path.
 *
 * Conventions
 *   - Every entry point returns an int status (GBX_OK == 0, negative on error)
 *     and never throws; gbx_last_error() gives a thread-local message.
 *   - Pointers named d_* / documented "device" are CUDA device pointers owned
 *     by the caller; "host" pointers are ordinary host memory.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *   - Node vectors are node-major, row-major: x[node * n + j]. Birkhoff
 *     variables are e = r * order + c (lmo.cuh:914-917).
 */
#ifndef GPUBOSCIA_GB300_H
#define GPUBOSCIA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBX_ABI_VERSION 4

/* ---- status codes ------------------------------------------------------ */
enum {
    GBX_OK = 0,
    GBX_ERR_INVALID = -1,      /* bad sizes, null pointers, bad enums        */
    GBX_ERR_UNSUPPORTED = -2,  /* objective/LMO/algorithm combination        */
    GBX_ERR_CUDA = -3,         /* a CUDA runtime call failed                 */
    GBX_ERR_WORKSPACE = -4,    /* workspace too small                        */
    GBX_ERR_TIMEOUT = -5       /* a bounded device wait gave up              */
};

/* ---- per-node status byte (device_resident_solver.cuh:192-202) --------- */
enum {
    GBX_NODE_FRACTIONAL_UNCONVERGED = 0,
    GBX_NODE_FRACTIONAL_CONVERGED = 1,
    GBX_NODE_INFEASIBLE = 2,
    GBX_NODE_INTEGRAL_UNCONVERGED = 3,
    GBX_NODE_INTEGRAL_CONVERGED = 4,
    /* input-only flag: x holds a caller-supplied start (DRSInitialPointSupplied) */
    GBX_NODE_INITIAL_POINT_SUPPLIED = 0x80
};

/* ---- objectives --------------------------------------------------------- */
enum {
    /* f(x) = 0.5*scale*x'Qx + scale*linear_scale*c'x + constant; Q symmetric
     * (GlobalCachedDenseQuadraticObjective, dense_quadratic_objectives.cuh:18-112) */
    GBX_OBJ_DENSE_QUADRATIC = 1,
    /* f(X) = scale*||A X - X B||_F^2 over order x order X
     * (GraphIsoObjective, examples/main.cu:131-181, is scale=0.5 with A,B swapped) */
    GBX_OBJ_GRAPH_MATCHING = 2
};

typedef struct gbx_objective {
    int kind;             /* GBX_OBJ_*                                        */
    int n;                /* number of variables                              */
    /* dense quadratic */
    const double* Q;      /* device, n*n; Q[k*n + j] multiplies x_k in grad_j
                           * (the transposed storage of
                           * dense_quadratic_objectives.cuh:22-23; a
                           * symmetric matrix needs no care)                */
    const double* c;      /* device, n (may be NULL)                          */
    double scale;         /* grad_scale                                       */
    double linear_scale;
    double constant;
    /* graph matching */
    int order;            /* n == order*order                                 */
    const double* A;      /* device, order*order row-major                    */
    const double* B;      /* device, order*order row-major                    */
} gbx_objective;

/* ---- linear minimization oracles (lmo.cuh) ----------------------------- */
enum {
    GBX_LMO_BOX = 1,                /* BoxLMO, lmo.cuh:212-321                        */
    GBX_LMO_SIMPLEX = 2,            /* UnitSimplexLMO<n,false>, lmo.cuh:335-907       */
    GBX_LMO_EQUALITY_SIMPLEX = 3,   /* EqualitySimplexLMO<n>, lmo.cuh:911-912         */
    GBX_LMO_BIRKHOFF = 4,           /* BirkhoffLMO<order>, lmo.cuh:918-1419           */
    GBX_LMO_CARDINALITY = 5,        /* x = (w, z), n = 2N: sum w = 1, 0 <= w <= z,
                                       sum z <= right_side, 0 <= z <= 1; node bounds on z
                                       (lb > 1/2 forced, ub < 1/2 forbidden); Frank-Wolfe
                                       only (no counterpart in the reference; the pattern
                                       of examples/sparse_sharpe.cu:266-546 plus sum w = 1) */
    GBX_LMO_LINKED_CARDINALITY = 6  /* LinkedCardinalityLMO, examples/sparse_sharpe.cu:266-546:
                                       x = (v, y), y at offset n/2; the first `order`
                                       assets are active (0: n/2), the rest padding;
                                       0 <= v_i <= upper[i] * y_i, sum y <= right_side,
                                       0 <= y <= 1; node bounds on y; FW and DICG;
                                       needs a dense quadratic objective */
};

typedef struct gbx_lmo {
    int kind;                 /* GBX_LMO_*                                    */
    int n;                    /* number of variables                          */
    double right_side;        /* simplex mass                                 */
    const uint8_t* is_int;    /* device, n: the simplex LMO's integer flags   */
    int order;                /* Birkhoff order; linked cardinality: active assets */
    const double* upper;      /* device [order]: linked cardinality bounds U_i */
} gbx_lmo;

/* ---- algorithm policy (algorithms.cuh, line_search_options.h) ---------- */
enum { GBX_ALG_FRANK_WOLFE = 0, GBX_ALG_DICG = 1 };
enum {                        /* same order as LineSearchKind                */
    GBX_LS_OPEN_LOOP = 0,
    GBX_LS_SCALED_OPEN_LOOP = 1,
    GBX_LS_SAFEGUARDED_SCALED_OPEN_LOOP = 2,
    GBX_LS_SECANT = 3,
    GBX_LS_QUADRATIC_EXACT = 4
};
enum {
    GBX_PRECISION_FP64 = 0,   /* plain FP64 method (the drop-in)              */
    GBX_PRECISION_MIXED = 1   /* BF16 split tensor-core gradient, FP64 certificate */
};

typedef struct gbx_algorithm {
    int kind;                 /* GBX_ALG_*                                    */
    int line_search;          /* GBX_LS_*                                     */
    int secant_iters;         /* SecantLS::max_iters (default 4)              */
    double secant_tol;        /* SecantLS::tolerance (default 1e-10)          */
    double secant_denom_eps;  /* SecantLS::denom_eps (default 1e-14)          */
    int precision;            /* GBX_PRECISION_*                              */
} gbx_algorithm;

/* ---- one batch of B&B nodes (the arguments of drs_fw_relax_batch_kernel,
 *      device_resident_solver.cuh:634-654) -------------------------------- */
typedef struct gbx_node_batch {
    int n_nodes;
    int max_iters;            /* FW iteration budget of this dispatch         */
    double candidate_tol;     /* integer tolerance for vertex scoring         */
    double* x;                /* device [n_nodes*n] in: start/resume, out: iterate */
    const double* lb;         /* device [n_nodes*n]                           */
    const double* ub;         /* device [n_nodes*n]                           */
    const double* eps;        /* device [n_nodes] FW gap tolerance per node   */
    int* iterations;          /* device [n_nodes] in: done so far, out: total */
    uint8_t* status;          /* device [n_nodes] in: 0 or 0x80, out: GBX_NODE_* */
    double* gap;              /* device [n_nodes] out: FW gap at returned x   */
    double* value;            /* device [n_nodes] out: f(x)                   */
    double* best_vertex;      /* device [n_nodes*n] out: best integral point  */
    double* best_vertex_val;  /* device [n_nodes] out: its value (1e300 none) */
    const uint8_t* integer_flags; /* device [n] problem integer flags         */
    /* device pointer to the incumbent value, or NULL (the reference's
     * behaviour). When set, a node stops iterating once its FW bound
     * f(x) - gap clears the incumbent (after at least one step of this
     * dispatch), since branch and bound prunes it at any bound above; the
     * returned gap, value and status are the usual exact certificate at the
     * returned iterate. No counterpart in the reference. */
    const double* cutoff;
} gbx_node_batch;

/* Library identity. */
int gbx_abi_version(void);
const char* gbx_last_error(void);

/* Bytes of device scratch gbx_relax_batch needs for this batch (node vectors
 * that do not fit in shared memory, Hungarian state, split-precision tiles).
 * Replaces the slot workspace sizing of DRSStreamSlot::alloc
 * (device_resident_solver.cuh:1094-1128). */
size_t gbx_relax_workspace_bytes(const gbx_objective* obj, const gbx_lmo* lmo,
                                 const gbx_algorithm* alg, int n_nodes);

/* Relax every node of the batch with FW/DICG on the GPU (one launch on
 * `stream`; asynchronous). Replaces drs_fw_relax_batch_kernel<<<N,...>>>
 * (device_resident_solver.cuh:1834-1851). `workspace` is caller-owned device
 * memory of at least gbx_relax_workspace_bytes() bytes. */
int gbx_relax_batch(const gbx_objective* obj, const gbx_lmo* lmo,
                    const gbx_algorithm* alg, const gbx_node_batch* batch,
                    void* workspace, size_t workspace_bytes, void* stream);

/* The same relaxation for callers that cannot allocate device memory (a host
 * language without a CUDA allocator, memory owned by another runtime's pool, a
 * loop where allocation is not allowed). No counterpart in the reference: the
 * scratch lives in a library-owned __device__ array of GBX_STATIC_SCRATCH_BYTES
 * (32 MiB, held on every GPU that loads the library until exit); batches that
 * need more are rejected with GBX_ERR_WORKSPACE. The first call on a device
 * looks the array up and should come before any stream capture. Calls share
 * the array, so calls that overlap on the GPU race: issue them on one stream.
 * Allocates nothing. */
#define GBX_STATIC_SCRATCH_BYTES (32u << 20)
int gbx_relax_batch_static(const gbx_objective* obj, const gbx_lmo* lmo,
                           const gbx_algorithm* alg, const gbx_node_batch* batch,
                           void* stream);

/* Autotuner (no counterpart in the reference): times each candidate launch
 * shape of this problem on the caller's batch -- the tensor-core or FP32 SIMT
 * gradient where both apply (mixed precision, Birkhoff orders 17..90), one CTA
 * per node or a persistent grid pulling nodes from a queue, and for mixed
 * precision at Birkhoff orders 129..404 a cluster of four CTAs per node that
 * splits the assignment oracles' columns (the replacement of the reference's
 * MultiBlock backend, include/gpuboscia/multiblock.cuh:36-103) -- keeping the
 * fastest of `repeats` runs each, and makes the winner the shape that later
 * gbx_relax_batch calls of the same problem shape use (process-wide). The
 * batch's x, iterations and status are restored, so the caller still owns an
 * unrelaxed batch. workspace: gbx_relax_workspace_bytes (it covers every
 * shape). chosen (may be NULL) receives {tensor-core gradient, persistent}
 * with persistent 2 for the cluster shape. */
int gbx_relax_autotune(const gbx_objective* obj, const gbx_lmo* lmo, const gbx_algorithm* alg,
                       const gbx_node_batch* batch, void* workspace, size_t workspace_bytes,
                       void* stream, int repeats, int* chosen);

/* Pins the launch shape of this problem shape by hand (what the autotuner
 * would store): tensor_core -1/0/1 (default rule / FP32 SIMT / tensor-core
 * gradient; mixed precision only), persistent 0/1/2/3 (one CTA per node /
 * persistent grid / a cluster of four CTAs per node: mixed precision, Birkhoff
 * orders 129..404 / a pair of CTAs per node splitting the objective's
 * products: FP64 dense quadratic objective with the node in shared memory, for
 * batches smaller than the GPU; GBX_ERR_UNSUPPORTED elsewhere). */
int gbx_relax_set_launch_shape(const gbx_objective* obj, const gbx_lmo* lmo, const gbx_algorithm* alg,
                               int tensor_core, int persistent);

/* Pins how many warps run each integer assignment oracle of a large-order
 * mixed-precision Birkhoff relaxation (orders 129..512, one CTA per node or the
 * persistent grid): 1 (one warp per oracle, the forward and in-face oracles on
 * two warps) or 4 (a group of four warps per oracle, one per SM sub-partition,
 * each lane scanning a quarter of the columns of a Dijkstra step); -1 restores
 * the default (4). The assignments are identical either way. Keeps the pinned
 * or tuned tensor-core / persistent choice; gbx_relax_set_launch_shape resets
 * this to the default. GBX_ERR_UNSUPPORTED for 4 outside those orders. */
int gbx_relax_set_oracle_warps(const gbx_objective* obj, const gbx_lmo* lmo, const gbx_algorithm* alg,
                               int warps);

/* Pins how many nodes (CTAs of 256 threads) each SM holds for the FP64
 * relaxation kernels: 2 (the default wherever two fit in shared memory: the
 * kernel is compiled for a 128-register cap, and one node's barrier waits
 * overlap the other's work) or 1 (no register cap; faster only when a batch
 * leaves SMs idle anyway); -1 restores the default. Results are identical.
 * Keeps the other pinned or tuned choices; gbx_relax_set_launch_shape resets
 * it. GBX_ERR_UNSUPPORTED for 2 in mixed precision (its kernels fix their own). */
int gbx_relax_set_nodes_per_sm(const gbx_objective* obj, const gbx_lmo* lmo, const gbx_algorithm* alg,
                               int per_sm);

/* Batched LMO calls, one case per row (the probes of tests/test_pipeline.cu:
 * 96-163). mode 0: forward v = argmin <direction, v> over the node's set
 * (LMO::compute_v); mode 1: in-face away oracle (LMO::compute_inface_v) on
 * the minimal face of x. All arrays are device [cases*n]; x may be NULL for
 * mode 0. out_step (device [cases], may be NULL) receives, for mode 1, the
 * DICG maximum step of x - gamma*(out - fwd) where fwd is the forward vertex
 * of -direction (dicg_maximum_step_local + dicg_sum_maximum_step). The box
 * LMO without out_step runs as one element stream over all cases (16-byte
 * accesses when every buffer is 16-byte aligned); the other sets and the
 * maximum step take one CTA per case. */
int gbx_lmo_batch(const gbx_lmo* lmo, int cases, int mode,
                  const double* direction, const double* x,
                  const double* lb, const double* ub, double* out,
                  double* out_step, void* stream);

/* Batched objective gradients g = grad f(x), one point per row of x and g
 * (device [cases*n]); replaces Objective::grad
 * (dense_quadratic_objectives.cuh:43-60; the graph-matching gradient of
 * examples/main.cu:131-181). precision GBX_PRECISION_FP64: the relaxation's own
 * FP64 gradient, bit-identical to it; GBX_PRECISION_MIXED (graph matching
 * only): the gradient of the mixed-precision relaxation, BF16 tensor-core
 * products with FP32 accumulation for orders 65..128, FP32 below, widened to
 * double. */
int gbx_objective_gradient_batch(const gbx_objective* obj, int precision, int cases,
                                 const double* x, double* g, void* stream);

/* The mixed-precision graph-matching gradient of FP32 points (device
 * [cases*n] in and out; orders up to 128), software-pipelined over a
 * persistent grid so that tensor-core MMAs of one point overlap the loads and
 * epilogues of the next (the batch form of gbx_objective_gradient_batch for
 * callers that hold FP32 iterates). Synchronises the stream; GBX_ERR_TIMEOUT
 * if a tensor-core wait ran out. */
int gbx_objective_gradient_batch_f32(const gbx_objective* obj, int cases, const float* x, float* g,
                                     void* stream);

/* Node feasibility before any objective work (drs_node_feasible,
 * device_resident_solver.cuh:206-217): out[case] = 1 feasible, 0 infeasible. */
int gbx_node_feasible_batch(const gbx_lmo* lmo, int cases, const double* lb,
                            const double* ub, const uint8_t* integer_flags,
                            uint8_t* out, void* stream);

/* ---- whole branch-and-bound solve (gpuboscia::solve, gpuboscia.cuh:108-170)
 * for callers without the C++ headers. Objective/LMO data are device pointers
 * owned by the caller (as in the reference); problem data are host arrays. */
typedef struct gbx_problem {
    int n_vars;
    const double* lb;         /* host [n_vars] */
    const double* ub;         /* host [n_vars] */
    const int* int_vars;      /* host [n_int]  */
    int n_int;
} gbx_problem;

/* ---------------------------------------------------------------------------
 * Learned branching scorer (no counterpart in the reference; it only changes
 * which fractional variables branch_pow2 splits on -- most-fractional stays the
 * fallback and the FW dual bound alone decides pruning and optimality).
 * An MLP n_features -> hidden -> hidden -> 1 with ReLU, parameters in one FP32
 * device array in the order W1[hidden][n_features], b1[hidden],
 * W2[hidden][hidden], b2[hidden], w3[hidden], b3; params_bf16 (optional) is the
 * BF16 copy used for inference.
 * ------------------------------------------------------------------------- */
#define GBX_SCORER_FEATURES 16
typedef struct gbx_scorer {
    int n_features;             /* GBX_SCORER_FEATURES */
    int hidden;                 /* 8..128, a multiple of 8 */
    float* params;              /* device [gbx_scorer_param_count] */
    unsigned short* params_bf16;/* device [gbx_scorer_param_count] or NULL */
} gbx_scorer;

int gbx_scorer_param_count(int n_features, int hidden);

/* Features of the branching candidates vars[0..n_cand) of one node (host
 * arrays [n]): distance to integrality, value and fractional part, the node's
 * depth and relative gap, and for Birkhoff orders > 0 the candidate's row and
 * column structure. Writes n_cand rows of GBX_SCORER_FEATURES floats to out. */
void gbx_branch_features(int n, const double* x, const double* lb, const double* ub, int order,
                         int depth, double gap, double value, int n_cand, const int* vars, float* out);

/* scores[r] = MLP(features[r]) for rows of device features [rows][n_features];
 * bf16 != 0 uses params_bf16 (FP32 accumulation). */
int gbx_scorer_forward(const gbx_scorer* s, int rows, const float* features, float* scores, int bf16,
                       void* stream);

/* Listwise loss over groups (one group = the candidates of one node, rows
 * group_ptr[g] .. group_ptr[g+1]-1): L = sum_g -sum_r target[r] log softmax_g(z)[r]
 * with target summing to 1 per group. Writes dL/dparams (device
 * [param_count], deterministic order) and, if loss != NULL, L (device, 1 float).
 * workspace: device, gbx_scorer_workspace_bytes(rows) bytes. */
size_t gbx_scorer_workspace_bytes(const gbx_scorer* s, int rows);
int gbx_scorer_gradient(const gbx_scorer* s, int rows, const float* features, int groups,
                        const int* group_ptr, const float* target, float* grad, float* loss,
                        void* workspace, size_t workspace_bytes, void* stream);

/* Adam step on params (m, v: device moment arrays, step >= 1), then refresh
 * params_bf16 when it is set. */
int gbx_scorer_adam(gbx_scorer* s, const float* grad, float* m, float* v, int step, float lr,
                    void* stream);

/* Per-round timing of a device-frontier search (no counterpart in the
 * reference): round r pops a batch, relaxes it and branches the batch popped
 * the round before. ms[r] is the round's device time (CUDA events on the
 * search's stream; the host's reads between graph replays are not counted),
 * nodes[r] the nodes whose processing the round finished. The host frontier
 * records nothing (count 0). */
typedef struct gbx_round_trace {
    int capacity;             /* entries ms and nodes hold                    */
    int count;                /* out: rounds recorded (at most capacity)      */
    float* ms;                /* host [capacity]                              */
    int* nodes;               /* host [capacity]                              */
} gbx_round_trace;

typedef struct gbx_settings {
    /* DeviceResidentConfig (device_resident_solver.cuh:1004-1025) */
    int gpu_batch_size;       /* 1024 */
    int num_streams;          /* 8    */
    int gpu_max_iters;        /* 20000 */
    double gpu_eps;           /* 1e-3 */
    double gpu_eps_decay;     /* 0.8  */
    double gpu_eps_min;       /* 1e-6 */
    double integer_tol;       /* 1e-6 */
    double abs_gap_tol;       /* 1e-6 */
    double rel_gap_tol;       /* 1e-2 */
    /* Settings (gpuboscia.cuh:21-32) */
    gbx_algorithm algorithm;
    double time_limit_seconds;   /* +inf */
    double natural_lower_bound;  /* -inf */
    const double* root_initial_point; /* host [n_vars] or NULL */
    int branch_k;             /* branch_pow2 k (3) */
    int use_cuda_graph;       /* capture the relax launch (1) */
    const gbx_scorer* scorer; /* learned branching (NULL: most fractional) */
    int autotune;             /* time the launch shapes on the first full batch (1) */
    /* frontier in device memory (no counterpart in the reference): open nodes
     * stay in HBM and each round of the search (pop the best batch, relax,
     * branch_pow2, merge the children) runs as kernels replayed from a CUDA
     * graph; batch <= 1024, branch_k <= 8; the learned scorer runs inside the
     * branching kernel; num_streams and autotune unused (a stored launch
     * shape still applies) */
    int device_frontier;      /* 0 */
    int incumbent_cutoff;     /* stop node relaxations at the incumbent (gbx_node_batch.cutoff); 0 */
    int frontier_capacity;    /* open nodes the pool holds (0: a quarter of free memory, <= 2^18) */
    int frontier_slots;       /* device frontier: batches in flight, 1 or 2 (2: one relaxes while
                                 the other is branched and merged); 2 */
    /* stop once this many nodes are processed (0: no limit; no counterpart in
     * the reference). The search stops at the end of the batch that reaches
     * it; the result's dual bound is the live bound then, a valid bound. */
    int node_limit;           /* 0 */
    gbx_round_trace* trace;   /* device frontier: per-round timing, or NULL */
} gbx_settings;

typedef struct gbx_result {
    double objective;         /* +inf when no incumbent                       */
    double dual_bound;
    int nodes_processed;
    double elapsed_seconds;
    int reached_tolerance;
    int reached_time_limit;
    int has_incumbent;
    double* x;                /* host [n_vars], caller-owned, filled when has_incumbent */
    int reached_node_limit;   /* gbx_settings.node_limit stopped the search */
    int batches;              /* relaxation launches (batches of nodes) the search made */
} gbx_result;

/* ---- graph-matching instance files (examples/main.cu:41-129 reads the
 * reference's test_instances MAT files this way). Host arrays, row-major.
 * gbx_read_mat: the real matrix `name` ("A" when NULL) of a MATLAB v5 file,
 * plain or zlib-compressed, any numeric storage type; with out == NULL only
 * rows / cols are returned. gbx_read_dimacs: the 0/1 symmetric adjacency of a
 * DIMACS edge list ("p edge n m", "e u v", 1-based). GBX_ERR_INVALID for a
 * missing file or variable or a short buffer, GBX_ERR_UNSUPPORTED for a
 * malformed or unsupported file. */
int gbx_read_mat(const char* path, const char* name, int* rows, int* cols, double* out, size_t capacity);
int gbx_read_dimacs(const char* path, int* n_vertices, double* out, size_t capacity);

/* Fill *s with the reference defaults (create_default_settings). */
void gbx_default_settings(gbx_settings* s);

int gbx_solve(const gbx_problem* problem, const gbx_objective* obj,
              const gbx_lmo* lmo, const gbx_settings* settings,
              gbx_result* result);

#ifdef __cplusplus
}
#endif

#endif /* GPUBOSCIA_GB300_H */
