// relax.cuh -- shared declarations of the node-relaxation kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/gpuboscia_gb300.h"

namespace gbx {

constexpr int kThreads = 256;          // threads per node CTA (8 warps)
constexpr int kWarps = kThreads / 32;
constexpr double kNone = 1e300;        // "no candidate" sentinel of the reference

// Node vectors of one relaxation (all n doubles).
enum Buf { B_X, B_G, B_V, B_AW, B_TX, B_TG, B_R, B_LB, B_UB, B_CAND, B_COUNT };

// Where every buffer of a node lives; computed once per launch on the host.
struct Layout {
    int off[B_COUNT];       // offset in doubles inside the buffer's region (-1: absent)
    int in_smem[B_COUNT];   // 1: the buffer lives in dynamic shared memory, 0: global workspace
    int nvec;
    int vec_smem;           // every present node vector is in shared memory
    size_t node_stride;     // doubles per node in the global workspace
    int obj_smem;           // objective matrices staged in shared memory
    size_t obj_doubles;
    int sort_size;          // simplex bitonic network size (0: none)
    int hung_order;         // Birkhoff order (0: none)
    int hung_warps;         // Hungarian workspaces (1 or 2)
    size_t hung_bytes;      // bytes per Hungarian workspace
    // byte offsets inside dynamic shared memory
    size_t sm_vec, sm_obj, sm_keys, sm_prefix, sm_idx, sm_fixed, sm_hung, sm_total;
    // mixed precision (GBX_PRECISION_MIXED, Birkhoff graph matching): FP32
    // x, gradient, residual, A, B, B' [6 n floats] and A, B as int8 [2 n]
    // (shared memory, or per node in the workspace when mx_global), forward /
    // in-face integer oracle costs [2 n ints], edge / face code bytes [2 n],
    // and two integer Hungarian workspaces with warm state
    int mixed;
    int mx_global;
    int tc;                   // gradient on the tensor cores (orders 17..128); the
                              // operand images share the cost matrices' memory
    int persistent;           // persistent grid over an atomic node queue
    size_t sm_mx, sm_cost, sm_code, sm_ihw, ihw_bytes;
    size_t mixed_node_bytes;  // bytes per node of the workspace's mixed region
    // orders whose oracle costs do not fit in shared memory (above ~128):
    // the costs and edge codes live in the node's mixed region at these
    // offsets, the gradient runs over the nonzero lists in FP32
    int cost_global;
    size_t mx_cost_off, mx_code_off;
    // those orders keep each oracle warp's per-column Hungarian state in
    // shared memory (cs_bytes per warp at sm_cs), so two nodes fit on an SM
    size_t sm_cs, cs_bytes;
    // ... and run each integer oracle on a group of four warps (forward on
    // warps 0-3, in-face on 4-7: a quarter of the columns per lane and step)
    // instead of one warp
    int oracle_group;
    // FP64 kernels: compiled for two CTAs per SM (a 128-register cap) when
    // two fit in shared memory, else one (the autotuner times both)
    int per_sm2;
    // FP64 dense quadratic objective with every node vector in shared memory:
    // a node on a pair of CTAs (a two-CTA cluster) that split the objective's
    // products, with a 256-double exchange buffer at sm_xch
    int pair;
    size_t sm_xch;
    // a cluster of `cluster` CTAs per node (0: one CTA): cl_cols columns of
    // packed oracle costs per CTA at sm_slice (the FP64 workspace shares it),
    // two per-oracle workspaces of chw_bytes at sm_chw, the leader's
    // row->column maps of both oracles at sm_lpi, the control block at sm_cl
    int cluster, cl_cols;
    size_t sm_slice, sm_chw, chw_bytes, sm_lpi, sm_cl;
    // the certificate's FP64 Hungarian reads the gradient staged in the cost
    // region (1), or straight from the node's gradient vector (0) when staging
    // would cost a resident node per SM
    int cert_stage;
    // the in-face oracle derives its costs from the forward ones (no second
    // cost array) -- only where that fits two nodes per SM
    int derive_inface;
    // graph matching: nonzero lists of A and B (rows and columns), built once
    // per launch at the end of the workspace; up to sparse_cap entries each
    int sparse_cap;
    size_t sparse_bytes;
};

struct Params {
    gbx_objective obj;
    gbx_lmo lmo;
    gbx_algorithm alg;
    gbx_node_batch b;
    Layout L;
    double* ws;             // global workspace (node vectors when not in smem)
    unsigned char* mixed;   // mixed-precision scratch
    unsigned char* sparse;  // nonzero lists of A and B (graph matching), or null
    int* queue;             // persistent grid: next-node counter (zeroed per launch), or null
    const int* live_count;  // device-side node count (<= b.n_nodes) read at launch, or null
};

#ifdef __CUDACC__
#define GBX_HD __host__ __device__
#else
#define GBX_HD
#endif

GBX_HD inline size_t align16(size_t v) { return (v + 15) & ~size_t(15); }

// Nonzero lists of the graph-matching matrices, CSR-like per line:
// list 0 = rows of A, 1 = columns of B, 2 = columns of A, 3 = rows of B;
// entries of a line in increasing index. ok[l] = 0 when list l overflowed.
struct SparseAB {
    int* ok;        // [4]
    int* ptr[4];    // [m + 1]
    int* idx[4];    // [cap]
    double* val[4]; // [cap]
};

GBX_HD inline size_t sparse_list_bytes(int m, int cap) {
    return align16((size_t)(m + 1) * sizeof(int)) + align16((size_t)cap * sizeof(int))
         + align16((size_t)cap * sizeof(double));
}

GBX_HD inline SparseAB sparse_at(unsigned char* base, int m, int cap) {
    SparseAB S;
    S.ok = reinterpret_cast<int*>(base);
    size_t o = 16;
    for (int l = 0; l < 4; ++l) {
        S.ptr[l] = reinterpret_cast<int*>(base + o);
        o += align16((size_t)(m + 1) * sizeof(int));
        S.idx[l] = reinterpret_cast<int*>(base + o);
        o += align16((size_t)cap * sizeof(int));
        S.val[l] = reinterpret_cast<double*>(base + o);
        o += align16((size_t)cap * sizeof(double));
    }
    return S;
}

// Column state of one integer-Hungarian warp held in shared memory instead of
// registers (the large-order kernel, 8 or 16 columns per lane): eight
// [CPL][32] int arrays, lane-contiguous so a warp's access to one slot is
// conflict-free.
enum { CS_COL, CS_PV, CS_MRAW, CS_WAY, CS_PJ, CS_USED, CS_UR, CS_RBR, CS_COUNT };
GBX_HD inline size_t colstate_bytes(int cpl) { return (size_t)CS_COUNT * cpl * 32 * sizeof(int); }

// Thread-block-cluster shape of the large-order mixed kernel (cluster.cuh):
// kClCtas CTAs per node, each holding up to 32 * kClCpl columns of the
// integer oracle costs.
constexpr int kClCtas = 4;              // CTAs of a node's cluster
constexpr int kClCpl = 4;               // columns per lane of a CTA's slice (slices of <= 128 columns)
enum { CL_ORACLE = 1, CL_EXIT = 2 };

// control block of a CTA (the leader's fields are the ones read remotely)
struct ClCtl {
    uint64_t bar_go;      // helpers: the leader posted a command (1 arrival)
    uint64_t bar_done;    // leader: every helper acknowledged the exit (kClCtas - 1 arrivals)
    int cmd[4];           // leader: op, cost shift, in-face restriction unchanged, DICG
    int released;         // leader: the helpers have left
    int err;              // a bounded wait gave up
};

// scal: [0] warm state valid, [1] shift of the stored potentials, [2] k+1 of the
// cached restriction (0: none), [3] first compacted column of this slice,
// [4] compacted columns of this slice, [5] phase events so far, [6] step
// exchanges so far, [8..11] / [12..15] receive slots of the final reductions

GBX_HD inline size_t chw_bytes(int m) {
    return align16((size_t)13 * (m + 1) * sizeof(int)) + align16(3 * 128 * sizeof(int)) + 16 * sizeof(int)
           + align16((size_t)CS_COUNT * kClCpl * 32 * sizeof(int)) + align16(2 * kClCtas * 8 * sizeof(int))
           + 16 * sizeof(int) + 2 * kClCtas * sizeof(int) + align16((size_t)m + 1);
}

// bytes of one FP64 Hungarian workspace (potentials, minv, path, forced maps)
GBX_HD inline size_t hung_ws_bytes(int m) {
    size_t b = 0;
    b += align16(3 * (size_t)(m + 1) * sizeof(double));     // u, pv, minv
    b += align16(2 * (size_t)(m + 1) * sizeof(int));        // p, way
    b += align16(6 * (size_t)m * sizeof(int));              // fcol frow rows cols pi pinv
    b += align16(8 * sizeof(int));                          // scalars
    b += align16((size_t)(m + 1));                          // used
    return b;
}

// bytes of the mixed path's FP32 / int8 node arrays (xf gf Rf Af Bf Btf, Ai Bi)
GBX_HD inline size_t mixed_array_bytes(int n) {
    return align16(6 * (size_t)n * sizeof(float)) + 2 * align16((size_t)n);
}

// bytes of a node's A / -B operand images of the tensor-core gradient
constexpr size_t kTcImageBytes = 2 * 128 * 128 * 2;
constexpr size_t kTcOperandBytes = 4 * 128 * 128 * 2;  // A, -B, two halves of X or R

// bytes of one integer Hungarian workspace of the mixed path (with warm state)
GBX_HD inline size_t ihw_bytes(int m) {
    size_t b = 0;
    b += align16(3 * (size_t)(m + 1) * sizeof(int));   // u rowb pvs
    b += align16(9 * (size_t)m * sizeof(int));         // rows cols rowpos fcol frow pi colpot match pinv
    b += align16((size_t)(m + 1));                     // rmatch
    b += align16(8 * sizeof(int));                     // scalars
    return b;
}

// thread-local message returned by gbx_last_error() (capi.cu)
void set_last_error(const std::string& msg);

// host helpers (relax.cu)
// Launch shape chosen by the autotuner (-1: the default rule).
struct Variant {
    int tc = -1;          // mixed Birkhoff: 1 tensor-core gradient, 0 FP32 SIMT gradient
    int persistent = -1;  // 1 persistent grid, 0 one CTA per node, 2 a cluster of kClCtas CTAs per node,
                          // 3 a pair of CTAs per node (FP64 dense quadratic objective)
    int oracle_warps = -1;  // large-order mixed Birkhoff: warps per integer oracle, 1 or 4
    int per_sm = -1;        // FP64 kernels: nodes (CTAs) per SM the kernel is compiled for, 1 or 2
};
int make_layout(const gbx_objective& o, const gbx_lmo& l, const gbx_algorithm& a,
                int n_nodes, Layout* L, std::string* err, const Variant* v = nullptr);
// the autotuner's choice for this shape (or the defaults)
Variant tuned_variant(const gbx_objective& o, const gbx_lmo& l, const gbx_algorithm& a);
void store_variant(const gbx_objective& o, const gbx_lmo& l, const gbx_algorithm& a, const Variant& v);
// candidate launch shapes of this problem (the first is the default)
std::vector<Variant> candidate_variants(const gbx_objective& o, const gbx_lmo& l, const gbx_algorithm& a);
size_t workspace_bytes(const Layout& L, int n_nodes);
size_t mixed_region_offset(const Layout& L, int n_nodes);  // bytes from the workspace start
size_t sparse_region_offset(const Layout& L, int n_nodes);
size_t queue_offset(const Layout& L, int n_nodes);   // persistent grid's node counter (int)
// workspace that fits every candidate launch shape (what the sizing call reports)
size_t workspace_bytes_any_variant(const gbx_objective& o, const gbx_lmo& l, const gbx_algorithm& a, int n_nodes);
int launch_sparse_build(const gbx_objective& o, const Layout& L, unsigned char* base, cudaStream_t st,
                        std::string* err);
int launch_relax(const Params& p, void* stream, std::string* err);
int launch_lmo_batch(const gbx_lmo& l, int cases, int mode, const double* dir,
                     const double* x, const double* lb, const double* ub, double* out,
                     double* out_step, void* stream, std::string* err);
// the box LMO over cases*n elements in HBM as one vectorised stream (lmo_stream.cu)
int launch_box_lmo_stream(int mode, size_t total, const double* dir, const double* x, const double* lb,
                          const double* ub, double* out, cudaStream_t st, std::string* err);
int launch_gradient_batch(const gbx_objective& o, int precision, int cases, const double* x, double* g,
                          cudaStream_t st, std::string* err);
int scorer_param_count(int F, int H);
int scorer_forward(const gbx_scorer* s, int rows, const float* X, float* z, int bf16, cudaStream_t st,
                   std::string* err);
size_t scorer_workspace_bytes(const gbx_scorer* s, int rows);
int scorer_gradient(const gbx_scorer* s, int rows, const float* X, int groups, const int* gp, const float* target,
                    float* grad, float* loss, void* ws, size_t ws_bytes, cudaStream_t st, std::string* err);
int scorer_adam(gbx_scorer* s, const float* g, float* m, float* v, int step, float lr, cudaStream_t st,
                std::string* err);
int launch_gradient_batch_f32(const gbx_objective& o, int cases, const float* x, float* g, cudaStream_t st,
                              std::string* err);
// branch and bound with the frontier in device memory (frontier.cu); root_x
// is the validated root start point or null
int solve_device_frontier(const gbx_problem& pr, const gbx_objective& obj, const gbx_lmo& lmo,
                          const gbx_settings& s, const double* root_x, gbx_result* res, std::string* err);
size_t frontier_slot_bytes(int n, int compact);
int launch_node_feasible(const gbx_lmo& l, int cases, const double* lb, const double* ub,
                         const uint8_t* flags, uint8_t* out, void* stream, std::string* err);

}  // namespace gbx
