// relax.cuh -- shared declarations of the node-relaxation kernels.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

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
    // x, gradient, residual, A, B, B' [6 n floats], forward / in-face integer
    // oracle costs [2 n ints], edge / face code bytes
    // [2 n], and two integer Hungarian workspaces with warm state
    int mixed;
    size_t sm_mx, sm_code, sm_ihw, ihw_bytes;
    size_t mixed_node_bytes;
};

struct Params {
    gbx_objective obj;
    gbx_lmo lmo;
    gbx_algorithm alg;
    gbx_node_batch b;
    Layout L;
    double* ws;             // global workspace (node vectors when not in smem)
    unsigned char* mixed;   // mixed-precision scratch
};

#ifdef __CUDACC__
#define GBX_HD __host__ __device__
#else
#define GBX_HD
#endif

GBX_HD inline size_t align16(size_t v) { return (v + 15) & ~size_t(15); }

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
int make_layout(const gbx_objective& o, const gbx_lmo& l, const gbx_algorithm& a,
                int n_nodes, Layout* L, std::string* err);
size_t workspace_bytes(const Layout& L, int n_nodes);
int launch_relax(const Params& p, void* stream, std::string* err);
int launch_lmo_batch(const gbx_lmo& l, int cases, int mode, const double* dir,
                     const double* x, const double* lb, const double* ub, double* out,
                     double* out_step, void* stream, std::string* err);
int launch_node_feasible(const gbx_lmo& l, int cases, const double* lb, const double* ub,
                         const uint8_t* flags, uint8_t* out, void* stream, std::string* err);

}  // namespace gbx
