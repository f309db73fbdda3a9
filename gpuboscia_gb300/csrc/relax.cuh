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
    int off[B_COUNT];       // offset in doubles inside the node-vector block (-1: absent)
    int nvec;
    int vec_smem;           // node vectors in dynamic shared memory
    size_t node_stride;     // doubles per node in the global workspace
    int obj_smem;           // objective matrices staged in shared memory
    size_t obj_doubles;
    int sort_size;          // simplex bitonic network size (0: none)
    int hung_order;         // Birkhoff order (0: none)
    int hung_warps;         // Hungarian workspaces (1 or 2)
    size_t hung_bytes;      // bytes per Hungarian workspace
    // byte offsets inside dynamic shared memory
    size_t sm_vec, sm_obj, sm_keys, sm_prefix, sm_idx, sm_fixed, sm_hung, sm_total;
    // bytes of the mixed-precision scratch (per node, global)
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
