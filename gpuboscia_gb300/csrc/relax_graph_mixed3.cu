// relax_graph_mixed3.cu -- the mixed-precision Birkhoff kernel, variant 3 (large orders, costs in the workspace).
#include "relax_impl.cuh"

namespace gbx {
template int launch_mix<GBX_OBJ_GRAPH_MATCHING, GBX_LMO_BIRKHOFF, 3>(const Params&, cudaStream_t, std::string*);
}  // namespace gbx
