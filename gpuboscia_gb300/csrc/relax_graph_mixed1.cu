// relax_graph_mixed1.cu -- the mixed-precision Birkhoff kernel, variant 1 (FP32 SIMT gradient).
#include "relax_impl.cuh"

namespace gbx {
template int launch_mix<GBX_OBJ_GRAPH_MATCHING, GBX_LMO_BIRKHOFF, 1>(const Params&, cudaStream_t, std::string*);
}  // namespace gbx
