// relax_graph_mixed2.cu -- the mixed-precision Birkhoff kernel, variant 2 (tensor-core gradient).
#include "relax_impl.cuh"

namespace gbx {
template int launch_mix<GBX_OBJ_GRAPH_MATCHING, GBX_LMO_BIRKHOFF, 2>(const Params&, cudaStream_t, std::string*);
}  // namespace gbx
