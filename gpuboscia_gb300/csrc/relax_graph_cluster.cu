// relax_graph_cluster.cu -- the mixed-precision Birkhoff kernel on a cluster of CTAs per node (large orders).
#include "relax_impl.cuh"

namespace gbx {
template int launch_cluster<GBX_OBJ_GRAPH_MATCHING, GBX_LMO_BIRKHOFF>(const Params&, cudaStream_t, std::string*);
}  // namespace gbx
