// relax_graph.cu -- kernels of the graph-matching objective (FP64 and mixed precision).
#include "relax_impl.cuh"

namespace gbx {
template int launch_one<GBX_OBJ_GRAPH_MATCHING, GBX_LMO_BIRKHOFF>(const Params&, cudaStream_t, std::string*);
template int launch_one<GBX_OBJ_GRAPH_MATCHING, GBX_LMO_BOX>(const Params&, cudaStream_t, std::string*);
}  // namespace gbx
