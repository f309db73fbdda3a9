// relax_graph.cu -- kernels of the graph-matching objective: the FP64 ones here,
// the mixed-precision Birkhoff variants in relax_graph_mixed*.cu (one unit
// each, so they compile in parallel).
#include "relax_impl.cuh"

namespace gbx {
// the one-CTA-per-SM FP64 kernels compile in relax_graph_one.cu
extern template int launch_mix<GBX_OBJ_GRAPH_MATCHING, GBX_LMO_BIRKHOFF, 0, 1>(const Params&, cudaStream_t, std::string*);
extern template int launch_mix<GBX_OBJ_GRAPH_MATCHING, GBX_LMO_BOX, 0, 1>(const Params&, cudaStream_t, std::string*);
extern template int launch_mix<GBX_OBJ_GRAPH_MATCHING, GBX_LMO_BIRKHOFF, 1>(const Params&, cudaStream_t,
                                                                             std::string*);
extern template int launch_mix<GBX_OBJ_GRAPH_MATCHING, GBX_LMO_BIRKHOFF, 2>(const Params&, cudaStream_t,
                                                                             std::string*);
extern template int launch_mix<GBX_OBJ_GRAPH_MATCHING, GBX_LMO_BIRKHOFF, 3>(const Params&, cudaStream_t,
                                                                             std::string*);
extern template int launch_cluster<GBX_OBJ_GRAPH_MATCHING, GBX_LMO_BIRKHOFF>(const Params&, cudaStream_t,
                                                                            std::string*);
template int launch_one<GBX_OBJ_GRAPH_MATCHING, GBX_LMO_BIRKHOFF>(const Params&, cudaStream_t, std::string*);
template int launch_one<GBX_OBJ_GRAPH_MATCHING, GBX_LMO_BOX>(const Params&, cudaStream_t, std::string*);
}  // namespace gbx
