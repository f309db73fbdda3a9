// relax_graph_one.cu -- the FP64 kernels of graph matching compiled for one CTA per SM (no
// register cap), the launch shape the autotuner times against two per SM;
// a unit of its own so that it compiles in parallel with relax_graph.cu.
#include "relax_impl.cuh"

namespace gbx {
template int launch_mix<GBX_OBJ_GRAPH_MATCHING, GBX_LMO_BIRKHOFF, 0, 1>(const Params&, cudaStream_t, std::string*);
template int launch_mix<GBX_OBJ_GRAPH_MATCHING, GBX_LMO_BOX, 0, 1>(const Params&, cudaStream_t, std::string*);
}  // namespace gbx
