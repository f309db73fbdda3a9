// relax_pair.cu -- the dense quadratic objective's kernels with a pair of CTAs
// per node (a two-CTA cluster splitting the objective's products), a launch
// shape for batches smaller than the GPU; a unit of its own so that it
// compiles in parallel with relax_dense.cu and relax_dense2.cu.
#include "relax_impl.cuh"

namespace gbx {
template int launch_pair<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_BOX>(const Params&, cudaStream_t, std::string*);
template int launch_pair<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_SIMPLEX>(const Params&, cudaStream_t, std::string*);
template int launch_pair<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_EQUALITY_SIMPLEX>(const Params&, cudaStream_t, std::string*);
template int launch_pair<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_BIRKHOFF>(const Params&, cudaStream_t, std::string*);
template int launch_pair<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_CARDINALITY>(const Params&, cudaStream_t, std::string*);
template int launch_pair<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_LINKED_CARDINALITY>(const Params&, cudaStream_t, std::string*);
}  // namespace gbx
