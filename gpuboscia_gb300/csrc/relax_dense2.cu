// relax_dense2.cu -- kernels of the dense quadratic objective over the
// Birkhoff, cardinality and linked cardinality LMOs.
#include "relax_impl.cuh"

namespace gbx {
template int launch_one<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_BIRKHOFF>(const Params&, cudaStream_t, std::string*);
template int launch_one<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_CARDINALITY>(const Params&, cudaStream_t, std::string*);
template int launch_one<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_LINKED_CARDINALITY>(const Params&, cudaStream_t, std::string*);
}  // namespace gbx
