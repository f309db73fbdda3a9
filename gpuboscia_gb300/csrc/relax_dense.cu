// relax_dense.cu -- kernels of the dense quadratic objective over every LMO.
#include "relax_impl.cuh"

namespace gbx {
template int launch_one<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_BOX>(const Params&, cudaStream_t, std::string*);
template int launch_one<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_SIMPLEX>(const Params&, cudaStream_t, std::string*);
template int launch_one<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_EQUALITY_SIMPLEX>(const Params&, cudaStream_t, std::string*);
template int launch_one<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_BIRKHOFF>(const Params&, cudaStream_t, std::string*);
template int launch_one<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_CARDINALITY>(const Params&, cudaStream_t, std::string*);
template int launch_one<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_LINKED_CARDINALITY>(const Params&, cudaStream_t, std::string*);
}  // namespace gbx
