// relax_dense2.cu -- kernels of the dense quadratic objective over the
// Birkhoff, cardinality and linked cardinality LMOs.
#include "relax_impl.cuh"

namespace gbx {
// the pair-per-node kernels compile in relax_pair.cu
extern template int launch_pair<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_BIRKHOFF>(const Params&, cudaStream_t, std::string*);
extern template int launch_pair<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_CARDINALITY>(const Params&, cudaStream_t, std::string*);
extern template int launch_pair<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_LINKED_CARDINALITY>(const Params&, cudaStream_t, std::string*);
// the one-CTA-per-SM FP64 kernels compile in relax_dense2_one.cu
extern template int launch_mix<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_BIRKHOFF, 0, 1>(const Params&, cudaStream_t, std::string*);
extern template int launch_mix<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_CARDINALITY, 0, 1>(const Params&, cudaStream_t, std::string*);
extern template int launch_mix<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_LINKED_CARDINALITY, 0, 1>(const Params&, cudaStream_t, std::string*);
template int launch_one<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_BIRKHOFF>(const Params&, cudaStream_t, std::string*);
template int launch_one<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_CARDINALITY>(const Params&, cudaStream_t, std::string*);
template int launch_one<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_LINKED_CARDINALITY>(const Params&, cudaStream_t, std::string*);
}  // namespace gbx
