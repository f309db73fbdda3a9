// relax_dense.cu -- kernels of the dense quadratic objective over the box and
// simplex LMOs (the other LMOs: relax_dense2.cu; two units compile in parallel).
#include "relax_impl.cuh"

namespace gbx {
// the pair-per-node kernels compile in relax_pair.cu
extern template int launch_pair<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_BOX>(const Params&, cudaStream_t, std::string*);
extern template int launch_pair<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_SIMPLEX>(const Params&, cudaStream_t, std::string*);
extern template int launch_pair<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_EQUALITY_SIMPLEX>(const Params&, cudaStream_t, std::string*);
// the one-CTA-per-SM FP64 kernels compile in relax_dense_one.cu
extern template int launch_mix<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_BOX, 0, 1>(const Params&, cudaStream_t, std::string*);
extern template int launch_mix<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_SIMPLEX, 0, 1>(const Params&, cudaStream_t, std::string*);
extern template int launch_mix<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_EQUALITY_SIMPLEX, 0, 1>(const Params&, cudaStream_t, std::string*);
template int launch_one<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_BOX>(const Params&, cudaStream_t, std::string*);
template int launch_one<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_SIMPLEX>(const Params&, cudaStream_t, std::string*);
template int launch_one<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_EQUALITY_SIMPLEX>(const Params&, cudaStream_t, std::string*);
}  // namespace gbx
