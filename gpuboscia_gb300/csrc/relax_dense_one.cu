// relax_dense_one.cu -- the FP64 kernels of the box and simplex LMOs compiled for one CTA per SM (no
// register cap), the launch shape the autotuner times against two per SM;
// a unit of its own so that it compiles in parallel with relax_dense.cu.
#include "relax_impl.cuh"

namespace gbx {
template int launch_mix<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_BOX, 0, 1>(const Params&, cudaStream_t, std::string*);
template int launch_mix<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_SIMPLEX, 0, 1>(const Params&, cudaStream_t, std::string*);
template int launch_mix<GBX_OBJ_DENSE_QUADRATIC, GBX_LMO_EQUALITY_SIMPLEX, 0, 1>(const Params&, cudaStream_t, std::string*);
}  // namespace gbx
