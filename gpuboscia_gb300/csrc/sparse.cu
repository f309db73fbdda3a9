// sparse.cu -- nonzero lists of the graph-matching matrices A and B, built once
// per relaxation launch into the workspace. The FP64 residual and gradient then
// skip the terms whose matrix coefficient is zero: with finite operands such a
// term adds a signed zero to an accumulator that is never -0, so the sums are
// bit-identical to the dense loops (the kernel checks finiteness first).
#include <cuda_runtime.h>

#include <string>

#include "relax.cuh"

namespace gbx {
namespace {

// block l builds list l: 0 rows of A, 1 columns of B, 2 columns of A, 3 rows of B
__global__ void __launch_bounds__(256) sparse_build_kernel(const double* A, const double* B, int m, int cap,
                                                           unsigned char* base) {
    __shared__ int cnt[1025];
    const SparseAB S = sparse_at(base, m, cap);
    const int l = blockIdx.x;
    const double* M = (l == 0 || l == 2) ? A : B;
    const bool by_row = l == 0 || l == 3;
    for (int line = threadIdx.x; line < m; line += blockDim.x) {
        int c = 0;
        for (int k = 0; k < m; ++k) c += (by_row ? M[line * m + k] : M[k * m + line]) != 0.0;
        cnt[line] = c;
    }
    __syncthreads();
    __shared__ int total;
    if (threadIdx.x == 0) {
        int t = 0;
        for (int line = 0; line < m; ++line) { S.ptr[l][line] = t; t += cnt[line]; }
        S.ptr[l][m] = t;
        total = t;
        S.ok[l] = t <= cap ? 1 : 0;
    }
    __syncthreads();
    if (total > cap) return;
    for (int line = threadIdx.x; line < m; line += blockDim.x) {
        int o = S.ptr[l][line];
        for (int k = 0; k < m; ++k) {
            const double v = by_row ? M[line * m + k] : M[k * m + line];
            if (v != 0.0) { S.idx[l][o] = k; S.val[l][o] = v; ++o; }
        }
    }
}

}  // namespace

int launch_sparse_build(const gbx_objective& o, const Layout& L, unsigned char* base, cudaStream_t st,
                        std::string* err) {
    if (o.order > 1024) { *err = "graph order above 1024"; return GBX_ERR_UNSUPPORTED; }
    sparse_build_kernel<<<4, 256, 0, st>>>(o.A, o.B, o.order, L.sparse_cap, base);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    return GBX_OK;
}

}  // namespace gbx
