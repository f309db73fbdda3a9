// grad_batch.cu -- gbx_objective_gradient_batch: objective gradients at a batch
// of points, one CTA per point, with the relaxation's own gradient code (FP64)
// or the mixed-precision one (tensor cores for orders 65..128, FP32 below).
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "relax_impl.cuh"

namespace gbx {
namespace {

// per-point scratch of the mixed gradient: xf, gf, Rf, A, B, B' (FP32), then
// the A / -B operand images
size_t mixed_point_bytes(int n) {
    return (align16(6 * (size_t)n * sizeof(float)) + 255) / 256 * 256 + kTcImageBytes;
}

__global__ void __launch_bounds__(kThreads, 1) grad_fp64_kernel(gbx_objective o, int cases, const double* x,
                                                                double* g, double* ws) {
    __shared__ double red[40];
    __shared__ int flag[8];
    const int k = blockIdx.x;
    if (k >= cases) return;
    Ctx c{};
    c.n = o.n;
    c.tid = threadIdx.x;
    c.red = red;
    c.flag = flag;
    c.ok = o.kind;
    c.m = o.order;
    c.Q = o.Q;
    c.c = o.c;
    c.s = o.scale;
    c.ls = o.linear_scale;
    c.k0 = o.constant;
    c.A = o.A;
    c.B = o.B;
    c.R = ws + (size_t)k * o.n;
    c.pr = -1;   // one CTA per gradient: no pair exchange
    c.xch = nullptr;
    obj_grad(c, x + (size_t)k * o.n, g + (size_t)k * o.n);
}

__global__ void __launch_bounds__(kThreads, 1) grad_mixed_kernel(gbx_objective o, int cases, const double* x,
                                                                 double* g, unsigned char* ws, size_t stride) {
    extern __shared__ __align__(16) unsigned char dsm[];
    __shared__ uint64_t bars[2];
    __shared__ uint32_t slot;
    const int k = blockIdx.x;
    if (k >= cases) return;
    const int n = o.n, m = o.order, tid = threadIdx.x;
    unsigned char* base = ws + (size_t)k * stride;
    float* xf = reinterpret_cast<float*>(base);
    float* gf = xf + n;
    float* Rf = gf + n;
    float* Af = Rf + n;
    float* Bf = Af + n;
    float* Btf = Bf + n;
    const double* xk = x + (size_t)k * n;
    for (int e = tid; e < n; e += kThreads) xf[e] = (float)xk[e];
    const float two_s = (float)(2.0 * o.scale);
    if (m > 64) {
        tc::Grad t;
        t.opA = dsm;
        t.opB = dsm + tc::kImgBytes;
        t.op0 = dsm + 2 * tc::kImgBytes;
        t.op1 = dsm + 3 * tc::kImgBytes;
        t.bar_tma = &bars[0];
        t.bar_mma = &bars[1];
        t.tmem_slot = &slot;
        unsigned char* img = base + (align16(6 * (size_t)n * sizeof(float)) + 255) / 256 * 256;
        t.img = img;
        t.ph_tma = t.ph_mma = 0;
        tc::build_images(img, o.A, o.B, m);
        tc::fence_async_all();
        if (tid < 32) tc::tmem_alloc(&slot);
        if (tid == 0) {
            tc::bar_init(&bars[0], 1);
            tc::bar_init(&bars[1], 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
        const bool ok = tc::gradient(t, m, xf, two_s, gf, nullptr);
        if (!ok && tid == 0) tc::bar_wait(t.bar_mma, t.ph_mma);
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
        if (tid < 32) tc::tmem_dealloc(slot);
        const double nan = __longlong_as_double(0x7ff8000000000000ll);
        for (int e = tid; e < n; e += kThreads) g[(size_t)k * n + e] = ok ? (double)gf[e] : nan;
        return;
    }
    for (int e = tid; e < n; e += kThreads) {
        const int i = e / m, j = e - (e / m) * m;
        Af[e] = (float)o.A[e];
        Bf[e] = (float)o.B[e];
        Btf[e] = (float)o.B[j * m + i];
    }
    __syncthreads();
    grad_f32(m, two_s, Af, Bf, Btf, xf, Rf, gf);
    for (int e = tid; e < n; e += kThreads) g[(size_t)k * n + e] = (double)gf[e];
}

}  // namespace

int launch_gradient_batch(const gbx_objective& o, int precision, int cases, const double* x, double* g,
                          cudaStream_t st, std::string* err) {
    if (cases == 0) return GBX_OK;
    cudaError_t e = cudaSuccess;
    if (precision == GBX_PRECISION_FP64) {
        double* ws = nullptr;
        e = cudaMallocAsync(&ws, (size_t)cases * o.n * sizeof(double), st);
        if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
        grad_fp64_kernel<<<cases, kThreads, 0, st>>>(o, cases, x, g, ws);
        e = cudaGetLastError();
        cudaFreeAsync(ws, st);
    } else {
        const size_t stride = mixed_point_bytes(o.n);
        unsigned char* ws = nullptr;
        e = cudaMallocAsync(&ws, (size_t)cases * stride, st);
        if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
        const int smem = o.order > 64 ? (int)kTcOperandBytes : 0;
        e = cudaFuncSetAttribute(grad_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 std::max(smem, 1));
        if (e == cudaSuccess) {
            grad_mixed_kernel<<<cases, kThreads, smem, st>>>(o, cases, x, g, ws, stride);
            e = cudaGetLastError();
        }
        cudaFreeAsync(ws, st);
    }
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    return GBX_OK;
}

}  // namespace gbx
