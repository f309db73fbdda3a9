// lmo_stream.cu -- the box LMO over a batch held in HBM.
//
// The box oracles are element-wise (BoxLMO::compute_v and compute_inface_v,
// lmo.cuh:270-300: v_j = lb_j where the direction is positive, ub_j
// otherwise; the in-face oracle keeps a coordinate at the bound x already
// sits on, within 1e-6 + 1e-4 |bound|). A batch of cases is then one flat
// stream of cases*n elements with no per-case state: a grid of resident CTAs
// strides over it with 16-byte loads and stores (two doubles per access,
// every warp access a contiguous 512 bytes), marked evict-first since nothing
// is reused. Bytes per element: 32 forward (direction, lb, ub in; v out), 40
// in-face (x as well). Results are the per-node kernel's, bit for bit: the
// same comparisons on the same doubles.
#include <cstdint>

#include "relax.cuh"

namespace gbx {
namespace {

constexpr int kStreamThreads = 256;

template <int MODE>
__device__ __forceinline__ double box_vertex(double g, double x, double l, double u) {
    if constexpr (MODE == 1) {
        const double atol = 1e-6, rtol = 1e-4;
        const double ut = atol + rtol * fabs(u);
        const double lt = atol + rtol * fabs(l);
        if (fabs(x - u) <= ut) return u;
        if (fabs(x - l) <= lt) return l;
    }
    return g > 0.0 ? l : u;
}

// VEC: every pointer 16-byte aligned; pairs of doubles per access, the odd
// last element (when total is odd) by thread 0 of CTA 0
template <int MODE, bool VEC>
__global__ void __launch_bounds__(kStreamThreads) box_lmo_stream_kernel(
    size_t total, const double* __restrict__ dir, const double* __restrict__ x,
    const double* __restrict__ lb, const double* __restrict__ ub, double* __restrict__ out) {
    const size_t stride = (size_t)gridDim.x * kStreamThreads;
    const size_t first = (size_t)blockIdx.x * kStreamThreads + threadIdx.x;
    if constexpr (VEC) {
        const size_t pairs = total >> 1;
        const double2* d2 = reinterpret_cast<const double2*>(dir);
        const double2* x2 = reinterpret_cast<const double2*>(x);
        const double2* l2 = reinterpret_cast<const double2*>(lb);
        const double2* u2 = reinterpret_cast<const double2*>(ub);
        double2* o2 = reinterpret_cast<double2*>(out);
        for (size_t p = first; p < pairs; p += stride) {
            const double2 g = __ldcs(d2 + p);
            const double2 l = __ldcs(l2 + p);
            const double2 u = __ldcs(u2 + p);
            double2 xx = make_double2(0.0, 0.0);
            if constexpr (MODE == 1) xx = __ldcs(x2 + p);
            double2 v;
            v.x = box_vertex<MODE>(g.x, xx.x, l.x, u.x);
            v.y = box_vertex<MODE>(g.y, xx.y, l.y, u.y);
            __stcs(o2 + p, v);
        }
        if ((total & 1) && first == 0) {
            const size_t j = total - 1;
            out[j] = box_vertex<MODE>(dir[j], MODE == 1 ? x[j] : 0.0, lb[j], ub[j]);
        }
    } else {
        for (size_t j = first; j < total; j += stride)
            __stcs(out + j, box_vertex<MODE>(__ldcs(dir + j), MODE == 1 ? __ldcs(x + j) : 0.0,
                                              __ldcs(lb + j), __ldcs(ub + j)));
    }
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

}  // namespace

// One launch over cases*n elements; mode 0 forward, 1 in-face (x required).
int launch_box_lmo_stream(int mode, size_t total, const double* dir, const double* x, const double* lb,
                          const double* ub, double* out, cudaStream_t st, std::string* err) {
    if (total == 0) return GBX_OK;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    const bool vec = aligned16(dir) && aligned16(lb) && aligned16(ub) && aligned16(out) &&
                     (mode == 0 || aligned16(x));
    auto k = mode == 0 ? (vec ? box_lmo_stream_kernel<0, true> : box_lmo_stream_kernel<0, false>)
                       : (vec ? box_lmo_stream_kernel<1, true> : box_lmo_stream_kernel<1, false>);
    // one wave of resident CTAs (as many per SM as the registers allow)
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kStreamThreads, 0);
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    const size_t items = vec ? total / 2 : total;
    const size_t need = (items + kStreamThreads - 1) / kStreamThreads;
    const size_t full = (size_t)sms * (size_t)(per_sm > 0 ? per_sm : 1);
    const unsigned grid = (unsigned)(need < full ? (need > 0 ? need : 1) : full);
    k<<<grid, kStreamThreads, 0, st>>>(total, dir, x, lb, ub, out);
    e = cudaGetLastError();
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    return GBX_OK;
}

}  // namespace gbx
