// grad_pipe.cu -- gbx_objective_gradient_batch_f32: graph-matching gradients of
// many FP32 points (orders <= 128) on the tensor cores, software-pipelined so
// that the MMAs of one point overlap the loads and epilogues of its neighbours.
//
// Persistent grid, one CTA per SM, 14 warps with fixed roles:
//   warps 0-3   R epilogue: TMEM R -> hi/lo BF16 images (the point's X images
//               are dead once its R MMAs have completed, so R overwrites them)
//   warps 4-7   G epilogue: TMEM G -> 2s * G -> global FP32
//   warps 8-11  converters: global FP32 x -> hi/lo BF16 images
//   warp 12     one thread issues every tcgen05.mma, each product as soon as
//               its inputs are ready (older points' G first)
//   warp 13     TMA producer: quarter points of raw x (32 rows) into two
//               shared-memory stages the converters read
// Shared memory: the A and -B images (built once per call, copied in by TMA) and two operand
// buffers (X, then R, of alternating points). TMEM: R and G accumulators of
// two points in flight (4 x 128 columns). Hand-offs are mbarriers; the k-th
// use of buffer b is phase k of its barriers. Every wait is bounded: a timeout
// sets an error flag and every role stops.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "relax.cuh"
#include "tc_grad.cuh"

namespace gbx {
namespace {

constexpr int kPipeWarps = 14;
constexpr int kStageRows = 32;                                     // rows of x per TMA stage
constexpr int kStageBytes = kStageRows * tc::kDim * 4;              // 16 KB
constexpr int kPipeThreads = kPipeWarps * 32;
constexpr uint32_t kPipeCols = 512;

struct PipeBars {
    uint64_t conv[2], rdone[2], rimg[2], rfree[2], gdone[2], gfree[2], drain, img, sfull[2], sempty[2];
};

__device__ __forceinline__ void bar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(tc::smem_u32(bar)) : "memory");
}

// bounded wait on phase `k` of a barrier; false (and the error flag) on timeout
__device__ __forceinline__ bool wait_k(uint64_t* bar, int k, volatile int* err) {
    if (*err) return false;
    if (!tc::bar_wait(bar, (uint32_t)(k & 1))) { *err = 1; return false; }
    return true;
}

__device__ __forceinline__ void split_store8(unsigned char* hi_img, unsigned char* lo_img, int r, int c0,
                                             const float (&v)[8]) {
    float h[8], l[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) tc::split2(v[k], h[k], l[k]);
    *reinterpret_cast<uint4*>(hi_img + tc::blk_off(r, c0)) =
        make_uint4(tc::pack_bf16(h[0], h[1]), tc::pack_bf16(h[2], h[3]), tc::pack_bf16(h[4], h[5]),
                   tc::pack_bf16(h[6], h[7]));
    *reinterpret_cast<uint4*>(lo_img + tc::blk_off(r, c0)) =
        make_uint4(tc::pack_bf16(l[0], l[1]), tc::pack_bf16(l[2], l[3]), tc::pack_bf16(l[4], l[5]),
                   tc::pack_bf16(l[6], l[7]));
}

// A and -B images, built once per call for every CTA to copy
__global__ void __launch_bounds__(256) pipe_images_kernel(const double* A, const double* B, int m,
                                                          unsigned char* img) {
    const int seg = blockIdx.x * blockDim.x + threadIdx.x;   // one 8-element segment each
    if (seg >= 2 * tc::kDim * (tc::kDim / 8)) return;
    const int which = seg / (tc::kDim * (tc::kDim / 8));
    const int s = seg - which * (tc::kDim * (tc::kDim / 8));
    const int r = s / (tc::kDim / 8), c0 = (s - r * (tc::kDim / 8)) * 8;
    const double* M = which ? B : A;
    const float sg = which ? -1.f : 1.f;
    float v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = (r < m && c0 + k < m) ? sg * (float)M[r * m + c0 + k] : 0.f;
    *reinterpret_cast<uint4*>(img + which * tc::kImgBytes + tc::blk_off(r, c0)) =
        make_uint4(tc::pack_bf16(v[0], v[1]), tc::pack_bf16(v[2], v[3]), tc::pack_bf16(v[4], v[5]),
                   tc::pack_bf16(v[6], v[7]));
}

__global__ void __launch_bounds__(kPipeThreads, 1) grad_pipe_kernel(const unsigned char* img, int m,
                                                                    float two_s, int cases, const float* x,
                                                                    float* g, int* error) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ PipeBars bars;
    __shared__ uint32_t tmem_slot;
    __shared__ int err;
    unsigned char* opA = sm;
    unsigned char* opB = sm + tc::kImgBytes;
    unsigned char* buf[2][2] = {{sm + 2 * tc::kImgBytes, sm + 3 * tc::kImgBytes},
                                {sm + 4 * tc::kImgBytes, sm + 5 * tc::kImgBytes}};
    // two TMA stages of raw FP32 rows (even orders: rows stay 16-byte aligned)
    float* stg[2] = {reinterpret_cast<float*>(sm + 6 * tc::kImgBytes),
                     reinterpret_cast<float*>(sm + 6 * tc::kImgBytes + kStageBytes)};
    const bool staged = (m & 1) == 0;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n = m * m;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(tc::smem_u32(&tmem_slot)), "r"(kPipeCols) : "memory");
    }
    if (tid == 0) {
        err = 0;
        for (int b = 0; b < 2; ++b) {
            tc::bar_init(&bars.conv[b], 128);
            tc::bar_init(&bars.rdone[b], 1);
            tc::bar_init(&bars.rimg[b], 128);
            tc::bar_init(&bars.rfree[b], 128);
            tc::bar_init(&bars.gdone[b], 1);
            tc::bar_init(&bars.gfree[b], 128);
            tc::bar_init(&bars.sfull[b], 1);
            tc::bar_init(&bars.sempty[b], 128);
        }
        tc::bar_init(&bars.drain, 1);
        tc::bar_init(&bars.img, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // the A / -B images by TMA (bulk copies completing on bars.img)
        tc::bar_expect_tx(&bars.img, 2 * tc::kImgBytes);
        tc::bulk_g2s(opA, img, tc::kImgBytes, &bars.img);
        tc::bulk_g2s(opB, img + tc::kImgBytes, tc::kImgBytes, &bars.img);
        if (!tc::bar_wait(&bars.img, 0)) err = 1;
    }
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_slot;
    volatile int* verr = &err;
    // points of this CTA: blockIdx.x, blockIdx.x + gridDim.x, ...
    const int npts = blockIdx.x < cases ? (cases - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    auto point = [&](int i) { return blockIdx.x + i * gridDim.x; };

    if (warp >= 8 && warp < 12) {
        // ---- converters
        const int ct = tid - 256;   // 0..127
        for (int i = 0; i < npts; ++i) {
            const int b = i & 1, k = i >> 1;
            if (k > 0 && !wait_k(&bars.gdone[b], k - 1, verr)) break;
            const float* xp = x + (size_t)point(i) * n;
            if (ct == 0 && i + 1 < npts && !staged) {
                // next point's x into L2 while this one is converted (a hint)
                const uint32_t bytes = (uint32_t)((size_t)n * 4) & ~15u;
                const float* nx = x + (size_t)point(i + 1) * n;
                if (bytes && ((reinterpret_cast<uintptr_t>(nx) & 15) == 0))
                    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" :: "l"(nx), "r"(bytes) : "memory");
            }
            // converter warp cw owns columns 32 cw .. 32 cw + 31; per instruction a
            // warp covers 8 rows x 32 columns. Lane (Q, q) = (lane / 8, lane % 8)
            // converts row 8 rg + q, column block cb = (Q + q / 2) % 4, and reads
            // the half h = q % 2 of its 8 columns first: the eight 16-byte reads of
            // a quarter warp then fall on eight different bank groups of the staged
            // rows (all rows share the banks: the row stride is 128 floats), and
            // its eight 16-byte image stores on eight different rows of core
            // matrices -- neither side has a bank conflict
            const int cw = warp - 8;
            const int cb = ((lane >> 3) + ((lane & 7) >> 1)) & 3, h = lane & 1;
            const int c0 = 8 * (4 * cw + cb);
            const bool vec = (m & 3) == 0 && c0 + 8 <= m;
            bool stop = false;
            for (int q = 0; q < 4 && staged; ++q) {
                // rows 32 q .. 32 q + 31 from TMA stage j % 2
                const int j = 4 * i + q, sg = j & 1;
                if (!wait_k(&bars.sfull[sg], j >> 1, verr)) { stop = true; break; }
                const float* st = stg[sg];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const int lr = 8 * t + (lane & 7), r = kStageRows * q + lr;
                    float v[8];
                    if (r < m && vec) {
                        const float4 a = *reinterpret_cast<const float4*>(st + lr * m + c0 + 4 * h);
                        const float4 b4 = *reinterpret_cast<const float4*>(st + lr * m + c0 + 4 * (1 - h));
                        const float4 lo4 = h ? b4 : a, hi4 = h ? a : b4;
                        v[0] = lo4.x; v[1] = lo4.y; v[2] = lo4.z; v[3] = lo4.w;
                        v[4] = hi4.x; v[5] = hi4.y; v[6] = hi4.z; v[7] = hi4.w;
                    } else {
#pragma unroll
                        for (int e = 0; e < 8; ++e) v[e] = (r < m && c0 + e < m) ? st[lr * m + c0 + e] : 0.f;
                    }
                    split_store8(buf[b][0], buf[b][1], r, c0, v);
                }
                bar_arrive(&bars.sempty[sg]);
            }
            if (stop) break;
            for (int half = 0; half < 2 && !staged; ++half) {
                float v[8][8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int r = 8 * (8 * half + u) + (lane & 7);
                    if (r < m && vec) {
                        const float4 a = *reinterpret_cast<const float4*>(xp + r * m + c0);
                        const float4 b4 = *reinterpret_cast<const float4*>(xp + r * m + c0 + 4);
                        v[u][0] = a.x; v[u][1] = a.y; v[u][2] = a.z; v[u][3] = a.w;
                        v[u][4] = b4.x; v[u][5] = b4.y; v[u][6] = b4.z; v[u][7] = b4.w;
                    } else {
#pragma unroll
                        for (int q = 0; q < 8; ++q) v[u][q] = (r < m && c0 + q < m) ? xp[r * m + c0 + q] : 0.f;
                    }
                }
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    split_store8(buf[b][0], buf[b][1], 8 * (8 * half + u) + (lane & 7), c0, v[u]);
            }
            tc::fence_async_smem();
            bar_arrive(&bars.conv[b]);
        }
    } else if (warp == 13) {
        // ---- TMA producer: quarter q of point i (rows 32 q ..) into stage (4 i + q) % 2
        if (lane == 0 && staged) {
            for (int i = 0; i < npts && !*verr; ++i) {
                const float* xp = x + (size_t)point(i) * n;
                for (int q = 0; q < 4; ++q) {
                    const int j = 4 * i + q, sg = j & 1;
                    if ((j >> 1) > 0 && !wait_k(&bars.sempty[sg], (j >> 1) - 1, verr)) break;
                    const int rows = min(kStageRows, m - kStageRows * q);
                    if (rows > 0) {
                        const uint32_t bytes = (uint32_t)(rows * m * 4);
                        tc::bar_expect_tx(&bars.sfull[sg], bytes);
                        tc::bulk_g2s(stg[sg], xp + kStageRows * q * m, bytes, &bars.sfull[sg]);
                    } else {
                        bar_arrive(&bars.sfull[sg]);
                    }
                }
            }
        }
        __syncwarp();
    } else if (warp == 12) {
        // ---- MMA issuer
        if (lane == 0) {
            const uint32_t id_kmn = tc::idesc_bf16(tc::kDim, tc::kDim, 0, 1);
            const uint32_t id_mnmn = tc::idesc_bf16(tc::kDim, tc::kDim, 1, 1);
            const uint32_t id_kk = tc::idesc_bf16(tc::kDim, tc::kDim, 0, 0);
            auto issue_g = [&](int i) {   // G_i into TMEM G[b]
                const int b = i & 1;
                tc::fence_after();
                const uint32_t d = tmem + 256 + 128 * b;
                for (int ks = 0; ks < tc::kDim / 16; ++ks) {
                    tc::mma(d, tc::mnview(opA, ks), tc::mnview(buf[b][0], ks), id_mnmn, ks > 0);
                    tc::mma(d, tc::mnview(opA, ks), tc::mnview(buf[b][1], ks), id_mnmn, 1);
                }
                for (int ks = 0; ks < tc::kDim / 16; ++ks) {
                    tc::mma(d, tc::kview(buf[b][0], ks), tc::kview(opB, ks), id_kk, 1);
                    tc::mma(d, tc::kview(buf[b][1], ks), tc::kview(opB, ks), id_kk, 1);
                }
                tc::commit(&bars.gdone[b]);
            };
            // greedy issue: whichever product is ready, the older point's G first
            auto issue_r = [&](int i) {
                const int b = i & 1;
                tc::fence_after();
                const uint32_t d = tmem + 128 * b;
                for (int ks = 0; ks < tc::kDim / 16; ++ks) {
                    tc::mma(d, tc::kview(opA, ks), tc::mnview(buf[b][0], ks), id_kmn, ks > 0);
                    tc::mma(d, tc::kview(opA, ks), tc::mnview(buf[b][1], ks), id_kmn, 1);
                }
                for (int ks = 0; ks < tc::kDim / 16; ++ks) {
                    tc::mma(d, tc::kview(buf[b][0], ks), tc::mnview(opB, ks), id_kmn, 1);
                    tc::mma(d, tc::kview(buf[b][1], ks), tc::mnview(opB, ks), id_kmn, 1);
                }
                tc::commit(&bars.rdone[b]);
            };
            int nr = 0, ng = 0;
            long long last = clock64();
            while (ng < npts && !*verr) {
                bool moved = false;
                if (ng < nr) {
                    const int b = ng & 1, k = ng >> 1;
                    if (tc::bar_test(&bars.rimg[b], k & 1) && (k == 0 || tc::bar_test(&bars.gfree[b], (k - 1) & 1))) {
                        issue_g(ng++);
                        moved = true;
                    }
                }
                if (nr < npts) {
                    const int b = nr & 1, k = nr >> 1;
                    if (tc::bar_test(&bars.conv[b], k & 1) && (k == 0 || tc::bar_test(&bars.rfree[b], (k - 1) & 1))) {
                        issue_r(nr++);
                        moved = true;
                    }
                }
                const long long now = clock64();
                if (moved) last = now;
                else if (now - last > tc::kWaitCycles) *verr = 1;
            }
            // every MMA this thread issued has completed once this commit arrives
            tc::commit(&bars.drain);
            if (!tc::bar_wait(&bars.drain, 0)) *verr = 1;
        }
        __syncwarp();
    } else {
        // ---- epilogues: warps 0-3 R (TMEM lanes 32 (w % 4) ..), warps 4-7 G
        const bool rgroup = warp < 4;
        const int row = 32 * (warp & 3) + lane;
        const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
        for (int i = 0; i < npts; ++i) {
            const int b = i & 1, k = i >> 1;
            if (rgroup) {
                if (!wait_k(&bars.rdone[b], k, verr)) break;
                tc::fence_after();
                const uint32_t t0 = tmem + lane_base + 128 * b;
                for (int c0 = 0; c0 < tc::kDim; c0 += 32) {
                    float v[32];
                    tc::tmem_ld32(t0 + c0, v);
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        float w8[8];
#pragma unroll
                        for (int e = 0; e < 8; ++e) w8[e] = v[8 * q + e];
                        split_store8(buf[b][0], buf[b][1], row, c0 + 8 * q, w8);
                    }
                }
                tc::fence_before();
                tc::fence_async_smem();
                bar_arrive(&bars.rfree[b]);
                bar_arrive(&bars.rimg[b]);
            } else {
                if (!wait_k(&bars.gdone[b], k, verr)) break;
                tc::fence_after();
                const uint32_t t0 = tmem + lane_base + 256 + 128 * b;
                float* gp = g + (size_t)point(i) * n;
                for (int c0 = 0; c0 < tc::kDim; c0 += 32) {
                    float v[32];
                    tc::tmem_ld32(t0 + c0, v);
                    if (row < m) {
                        if ((m & 3) == 0 && c0 + 32 <= m) {
#pragma unroll
                            for (int e = 0; e < 32; e += 4)
                                *reinterpret_cast<float4*>(gp + row * m + c0 + e) =
                                    make_float4(two_s * v[e], two_s * v[e + 1], two_s * v[e + 2], two_s * v[e + 3]);
                        } else {
#pragma unroll
                            for (int e = 0; e < 32; ++e)
                                if (c0 + e < m) gp[row * m + c0 + e] = two_s * v[e];
                        }
                    }
                }
                tc::fence_before();
                bar_arrive(&bars.gfree[b]);
            }
        }
    }
    tc::fence_before();
    __syncthreads();
    if (err && tid == 0) atomicExch(error, 1);
    tc::fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(kPipeCols) : "memory");
}

}  // namespace

int launch_gradient_batch_f32(const gbx_objective& o, int cases, const float* x, float* g, cudaStream_t st,
                              std::string* err) {
    if (cases == 0) return GBX_OK;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t smem = 6 * (size_t)tc::kImgBytes + 2 * (size_t)kStageBytes;
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(grad_pipe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    unsigned char* scratch = nullptr;   // [A image | -B image | error flag]
    if (e == cudaSuccess) e = cudaMallocAsync(&scratch, 2 * (size_t)tc::kImgBytes + 256, st);
    int* flag = scratch ? reinterpret_cast<int*>(scratch + 2 * (size_t)tc::kImgBytes) : nullptr;
    if (e == cudaSuccess) e = cudaMemsetAsync(flag, 0, sizeof(int), st);
    if (e == cudaSuccess) {
        pipe_images_kernel<<<(2 * tc::kDim * (tc::kDim / 8) + 255) / 256, 256, 0, st>>>(o.A, o.B, o.order, scratch);
        const int grid = std::min(cases, sms);
        grad_pipe_kernel<<<grid, kPipeThreads, smem, st>>>(scratch, o.order, (float)(2.0 * o.scale), cases, x, g,
                                                           flag);
        e = cudaGetLastError();
    }
    int h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (scratch) cudaFreeAsync(scratch, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    if (h) { *err = "gradient pipeline: a tensor-core wait timed out"; return GBX_ERR_TIMEOUT; }
    return GBX_OK;
}

}  // namespace gbx
