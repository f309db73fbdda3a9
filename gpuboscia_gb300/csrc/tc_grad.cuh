// tc_grad.cuh -- graph-matching gradient on the 5th-generation tensor cores.
//
// For one node (Birkhoff order 64 < m <= 128) the mixed-precision loop needs
//     R = A X - X B,   G = 2s (A' R - R B')
// in FP32. The four products run as tcgen05.mma kind::f16 with BF16 operands
// and FP32 accumulation in tensor memory (TMEM), every dimension padded to 128:
//   * A and B are small integers (graph adjacency), exact in BF16; -B is
//     stored so that every product accumulates;
//   * X (and then R) is carried as a split pair hi = bf16(v), lo = bf16(v - hi),
//     about 16 significant bits, and each product runs once per half.
// Operands sit in shared memory in 8x8 blocks of 128 bytes (a row of 8 BF16 per
// 16 bytes); one image serves as the K-major operand of a matrix and as the
// MN-major operand of its transpose, so A, -B, X and R need one copy each.
// The A / -B images are built once per launch in the node's workspace and
// brought in by TMA (cp.async.bulk) every iteration, because the shared memory
// they use is the integer cost matrices' during the oracle phase.
//
// One elected thread issues the MMAs; completion is signalled through an
// mbarrier by tcgen05.commit. Every wait is bounded (kWaitCycles): on a
// timeout the caller stops iterating and the FP64 certificate is computed at
// the iterate reached, so a node's result stays exact.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

namespace gbx {
namespace tc {

constexpr int kDim = 128;                        // padded M = N = K
constexpr int kBlkRow = (kDim / 8) * 128;        // bytes between 8-row blocks (2048)
constexpr int kImgBytes = kDim * kDim * 2;       // one BF16 operand image (32 KB)
constexpr uint32_t kTmemCols = 128;              // one FP32 128x128 accumulator
constexpr long long kWaitCycles = 1ll << 31;     // ~1 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (r, c) inside a blocked 128x128 BF16 image
__device__ __forceinline__ int blk_off(int r, int c) {
    return (r >> 3) * kBlkRow + (c >> 3) * 128 + (r & 7) * 16 + (c & 7) * 2;
}

// Shared-memory matrix descriptor, no swizzle: start, leading-dimension byte
// offset (between core matrices adjacent along K for K-major operands) and
// stride-dimension byte offset, descriptor version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFF) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16: BF16 A and B, FP32 D, M x N, with the
// K-major (0) or MN-major (1) flag of each operand.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N, int a_mn, int b_mn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)a_mn << 15) | ((uint32_t)b_mn << 16)
         | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
        :: "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(acc) : "memory");
}

__device__ __forceinline__ void commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_async_all() { asm volatile("fence.proxy.async;" ::: "memory"); }

__device__ __forceinline__ void bar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool bar_try(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return ok != 0;
}

// non-blocking test of the phase with the given parity
__device__ __forceinline__ bool bar_test(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return ok != 0;
}

// bounded wait for the phase with the given parity to complete
__device__ __forceinline__ bool bar_wait(uint64_t* bar, uint32_t parity) {
    const long long t0 = clock64();
    for (uint32_t i = 0;; ++i) {
        if (bar_try(bar, parity)) return true;
        if ((i & 15) == 15 && clock64() - t0 > kWaitCycles) return false;
    }
}

__device__ __forceinline__ void bar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 :: "r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// TMA bulk copy global -> shared (16-byte aligned, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

// whole warp: allocate kTmemCols columns, base address written to *slot. The
// CTA keeps its allocation permit: a persistent CTA allocates again for every
// node it takes (each allocation is released by tmem_dealloc first).
__device__ __forceinline__ void tmem_alloc(uint32_t* slot) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_u32(slot)), "r"(kTmemCols) : "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t base) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(base), "r"(kTmemCols) : "memory");
}

// whole warp: 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr) : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const uint32_t lo = __bfloat16_as_ushort(__float2bfloat16_rn(a));
    const uint32_t hi = __bfloat16_as_ushort(__float2bfloat16_rn(b));
    return lo | (hi << 16);
}

// split v into bf16 hi + bf16 lo
__device__ __forceinline__ void split2(float v, float& hi, float& lo) {
    hi = __bfloat162float(__float2bfloat16_rn(v));
    lo = v - hi;
}

// Per-CTA state of the tensor-core gradient.
struct Grad {
    unsigned char* opA;        // shared: A image
    unsigned char* opB;        // shared: -B image
    unsigned char* op0;        // shared: X hi, then R hi
    unsigned char* op1;        // shared: X lo, then R lo
    uint64_t* bar_tma;         // TMA completion
    uint64_t* bar_mma;         // MMA completion
    uint32_t* tmem_slot;       // TMEM base written by tcgen05.alloc
    const unsigned char* img;  // global: A image, then -B image (2 * kImgBytes)
    uint32_t ph_tma, ph_mma;   // parities of the next phases to wait for
};

// Build the A / -B images of one node in global memory (all threads; the
// caller fences and synchronises before the first TMA read).
__device__ inline void build_images(unsigned char* img, const double* A, const double* B, int m) {
    for (int seg = threadIdx.x; seg < 2 * kDim * (kDim / 8); seg += blockDim.x) {
        const int which = seg / (kDim * (kDim / 8));
        const int s = seg - which * (kDim * (kDim / 8));
        const int r = s / (kDim / 8), c0 = (s - r * (kDim / 8)) * 8;
        const double* M = which ? B : A;
        const float sg = which ? -1.f : 1.f;
        float v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = (r < m && c0 + k < m) ? sg * (float)M[r * m + c0 + k] : 0.f;
        uint4 q;
        q.x = pack_bf16(v[0], v[1]);
        q.y = pack_bf16(v[2], v[3]);
        q.z = pack_bf16(v[4], v[5]);
        q.w = pack_bf16(v[6], v[7]);
        *reinterpret_cast<uint4*>(img + which * kImgBytes + blk_off(r, c0)) = q;
    }
}

// Descriptors of the two views of a blocked image at K step ks (16 deep).
// K-major (rows = M or N, columns = K): core matrices adjacent along K are
// 128 bytes apart (LBO), along M/N one block row apart (SBO).
__device__ __forceinline__ uint64_t kview(const unsigned char* op, int ks) {
    return sdesc(smem_u32(op) + ks * 256, 128, kBlkRow);
}
// MN-major (rows = K, columns = M or N): along K one block row apart (LBO),
// along M/N 128 bytes apart (SBO).
__device__ __forceinline__ uint64_t mnview(const unsigned char* op, int ks) {
    return sdesc(smem_u32(op) + ks * 2 * kBlkRow, kBlkRow, 128);
}

// G (and R when Rf != nullptr) of the node's FP32 iterate xf; m x m row-major
// outputs in global memory. All threads of the CTA call it; returns false
// when a wait timed out (G is then not valid).
__device__ inline bool gradient(Grad& t, int m, const float* xf, float two_s, float* gf, float* Rf) {
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t tmem = *t.tmem_slot;
    // X split into the two operand images (pads are zero)
    for (int s = tid; s < kDim * (kDim / 8); s += blockDim.x) {
        const int r = s / (kDim / 8), c0 = (s - r * (kDim / 8)) * 8;
        float h[8], l[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) split2((r < m && c0 + k < m) ? xf[r * m + c0 + k] : 0.f, h[k], l[k]);
        const uint4 qh = make_uint4(pack_bf16(h[0], h[1]), pack_bf16(h[2], h[3]), pack_bf16(h[4], h[5]),
                                    pack_bf16(h[6], h[7]));
        const uint4 ql = make_uint4(pack_bf16(l[0], l[1]), pack_bf16(l[2], l[3]), pack_bf16(l[4], l[5]),
                                    pack_bf16(l[6], l[7]));
        *reinterpret_cast<uint4*>(t.op0 + blk_off(r, c0)) = qh;
        *reinterpret_cast<uint4*>(t.op1 + blk_off(r, c0)) = ql;
    }
    fence_async_smem();
    __syncthreads();
    __shared__ int timed_out;
    if (tid == 0) {
        timed_out = 0;
        bar_expect_tx(t.bar_tma, 2 * kImgBytes);
        bulk_g2s(t.opA, t.img, kImgBytes, t.bar_tma);
        bulk_g2s(t.opB, t.img + kImgBytes, kImgBytes, t.bar_tma);
        bool ok = bar_wait(t.bar_tma, t.ph_tma);
        fence_after();
        if (ok) {
            const uint32_t id_kmn = idesc_bf16(kDim, kDim, 0, 1);
            // R = A Xhi + A Xlo + Xhi (-B) + Xlo (-B)
            for (int ks = 0; ks < kDim / 16; ++ks) {
                mma(tmem, kview(t.opA, ks), mnview(t.op0, ks), id_kmn, ks > 0);
                mma(tmem, kview(t.opA, ks), mnview(t.op1, ks), id_kmn, 1);
            }
            for (int ks = 0; ks < kDim / 16; ++ks) {
                mma(tmem, kview(t.op0, ks), mnview(t.opB, ks), id_kmn, 1);
                mma(tmem, kview(t.op1, ks), mnview(t.opB, ks), id_kmn, 1);
            }
            commit(t.bar_mma);
        } else {
            timed_out = 1;
        }
    }
    t.ph_tma ^= 1;
    __syncthreads();
    if (timed_out) return false;
    // R: TMEM -> R hi / lo images (and Rf). Warp w reads lanes 32 (w % 4) ..,
    // columns 64 (w / 4) .. + 64.
    const int row = 32 * (warp & 3) + lane;
    const int cbase = 64 * (warp >> 2);
    const uint32_t tl = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
    if (!bar_wait(t.bar_mma, t.ph_mma)) timed_out = 1;
    t.ph_mma ^= 1;
    fence_after();
    __syncthreads();
    if (timed_out) return false;
    for (int half = 0; half < 2; ++half) {
        const int c0 = cbase + 32 * half;
        float v[32];
        tmem_ld32(tl + c0, v);
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            float h[8], l[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) split2(v[8 * g + k], h[k], l[k]);
            const uint4 qh = make_uint4(pack_bf16(h[0], h[1]), pack_bf16(h[2], h[3]), pack_bf16(h[4], h[5]),
                                        pack_bf16(h[6], h[7]));
            const uint4 ql = make_uint4(pack_bf16(l[0], l[1]), pack_bf16(l[2], l[3]), pack_bf16(l[4], l[5]),
                                        pack_bf16(l[6], l[7]));
            *reinterpret_cast<uint4*>(t.op0 + blk_off(row, c0 + 8 * g)) = qh;
            *reinterpret_cast<uint4*>(t.op1 + blk_off(row, c0 + 8 * g)) = ql;
        }
        if (Rf && row < m) {
#pragma unroll
            for (int k = 0; k < 32; ++k)
                if (c0 + k < m) Rf[row * m + c0 + k] = v[k];
        }
    }
    fence_before();
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
        fence_after();
        const uint32_t id_mnmn = idesc_bf16(kDim, kDim, 1, 1);
        const uint32_t id_kk = idesc_bf16(kDim, kDim, 0, 0);
        // G / 2s = A' Rhi + A' Rlo + Rhi (-B') + Rlo (-B')
        for (int ks = 0; ks < kDim / 16; ++ks) {
            mma(tmem, mnview(t.opA, ks), mnview(t.op0, ks), id_mnmn, ks > 0);
            mma(tmem, mnview(t.opA, ks), mnview(t.op1, ks), id_mnmn, 1);
        }
        for (int ks = 0; ks < kDim / 16; ++ks) {
            mma(tmem, kview(t.op0, ks), kview(t.opB, ks), id_kk, 1);
            mma(tmem, kview(t.op1, ks), kview(t.opB, ks), id_kk, 1);
        }
        commit(t.bar_mma);
    }
    if (!bar_wait(t.bar_mma, t.ph_mma)) timed_out = 1;
    t.ph_mma ^= 1;
    fence_after();
    __syncthreads();
    if (timed_out) return false;
    for (int half = 0; half < 2; ++half) {
        const int c0 = cbase + 32 * half;
        float v[32];
        tmem_ld32(tl + c0, v);
        if (row < m) {
#pragma unroll
            for (int k = 0; k < 32; ++k)
                if (c0 + k < m) gf[row * m + c0 + k] = two_s * v[k];
        }
    }
    fence_before();
    __syncthreads();
    return true;
}

}  // namespace tc
}  // namespace gbx
