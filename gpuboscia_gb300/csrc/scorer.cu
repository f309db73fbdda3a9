// scorer.cu -- the learned branching scorer: an MLP n_features -> H -> H -> 1
// (ReLU) trained on the GPU with a listwise softmax loss over the candidates
// of each node, and evaluated in BF16 or FP32 for branching.
//
// Kernels (one launch each, deterministic):
//   mlp_forward      one thread per candidate row, parameters staged in shared
//                    memory (BF16 weights widened to FP32, FP32 accumulation);
//   group_softmax    one warp per node group: dL/dz = softmax(z) - target and
//                    the group's loss;
//   mlp_backward     a tile of 64 rows per CTA: activations and deltas of the
//                    tile in shared memory, then every parameter's partial sum
//                    over the tile (fixed order) into a per-tile slot;
//   reduce_tiles     parameter-wise sum of the tile partials in tile order,
//                    and the loss sum in group order;
//   adam             the Adam update, then the BF16 copy.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>

#include "relax.cuh"
#include "scorer_mlp.cuh"

namespace gbx {
namespace {

using namespace mlp;
constexpr int kTile = 64;

template <int H>
__global__ void __launch_bounds__(128) mlp_forward(const float* P, const unsigned short* Pb, int rows,
                                                   const float* X, float* z) {
    extern __shared__ float w[];
    const int cnt = param_count(kF, H);
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) w[i] = Pb ? bf16_to_f(Pb[i]) : P[i];
    __syncthreads();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    float x[kF], a1[H], a2[H];
#pragma unroll
    for (int f = 0; f < kF; ++f) x[f] = X[(size_t)r * kF + f];
    z[r] = forward_row<H>(w, offsets(kF, H), x, a1, a2);
}

__global__ void group_softmax(int groups, const int* gp, const float* z, const float* target, float* dz,
                              float* gloss) {
    const int g = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (g >= groups) return;
    const int b = gp[g], e = gp[g + 1];
    float mx = -INFINITY;
    for (int r = b + lane; r < e; r += 32) mx = fmaxf(mx, z[r]);
    for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    float se = 0.f;
    for (int r = b + lane; r < e; r += 32) se += expf(z[r] - mx);
    for (int off = 16; off > 0; off >>= 1) se += __shfl_xor_sync(0xffffffffu, se, off);
    const float lse = mx + logf(se);
    float l = 0.f;
    for (int r = b + lane; r < e; r += 32) {
        const float p = expf(z[r] - lse);
        dz[r] = p - target[r];
        l -= target[r] * (z[r] - lse);
    }
    for (int off = 16; off > 0; off >>= 1) l += __shfl_xor_sync(0xffffffffu, l, off);
    if (lane == 0) gloss[g] = e > b ? l : 0.f;
}

// per tile: rows [t*kTile, +kTile) -> partial[t][cnt]
template <int H>
__global__ void __launch_bounds__(kTile) mlp_backward(const float* P, int rows, const float* X, const float* dz,
                                                      float* partial) {
    extern __shared__ float sm[];
    const int cnt = param_count(kF, H);
    const Off o = offsets(kF, H);
    float* w = sm;                       // [cnt]
    float* sx = w + cnt;                 // [kTile][kF]
    float* sh1 = sx + kTile * kF;        // relu(a1) [kTile][H]
    float* sd1 = sh1 + kTile * H;        // dL/da1
    float* sh2 = sd1 + kTile * H;        // relu(a2)
    float* sd2 = sh2 + kTile * H;        // dL/da2
    float* sdz = sd2 + kTile * H;        // [kTile]
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) w[i] = P[i];
    __syncthreads();
    const int t = threadIdx.x;
    const int r = blockIdx.x * kTile + t;
    float x[kF], a1[H], a2[H];
    if (r < rows) {
#pragma unroll
        for (int f = 0; f < kF; ++f) x[f] = X[(size_t)r * kF + f];
        forward_row<H>(w, o, x, a1, a2);
    } else {
#pragma unroll
        for (int f = 0; f < kF; ++f) x[f] = 0.f;
#pragma unroll
        for (int i = 0; i < H; ++i) { a1[i] = 0.f; a2[i] = 0.f; }
    }
    const float d = r < rows ? dz[r] : 0.f;
    sdz[t] = d;
#pragma unroll
    for (int f = 0; f < kF; ++f) sx[t * kF + f] = x[f];
    for (int i = 0; i < H; ++i) {
        const float d2 = a2[i] > 0.f ? d * w[o.w3 + i] : 0.f;
        sh2[t * H + i] = fmaxf(a2[i], 0.f);
        sd2[t * H + i] = d2;
        sh1[t * H + i] = fmaxf(a1[i], 0.f);
    }
    for (int j = 0; j < H; ++j) {
        float s = 0.f;
        for (int i = 0; i < H; ++i) s = fmaf(w[o.W2 + i * H + j], sd2[t * H + i], s);
        sd1[t * H + j] = a1[j] > 0.f ? s : 0.f;
    }
    __syncthreads();
    float* out = partial + (size_t)blockIdx.x * cnt;
    for (int p = threadIdx.x; p < cnt; p += blockDim.x) {
        float s = 0.f;
        if (p < o.b1) {                      // W1[i][f]
            const int i = p / kF, f = p - (p / kF) * kF;
            for (int q = 0; q < kTile; ++q) s = fmaf(sd1[q * H + i], sx[q * kF + f], s);
        } else if (p < o.W2) {               // b1[i]
            const int i = p - o.b1;
            for (int q = 0; q < kTile; ++q) s += sd1[q * H + i];
        } else if (p < o.b2) {               // W2[i][j]
            const int i = (p - o.W2) / H, j = (p - o.W2) - ((p - o.W2) / H) * H;
            for (int q = 0; q < kTile; ++q) s = fmaf(sd2[q * H + i], sh1[q * H + j], s);
        } else if (p < o.w3) {               // b2[i]
            const int i = p - o.b2;
            for (int q = 0; q < kTile; ++q) s += sd2[q * H + i];
        } else if (p < o.b3) {               // w3[i]
            const int i = p - o.w3;
            for (int q = 0; q < kTile; ++q) s = fmaf(sdz[q], sh2[q * H + i], s);
        } else {                             // b3
            for (int q = 0; q < kTile; ++q) s += sdz[q];
        }
        out[p] = s;
    }
}

__global__ void reduce_tiles(int cnt, int tiles, const float* partial, float* grad, int groups, const float* gloss,
                             float* loss) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < cnt) {
        float s = 0.f;
        for (int t = 0; t < tiles; ++t) s += partial[(size_t)t * cnt + p];
        grad[p] = s;
    }
    if (loss && blockIdx.x == 0 && threadIdx.x == 0) {
        float l = 0.f;
        for (int g = 0; g < groups; ++g) l += gloss[g];
        *loss = l;
    }
}

__global__ void adam(int cnt, float* P, unsigned short* Pb, const float* g, float* m, float* v, float lr,
                     float c1, float c2) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= cnt) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float mi = b1 * m[p] + (1.f - b1) * g[p];
    const float vi = b2 * v[p] + (1.f - b2) * g[p] * g[p];
    m[p] = mi;
    v[p] = vi;
    const float w = P[p] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    P[p] = w;
    if (Pb) Pb[p] = __bfloat16_as_ushort(__float2bfloat16_rn(w));
}

int check_scorer(const gbx_scorer* s, std::string* err) {
    if (!s || !s->params) { *err = "scorer: null descriptor or parameters"; return GBX_ERR_INVALID; }
    if (s->n_features != kF) { *err = "scorer: n_features must be GBX_SCORER_FEATURES"; return GBX_ERR_INVALID; }
    if (s->hidden != 16 && s->hidden != 32 && s->hidden != 64) {
        *err = "scorer: hidden must be 16, 32 or 64";
        return GBX_ERR_UNSUPPORTED;
    }
    return GBX_OK;
}

size_t tiles_of(int rows) { return (size_t)(rows + kTile - 1) / kTile; }

}  // namespace

int scorer_param_count(int F, int H) { return param_count(F, H); }

int scorer_forward(const gbx_scorer* s, int rows, const float* X, float* z, int bf16, cudaStream_t st,
                   std::string* err) {
    int rc = check_scorer(s, err);
    if (rc) return rc;
    if (bf16 && !s->params_bf16) { *err = "scorer: BF16 inference needs params_bf16"; return GBX_ERR_INVALID; }
    if (rows == 0) return GBX_OK;
    const int H = s->hidden;
    const size_t smem = (size_t)param_count(kF, H) * sizeof(float);
    const unsigned short* pb = bf16 ? s->params_bf16 : nullptr;
    const int blocks = (rows + 127) / 128;
    if (H == 16) mlp_forward<16><<<blocks, 128, smem, st>>>(s->params, pb, rows, X, z);
    else if (H == 32) mlp_forward<32><<<blocks, 128, smem, st>>>(s->params, pb, rows, X, z);
    else mlp_forward<64><<<blocks, 128, smem, st>>>(s->params, pb, rows, X, z);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    return GBX_OK;
}

size_t scorer_workspace_bytes(const gbx_scorer* s, int rows) {
    if (!s || rows < 0) return 0;
    const int cnt = param_count(kF, s->hidden);
    return align16((size_t)rows * 4) * 3 + align16(tiles_of(rows) * (size_t)cnt * 4) + 256;
}

int scorer_gradient(const gbx_scorer* s, int rows, const float* X, int groups, const int* gp, const float* target,
                    float* grad, float* loss, void* ws, size_t ws_bytes, cudaStream_t st, std::string* err) {
    int rc = check_scorer(s, err);
    if (rc) return rc;
    if (rows < 1 || groups < 1 || !X || !gp || !target || !grad) {
        *err = "scorer gradient: empty batch or null buffer";
        return GBX_ERR_INVALID;
    }
    if (!ws || ws_bytes < scorer_workspace_bytes(s, rows)) {
        *err = "scorer gradient: workspace smaller than gbx_scorer_workspace_bytes()";
        return GBX_ERR_WORKSPACE;
    }
    const int H = s->hidden, cnt = param_count(kF, H);
    const int tiles = (int)tiles_of(rows);
    unsigned char* p = static_cast<unsigned char*>(ws);
    float* z = reinterpret_cast<float*>(p);
    p += align16((size_t)rows * 4);
    float* dz = reinterpret_cast<float*>(p);
    p += align16((size_t)rows * 4);
    float* gl = reinterpret_cast<float*>(p);  // groups <= rows
    p += align16((size_t)rows * 4);
    float* partial = reinterpret_cast<float*>(p);
    if (groups > rows) { *err = "scorer gradient: more groups than rows"; return GBX_ERR_INVALID; }
    rc = scorer_forward(s, rows, X, z, 0, st, err);
    if (rc) return rc;
    group_softmax<<<(groups + 3) / 4, 128, 0, st>>>(groups, gp, z, target, dz, gl);
    const size_t smem = ((size_t)cnt + kTile * kF + 4 * (size_t)kTile * H + kTile) * sizeof(float);
    cudaError_t e = cudaSuccess;
    if (H == 16) {
        mlp_backward<16><<<tiles, kTile, smem, st>>>(s->params, rows, X, dz, partial);
    } else if (H == 32) {
        mlp_backward<32><<<tiles, kTile, smem, st>>>(s->params, rows, X, dz, partial);
    } else {
        e = cudaFuncSetAttribute(mlp_backward<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) mlp_backward<64><<<tiles, kTile, smem, st>>>(s->params, rows, X, dz, partial);
    }
    if (e == cudaSuccess) {
        reduce_tiles<<<(cnt + 255) / 256, 256, 0, st>>>(cnt, tiles, partial, grad, groups, gl, loss);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    return GBX_OK;
}

int scorer_adam(gbx_scorer* s, const float* g, float* m, float* v, int step, float lr, cudaStream_t st,
                std::string* err) {
    int rc = check_scorer(s, err);
    if (rc) return rc;
    if (!g || !m || !v || step < 1) { *err = "scorer adam: null buffer or step < 1"; return GBX_ERR_INVALID; }
    const int cnt = param_count(kF, s->hidden);
    const float c1 = 1.f - powf(0.9f, (float)step), c2 = 1.f - powf(0.999f, (float)step);
    adam<<<(cnt + 255) / 256, 256, 0, st>>>(cnt, s->params, s->params_bf16, g, m, v, lr, c1, c2);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return GBX_ERR_CUDA; }
    return GBX_OK;
}

}  // namespace gbx
