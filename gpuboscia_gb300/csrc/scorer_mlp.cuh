// scorer_mlp.cuh -- parameter layout and row evaluation of the learned
// branching scorer (an MLP GBX_SCORER_FEATURES -> H -> H -> 1 with ReLU),
// shared by the scorer kernels and the device frontier's branching.
#pragma once

#include <cstdint>

#include "../../include/gpuboscia_gb300.h"

namespace gbx {
namespace mlp {

constexpr int kF = GBX_SCORER_FEATURES;

__host__ __device__ inline int param_count(int F, int H) { return H * F + H + H * H + H + H + 1; }

// W1[H][F], b1[H], W2[H][H], b2[H], w3[H], b3
struct Off {
    int W1, b1, W2, b2, w3, b3;
};
__host__ __device__ inline Off offsets(int F, int H) {
    Off o;
    o.W1 = 0;
    o.b1 = H * F;
    o.W2 = o.b1 + H;
    o.b2 = o.W2 + H * H;
    o.w3 = o.b2 + H;
    o.b3 = o.w3 + H;
    return o;
}

__device__ inline float bf16_to_f(unsigned short v) { return __uint_as_float((uint32_t)v << 16); }

// z of one feature row; a1 / a2 receive the two hidden layers' pre-activations.
// FP32 with explicit fused multiply-adds in a fixed order.
template <int H>
__device__ inline float forward_row(const float* w, const Off& o, const float* x, float* a1, float* a2) {
#pragma unroll 4
    for (int i = 0; i < H; ++i) {
        float s = w[o.b1 + i];
#pragma unroll
        for (int f = 0; f < kF; ++f) s = fmaf(w[o.W1 + i * kF + f], x[f], s);
        a1[i] = s;
    }
    float z = w[o.b3];
#pragma unroll 4
    for (int i = 0; i < H; ++i) {
        float s = w[o.b2 + i];
        for (int j = 0; j < H; ++j) s = fmaf(w[o.W2 + i * H + j], fmaxf(a1[j], 0.f), s);
        a2[i] = s;
        z = fmaf(w[o.w3 + i], fmaxf(s, 0.f), z);
    }
    return z;
}

}  // namespace mlp
}  // namespace gbx
