// The learned delta proposal's MLP (65 -> 128 -> 128 -> 1, tanh-GELU) on tiles of rows: shared by the training
// kernels (flmm_mlp_train.cu) and the inference kernel of the learned fit (flmm_delta_learned.cu).
//
// A CTA of kMlpThreads threads (thread j = hidden unit j) holds W1 (128 x 65) and W2 (128 x 128, rows padded to
// kLdW2 so that column reads by consecutive threads are conflict-free) in shared memory and runs kMlpRows rows at a
// time; per row the products accumulate in FP32 registers.
#pragma once

#include <cuda_bf16.h>
#include <math.h>

#include "flmm_common.cuh"

namespace flmm {
namespace mlp {

constexpr int kIn = 65, kHid = 128, kMlpRows = 16, kMlpThreads = 128;
constexpr int kLdW2 = kHid + 1;

__device__ __forceinline__ float round_bf16(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

constexpr float kGeluC = 0.7978845608028654f;  // sqrt(2 / pi)
constexpr float kGeluA = 0.044715f;

__device__ __forceinline__ float gelu_tanh(float x) {
    return 0.5f * x * (1.0f + tanhf(kGeluC * (x + kGeluA * x * x * x)));
}

__device__ __forceinline__ float gelu_tanh_grad(float x) {
    const float t = tanhf(kGeluC * (x + kGeluA * x * x * x));
    return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * kGeluC * (1.0f + 3.0f * kGeluA * x * x);
}

// W1s (kHid, kIn) and W2s (kHid, kLdW2) from row-major W1 (128, 65), W2 (128, 128); op rounds the operands (or not)
template <class Op>
__device__ __forceinline__ void load_weights(const float* __restrict__ W1, const float* __restrict__ W2, float* W1s,
                                             float* W2s, Op op) {
    for (int t = threadIdx.x; t < kHid * kIn; t += kMlpThreads) W1s[t] = op(W1[t]);
    for (int t = threadIdx.x; t < kHid * kHid; t += kMlpThreads) W2s[(t / kHid) * kLdW2 + t % kHid] = op(W2[t]);
}

// Forward pass of the tile's rows xs (kMlpRows, kIn) for unit j = threadIdx.x: pre-activations z1, z2 of unit j,
// a2 = op(gelu(z2)), and a1s (kMlpRows, kHid) = op(gelu(z1)) in shared memory.  Ends with a1s complete (one
// __syncthreads inside); the caller reduces w3 . a2 over the units.
template <class Op>
__device__ __forceinline__ void forward_tile(const float* W1s, const float* W2s, const float* xs, float* a1s, float b1j,
                                             float b2j, float (&z1)[kMlpRows], float (&z2)[kMlpRows],
                                             float (&a2)[kMlpRows], Op op) {
    const int j = threadIdx.x;
#pragma unroll
    for (int r = 0; r < kMlpRows; ++r) z1[r] = b1j;
    for (int k = 0; k < kIn; ++k) {
        const float w = W1s[j * kIn + k];
#pragma unroll
        for (int r = 0; r < kMlpRows; ++r) z1[r] = fmaf(w, xs[r * kIn + k], z1[r]);
    }
#pragma unroll
    for (int r = 0; r < kMlpRows; ++r) a1s[r * kHid + j] = op(gelu_tanh(z1[r]));
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kMlpRows; ++r) z2[r] = b2j;
    for (int i = 0; i < kHid; ++i) {
        const float w = W2s[j * kLdW2 + i];
#pragma unroll
        for (int r = 0; r < kMlpRows; ++r) z2[r] = fmaf(w, a1s[r * kHid + i], z2[r]);
    }
#pragma unroll
    for (int r = 0; r < kMlpRows; ++r) a2[r] = op(gelu_tanh(z2[r]));
}

// Per-row outputs w3 . a2 into red (4, kMlpRows): one partial per warp, added in a fixed order by the caller.
__device__ __forceinline__ void output_partials(float w3j, const float (&a2)[kMlpRows], float* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int r = 0; r < kMlpRows; ++r) {
        const float v = warp_sum(w3j * a2[r]);
        if (lane == 0) red[warp * kMlpRows + r] = v;
    }
}

__device__ __forceinline__ float row_output(const float* red, int r, float b3) {
    return ((red[r] + red[kMlpRows + r]) + (red[2 * kMlpRows + r] + red[3 * kMlpRows + r])) + b3;
}

}  // namespace mlp
}  // namespace flmm
