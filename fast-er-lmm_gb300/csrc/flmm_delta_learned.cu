// Learned delta proposal for the fast delta fit (no counterpart in the reference, which searches a grid).
//
// A small MLP maps cheap per-column features of the rotated phenotype to log delta:
//   f_b = log(e_b / E + 1e-12), e_b = sum of UY^2 over the b-th of 32 equal-count bins of the ascending spectrum,
//   g_b = log(mean of s over bin b + 1e-4)   (the spectrum's shape, shared by all columns of a chromosome),
//   log(Neff) / 10,
// 65 inputs -> 128 -> 128 -> 1 with tanh-GELU.  The proposal only chooses where the exact refinement starts: it
// must fall inside the basin of the FP32 grid argmin ([grid[i-1], grid[i+1]], the reference's golden-section
// bracket), the sign of d loss / d log delta at the proposal picks the half of the basin that holds the stationary
// point, one more evaluation at that half's end confirms the sign change, and the fast fit's safeguarded Newton
// iteration runs in that half, starting from the proposal.  Otherwise the column takes the grid path unchanged.
// Either way the answer is the exact stationary point of the same loss, so the proposal changes speed, not results.
#include <math.h>

#include "flmm_common.cuh"
#include "flmm_delta_eval.cuh"

using namespace flmm;
using namespace flmm::dfit;

namespace {

constexpr int kBins = 32;
constexpr int kIn = 2 * kBins + 1;
constexpr int kHid = 128;

__device__ __forceinline__ float gelu_tanh(float x) {
    return 0.5f * x * (1.0f + tanhf(0.7978845608028654f * (x + 0.044715f * x * x * x)));
}

// Features of one column per warp: feats[p, b] = f_b, feats[p, 32 + b] = g_b, feats[p, 64] = log(Neff) / 10.
__global__ void k_delta_features(const double* __restrict__ s, int Neff, const float* __restrict__ UYt, int64_t ldu,
                                 int P, float* __restrict__ feats) {
    const int lane = threadIdx.x & 31;
    const int64_t p = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    if (p >= P) return;
    const float* u = UYt + p * ldu;
    // bin `lane` covers eigen-indices [lane Neff / 32, (lane + 1) Neff / 32)
    const int n0 = static_cast<int>((static_cast<int64_t>(lane) * Neff) / kBins);
    const int n1 = static_cast<int>((static_cast<int64_t>(lane + 1) * Neff) / kBins);
    float e = 0.0f, sm = 0.0f;
    for (int n = n0; n < n1; ++n) {
        e += u[n] * u[n];
        sm += static_cast<float>(s[n]);
    }
    const float E = warp_sum(e);
    float* f = feats + p * kIn;
    f[lane] = logf((E > 0.0f ? e / E : 0.0f) + 1e-12f);
    f[kBins + lane] = logf((n1 > n0 ? sm / static_cast<float>(n1 - n0) : 0.0f) + 1e-4f);
    if (lane == 0) f[2 * kBins] = logf(static_cast<float>(Neff)) * 0.1f;
}

// The MLP, one warp per column: lane j holds hidden units j, j + 32, j + 64, j + 96; x = clamp(out, lo, hi).
__global__ void k_delta_mlp(const float* __restrict__ feats, int P, const float* __restrict__ W1,
                            const float* __restrict__ b1, const float* __restrict__ W2, const float* __restrict__ b2,
                            const float* __restrict__ w3, float b3, double lo, double hi, double* __restrict__ x_out) {
    const int lane = threadIdx.x & 31;
    const int64_t p = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    if (p >= P) return;
    const float* f = feats + p * kIn;
    const float fb = f[lane], gb = f[kBins + lane], lgn = f[2 * kBins];
    float h1[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) h1[k] = b1[lane + 32 * k];
    for (int b = 0; b < kBins; ++b) {
        const float xf = __shfl_sync(0xffffffffu, fb, b);
        const float xg = __shfl_sync(0xffffffffu, gb, b);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float* w = W1 + (lane + 32 * k) * kIn;
            h1[k] = fmaf(w[b], xf, h1[k]);
            h1[k] = fmaf(w[kBins + b], xg, h1[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) h1[k] = gelu_tanh(fmaf(W1[(lane + 32 * k) * kIn + 2 * kBins], lgn, h1[k]));
    float h2[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) h2[k] = b2[lane + 32 * k];
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
        for (int src = 0; src < 32; ++src) {
            const float x = __shfl_sync(0xffffffffu, h1[kk], src);
            const int i = src + 32 * kk;
#pragma unroll
            for (int k = 0; k < 4; ++k) h2[k] = fmaf(W2[(lane + 32 * k) * kHid + i], x, h2[k]);
        }
    }
    float o = 0.0f;
#pragma unroll
    for (int k = 0; k < 4; ++k) o = fmaf(w3[lane + 32 * k], gelu_tanh(h2[k]), o);
    o = warp_sum(o) + b3;
    if (lane == 0) x_out[p] = fmin(fmax(static_cast<double>(o), lo), hi);
}

// Exact refinement from the proposal, with the grid path as fallback (see the file comment).
__global__ void k_newton_from_proposal(const double* __restrict__ s, int Neff, const float* __restrict__ UYt,
                                       int64_t ldu, int P, const double* __restrict__ grid, int G,
                                       const int32_t* __restrict__ idx, const double* __restrict__ x_prop,
                                       double* __restrict__ log_delta, int32_t* __restrict__ n_fallback) {
    extern __shared__ float sm[];
    float* s32 = sm;
    float* dsb = sm + Neff;
    __shared__ float sbar_s;
    const float sbar = load_spectrum(s, Neff, s32, dsb, &sbar_s);
    const int lane = threadIdx.x & 31;
    const int64_t p = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    if (p >= P) return;
    const float* u = UYt + p * ldu;
    float uh = 0.f, uc = 0.f;
    for (int n = lane; n < Neff; n += 32) neumaier(uh, uc, u[n] * u[n]);
    const GlobalColumn ev{s32, dsb, u, Neff, sbar, warp_sum_pair(uh, uc)};
    const int i = idx[p];
    const double a = grid[max(i - 1, 0)], b = grid[min(i + 1, G - 1)];
    const double x0 = x_prop[p];
    double out = 0.0;
    bool done = false;
    if (i > 0 && i < G - 1 && x0 > a && x0 < b) {
        // the proposal splits the grid argmin's basin: the half towards -g must end with the opposite sign
        const NewtonEval e0 = ev(x0, false);
        if (e0.g == 0.0f) {
            out = x0;
            done = true;
        } else {
            const double xe = e0.g < 0.0f ? b : a;
            const NewtonEval ee = ev(xe, false);
            if ((e0.g < 0.0f && ee.g > 0.0f) || (e0.g > 0.0f && ee.g < 0.0f)) {
                const double blo = e0.g < 0.0f ? x0 : xe, bhi = e0.g < 0.0f ? xe : x0;
                out = newton_in_bracket(ev, blo, bhi, x0, &e0);
                done = true;
            }
        }
    }
    if (!done) {
        out = refine_column(ev, grid, G, i, 1);
        if (lane == 0) atomicAdd(n_fallback, 1);
    }
    if (lane == 0) log_delta[p] = out;
}

}  // namespace

extern "C" int flmm_delta_features_f32(const double* s, int Neff, const float* UYt, int64_t ldu, int P, float* feats,
                                       void* stream) {
    FLMM_REQUIRE(s && UYt && feats && Neff >= kBins && ldu >= Neff && P >= 0,
                 "flmm_delta_features_f32: bad arguments (Neff must be >= 32)");
    if (P == 0) return FLMM_OK;
    k_delta_features<<<ceil_div(static_cast<int64_t>(P) * 32, 256), 256, 0, as_stream(stream)>>>(s, Neff, UYt, ldu,
                                                                                                 P, feats);
    return check_launch("k_delta_features");
}

extern "C" int flmm_delta_mlp_f32(const float* feats, int P, const float* W1, const float* b1, const float* W2,
                                  const float* b2, const float* w3, float b3, double lo, double hi, double* x_out,
                                  void* stream) {
    FLMM_REQUIRE(feats && W1 && b1 && W2 && b2 && w3 && x_out && P >= 0, "flmm_delta_mlp_f32: bad arguments");
    if (P == 0) return FLMM_OK;
    k_delta_mlp<<<ceil_div(static_cast<int64_t>(P) * 32, 256), 256, 0, as_stream(stream)>>>(feats, P, W1, b1, W2, b2,
                                                                                            w3, b3, lo, hi, x_out);
    return check_launch("k_delta_mlp");
}

extern "C" int flmm_newton_from_proposal(const double* s, int Neff, const float* UYt, int64_t ldu, int P,
                                         const double* grid, int n_grid, const int32_t* grid_idx,
                                         const double* x_prop, double* log_delta, int32_t* n_fallback, void* stream) {
    FLMM_REQUIRE(s && UYt && grid && grid_idx && x_prop && log_delta && n_fallback && Neff > 0 && n_grid > 0 &&
                     ldu >= Neff && P >= 0,
                 "flmm_newton_from_proposal: bad arguments");
    FLMM_REQUIRE(Neff <= 12288, "flmm_newton_from_proposal: Neff must be <= 12288 (shared-memory spectrum)");
    if (P == 0) return FLMM_OK;
    const size_t smem = 2 * sizeof(float) * static_cast<size_t>(Neff);
    if (smem > 48 * 1024)
        FLMM_CUDA(cudaFuncSetAttribute(k_newton_from_proposal, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem)));
    k_newton_from_proposal<<<ceil_div(static_cast<int64_t>(P) * 32, 256), 256, smem, as_stream(stream)>>>(
        s, Neff, UYt, ldu, P, grid, n_grid, grid_idx, x_prop, log_delta, n_fallback);
    return check_launch("k_newton_from_proposal");
}
