// Shared helpers of the fasterlmm_gb300 CUDA library: status handling, argument checks, warp reductions and the
// FP64 atomic max used by the per-column genome max.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fasterlmm_gb300.h"

namespace flmm {

// Records a printf-style message as this thread's last error (read back by flmm_last_error) and returns `status`.
int fail(int status, const char* fmt, ...);

// Counts one kernel launch of this library and converts the pending CUDA error (if any) into FLMM_ERR_CUDA with
// the kernel's name.  Call once right after each <<<...>>> launch.
int check_launch(const char* what);

// Same error conversion without counting a launch (after library calls such as cuSOLVER).
int check_cuda(const char* what);

// Device int raised by kernels without a context (e.g. the refinement's tensor-core product) when a bounded wait
// gives up; one per device, allocated on first use, reported and cleared by flmm_context_check.  nullptr if the
// allocation failed.
int* device_err_flag(int device);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// The library's own batched FP32 eigensolver (csrc/flmm_eigh_own.cu): A (batch, N, N) symmetric in, one eigenvector
// per row out, evals (batch, N) ascending; work of eigh_own_workspace_bytes(N, batch) bytes.
size_t eigh_own_workspace_bytes(int N, int batch);
int eigh_own_f32(float* A, int N, int batch, float* evals, void* work, cudaStream_t st);

// The refinement's FP64-accurate product on the tensor cores (csrc/flmm_ozaki.cu): W (batch, N, N) = U~ A^T, U~ the
// digit-plane rounding of U (written to Ut); work of refine_product_tc_bytes(N, batch) bytes.
size_t refine_product_tc_bytes(int N, int batch);
int refine_product_tc(const float* U, const double* A, int N, int batch, float* Ut, double* W, void* work,
                      cudaStream_t st);
// The step's corrections on the same workspace, after refine_product_tc: M = U~ R^T, then U_out = U~ + T U~ with T
// (batch, N, N) FP32 stored at the start of the workspace and scratch an (batch, N, N) FP32 buffer.
int refine_m_tc(const float* R, int N, int batch, float* M, void* work, cudaStream_t st);
int refine_update_tc(const float* T, const float* Ut, float* scratch, int N, int batch, float* U_out, void* work,
                     cudaStream_t st);

inline unsigned ceil_div(int64_t a, int64_t b) { return static_cast<unsigned>((a + b - 1) / b); }

#define FLMM_REQUIRE(cond, ...)                                                       \
    do {                                                                              \
        if (!(cond)) return ::flmm::fail(FLMM_ERR_ARG, __VA_ARGS__);                  \
    } while (0)

#define FLMM_CUDA(call)                                                               \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess)                                                        \
            return ::flmm::fail(FLMM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Neumaier-compensated running sum: comp collects the rounding error of every addition, so sum + comp is the sum of
// the added terms without the accumulated FP32 rounding
__device__ __forceinline__ void neumaier(float& sum, float& comp, float x) {
    const float t = sum + x;
    comp += (fabsf(sum) >= fabsf(x)) ? ((sum - t) + x) : ((x - t) + sum);
    sum = t;
}

// exact sum and error of a + b (Knuth's TwoSum)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// warp-wide sum of a compensated pair (hi + lo), TwoSum at every level of the butterfly
__device__ __forceinline__ float warp_sum_pair(float hi, float lo) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, hi, o);
        const float ol = __shfl_xor_sync(0xffffffffu, lo, o);
        float sum, err;
        two_sum(hi, oh, sum, err);
        hi = sum;
        lo = lo + ol + err;
    }
    return hi + lo;
}

__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// max over non-negative (or NaN) doubles stored as their bit patterns: for x >= 0 the IEEE bit pattern read as a
// signed 64-bit integer is monotone in x, -inf (the initial value) reads negative, and NaN reads above +inf, so
// a NaN column statistic propagates as torch.maximum would.
__device__ __forceinline__ void atomic_max_nonneg(double* addr, double v) {
    atomicMax(reinterpret_cast<long long*>(addr), __double_as_longlong(v));
}

__device__ __forceinline__ void atomic_max_nonneg(float* addr, float v) {
    atomicMax(reinterpret_cast<int*>(addr), __float_as_int(v));
}

// FP64 helpers that are never contracted into an FMA, so an expression evaluates with the same roundings as the
// reference's separate tensor operations.
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

// Positive clamp floor of the FP64 path (fasterlmm/core.py:80-86).
constexpr double kPosFloor = 1e-300;

}  // namespace flmm
