// The split-FP16 operand format of the tensor-core products: a row of FP32 values x is stored as FP16 pairs
// x = (hi + lo) * 2^-e with one power-of-two exponent e per row, chosen so the row's largest |x| 2^e lies in
// [2^14, 2^15); |x - (hi + lo) 2^-e| <= 2^-22 |x| in the normal range.
#pragma once

#include <cuda_fp16.h>
#include <math.h>
#include <stdint.h>

namespace flmm {

// 2^e for a row whose largest magnitude is amax (e written to *e_out); rows of zeros keep e = 0
__device__ __forceinline__ float row_scale_exp(float amax, int* e_out) {
    int e = 0;
    if (amax > 0.0f && isfinite(amax)) {
        int ex;
        frexpf(amax, &ex);  // amax = m 2^ex, m in [0.5, 1)
        e = 15 - ex;
    }
    *e_out = e;
    return ldexpf(1.0f, e);
}

// hi / lo pair of x at the row's scale mul = 2^e, stored at offset o
__device__ __forceinline__ void split_store(float x, float mul, __half* hi, __half* lo, int64_t o) {
    const float xs = x * mul;  // exact: power-of-two scale
    const __half h = __float2half_rn(xs);
    hi[o] = h;
    lo[o] = __float2half_rn(xs - __half2float(h));
}

}  // namespace flmm
