// Batched epistasis Wald (LUX tier 2, lux/src/fasterlmm_lux/epi/_kernel.py:21-150): the per-test statistics from
// the two products the scan forms on the tensor cores.
//
// For one anchor and a chunk of Pc phenotypes the row operand stacks, per phenotype p, the C rows of
// Q_p = L_p^-1 X^T W_p (L_p the Cholesky factor of A_p = X^T W_p X) and the row (w_p o r_p); multiplied by the test
// columns S (N, Mc) they give G1 (Pc (C + 1), Mc): quad = B^T A^-1 B = ||Q_p s_m||^2 is the sum of squares of a
// phenotype's C rows, num = (w o r)^T s_m its last row.  G2 (Pc, Mc) = W (S o S) holds sWs.  Per test:
//     denom = max(sWs - quad, 1e-300), beta = num / denom, rss = max(rWr - num^2 / denom, 1e-300),
//     var_beta = rss / (N - C - 1) / denom, se = sqrt(var_beta), F = beta^2 / var_beta,
// and F = 0 where sWs - quad < floor_rel sWs (the near-self pair guard).  The sum of squares runs in FP32 (the
// products are FP32), the rest in FP64.  One block per phenotype: it also forms the chunk's maximum F and the first
// column reaching it, and merges them into the running maximum the way the reference does (a chunk replaces it
// only when strictly greater; a chunk whose maximum is NaN never does).
#include <math.h>
#include <stdint.h>

#include "flmm_common.cuh"

using namespace flmm;

namespace {

constexpr int kEpiThreads = 256;

__global__ void __launch_bounds__(kEpiThreads)
k_epi_wald(const float* __restrict__ G1, int64_t ldg1, const float* __restrict__ G2, int64_t ldg2,
           const double* __restrict__ rWr, int C, int Mc, int m0, int p0, int n_real, double var_df,
           double floor_rel, double* __restrict__ beta_o, double* __restrict__ se_o, double* __restrict__ f_o,
           int64_t ldo, double* __restrict__ max_f, int64_t* __restrict__ argmax) {
    __shared__ double red_v[kEpiThreads / 32];
    __shared__ int red_m[kEpiThreads / 32];
    __shared__ int red_nan[kEpiThreads / 32];
    const int p = blockIdx.x;  // phenotype within the chunk
    const int gp = p0 + p;
    const bool real = gp < n_real;
    const double rwr = rWr[p];
    const float* g = G1 + static_cast<int64_t>(p) * (C + 1) * ldg1;
    double best = -INFINITY;
    int best_m = 0x7fffffff;
    int saw_nan = 0;
    for (int m = threadIdx.x; m < Mc; m += kEpiThreads) {
        float q = 0.0f;
        for (int c = 0; c < C; ++c) {
            const float v = g[static_cast<int64_t>(c) * ldg1 + m];
            q = fmaf(v, v, q);
        }
        const double num = g[static_cast<int64_t>(C) * ldg1 + m];
        const double sws = G2[static_cast<int64_t>(p) * ldg2 + m];
        const double denom_raw = sws - static_cast<double>(q);
        const double denom = fmax(denom_raw, 1e-300);
        const double beta = num / denom;
        const double rss = fmax(rwr - num * num / denom, 1e-300);
        const double var_beta = rss / var_df / denom;
        double F = beta * beta / var_beta;
        if (floor_rel > 0.0 && denom_raw < floor_rel * sws) F = 0.0;
        if (real) {
            const int64_t o = static_cast<int64_t>(m0 + m) * ldo + gp;
            beta_o[o] = beta;
            se_o[o] = sqrt(var_beta);
            f_o[o] = F;
        }
        if (F != F) saw_nan = 1;
        else if (F > best) { best = F; best_m = m; }
    }
    // block maximum, first column on ties
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double v = __shfl_xor_sync(0xffffffffu, best, o);
        const int mm = __shfl_xor_sync(0xffffffffu, best_m, o);
        if (v > best || (v == best && mm < best_m)) { best = v; best_m = mm; }
        saw_nan |= __shfl_xor_sync(0xffffffffu, saw_nan, o);
    }
    if (lane == 0) {
        red_v[warp] = best;
        red_m[warp] = best_m;
        red_nan[warp] = saw_nan;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = -INFINITY;
        int bm = 0x7fffffff, nan = 0;
        for (int w = 0; w < kEpiThreads / 32; ++w) {
            nan |= red_nan[w];
            if (red_v[w] > b || (red_v[w] == b && red_m[w] < bm)) { b = red_v[w]; bm = red_m[w]; }
        }
        // the reference's chunk maximum is NaN when any F of the chunk is; NaN never replaces the running value
        if (!nan && bm != 0x7fffffff && b > max_f[gp]) {
            max_f[gp] = b;
            argmax[gp] = m0 + bm;
        }
    }
}

}  // namespace

extern "C" int flmm_epi_wald_f32(const float* G1, int64_t ldg1, const float* G2, int64_t ldg2, const double* rWr,
                                 int Pc, int C, int Mc, int m0, int p0, int n_real, double var_df, double floor_rel,
                                 double* beta, double* se, double* F, int64_t ldo, double* max_f, int64_t* argmax,
                                 void* stream) {
    FLMM_REQUIRE(Pc >= 0 && C >= 1 && Mc >= 0 && m0 >= 0 && p0 >= 0 && n_real >= 0 && var_df > 0,
                 "flmm_epi_wald_f32: bad sizes");
    if (Pc == 0 || Mc == 0) return FLMM_OK;
    FLMM_REQUIRE(G1 && G2 && rWr && max_f && argmax && ldg1 >= Mc && ldg2 >= Mc, "flmm_epi_wald_f32: bad arguments");
    FLMM_REQUIRE(p0 >= n_real || (beta && se && F && ldo >= n_real), "flmm_epi_wald_f32: real-column outputs missing");
    k_epi_wald<<<Pc, kEpiThreads, 0, as_stream(stream)>>>(G1, ldg1, G2, ldg2, rWr, C, Mc, m0, p0, n_real, var_df,
                                                          floor_rel, beta, se, F, ldo, max_f, argmax);
    return check_launch("k_epi_wald");
}
