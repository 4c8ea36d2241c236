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
//
// The per-phenotype setup that feeds those products (lux/src/fasterlmm_lux/epi/_kernel.py, the per-chunk block
// before the test-column loop) runs in FP64 in two kernels: k_epi_normal (one block per phenotype) forms
// A_p = X^T W_p X and u_p = X^T W_p y_p over row tiles staged in shared memory, factors A_p = L_p L_p^T in shared
// memory (packed lower triangle, column by column), solves for the covariate fit beta_x = A_p^-1 u_p, and writes
// w_p, the row w_p o r_p (r_p = y_p - X beta_x) and rWr = sum w r^2; k_epi_q (one thread per sample) solves
// L_p q = w_n x_n by forward substitution for every sample n, the columns of Q_p = L_p^-1 X^T W_p.  A pivot that
// is not positive (A_p not positive definite) sets *info, and that phenotype's outputs are NaN.
#include <math.h>
#include <stdint.h>

#include <algorithm>

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

constexpr int kSetupThreads = 256;
constexpr int kMaxEpiC = 200;
constexpr size_t kSetupSmemMax = 226 * 1024;  // the opt-in 227 KB less room for static shared memory

__device__ __forceinline__ int tri(int i) { return i * (i + 1) / 2; }

// One block per phenotype p of the chunk.  Shared memory: packed A (C (C + 1) / 2) | u (C) | X tile (T1 x C) |
// w tile (T1) | y tile (T1) | reduction (32).
__global__ void __launch_bounds__(kSetupThreads)
k_epi_normal(const double* __restrict__ s, int N, const double* __restrict__ X, int64_t ldx, int C,
             const double* __restrict__ Y, int64_t ldy, const double* __restrict__ log_delta, int T1,
             double* __restrict__ R1, double* __restrict__ W, double* __restrict__ rWr, double* __restrict__ Lout,
             int* __restrict__ info) {
    extern __shared__ double sm[];
    __shared__ int fail;
    const int CP = tri(C);
    double* Ap = sm;
    double* u = Ap + CP;
    double* Xs = u + C;
    double* ws = Xs + static_cast<int64_t>(T1) * C;
    double* ys = ws + T1;
    double* red = ys + T1;
    const int p = blockIdx.x;
    const int tid = threadIdx.x;
    const double delta = exp(log_delta[p]);
    for (int e = tid; e < CP + C; e += kSetupThreads) sm[e] = 0.0;
    if (tid == 0) fail = 0;
    __syncthreads();
    // A = sum_n w_n x_n x_n^T (lower triangle) and u = sum_n w_n x_n y_n, in sample order
    for (int n0 = 0; n0 < N; n0 += T1) {
        const int T = min(T1, N - n0);
        for (int e = tid; e < T * C; e += kSetupThreads) {
            const int t = e / C, c = e - t * C;
            Xs[e] = X[static_cast<int64_t>(n0 + t) * ldx + c];
        }
        for (int t = tid; t < T; t += kSetupThreads) {
            ws[t] = 1.0 / (s[n0 + t] + delta);
            ys[t] = Y[static_cast<int64_t>(n0 + t) * ldy + p];
        }
        __syncthreads();
        for (int e = tid; e < C * C + C; e += kSetupThreads) {
            if (e < C * C) {
                const int i = e / C, j = e - i * C;
                if (j > i) continue;
                double acc = Ap[tri(i) + j];
                for (int t = 0; t < T; ++t) acc = fma(ws[t] * Xs[t * C + i], Xs[t * C + j], acc);
                Ap[tri(i) + j] = acc;
            } else {
                const int i = e - C * C;
                double acc = u[i];
                for (int t = 0; t < T; ++t) acc = fma(ws[t] * Xs[t * C + i], ys[t], acc);
                u[i] = acc;
            }
        }
        __syncthreads();
    }
    // Cholesky factor in place, one column at a time: the pivot by warp 0, then the column below it
    for (int j = 0; j < C; ++j) {
        if (tid < 32) {
            double acc = 0.0;
            for (int k = tid; k < j; k += 32) acc = fma(Ap[tri(j) + k], Ap[tri(j) + k], acc);
            acc = warp_sum(acc);
            if (tid == 0) {
                const double d = Ap[tri(j) + j] - acc;
                if (!(d > 0.0)) fail = 1;
                Ap[tri(j) + j] = d > 0.0 ? sqrt(d) : NAN;
            }
        }
        __syncthreads();
        const double djj = Ap[tri(j) + j];
        for (int i = j + 1 + tid; i < C; i += kSetupThreads) {
            double acc = Ap[tri(i) + j];
            for (int k = 0; k < j; ++k) acc = fma(-Ap[tri(i) + k], Ap[tri(j) + k], acc);
            Ap[tri(i) + j] = acc / djj;
        }
        __syncthreads();
    }
    // beta_x = L^-T L^-1 u, column-oriented substitutions by warp 0 (u is overwritten by z, then by beta_x)
    if (tid < 32) {
        for (int i = 0; i < C; ++i) {
            const double zi = u[i] / Ap[tri(i) + i];
            __syncwarp();
            for (int k = i + 1 + tid; k < C; k += 32) u[k] = fma(-Ap[tri(k) + i], zi, u[k]);
            if (tid == 0) u[i] = zi;
            __syncwarp();
        }
        for (int i = C - 1; i >= 0; --i) {
            const double bi = u[i] / Ap[tri(i) + i];
            __syncwarp();
            for (int k = tid; k < i; k += 32) u[k] = fma(-Ap[tri(i) + k], bi, u[k]);
            if (tid == 0) u[i] = bi;
            __syncwarp();
        }
    }
    __syncthreads();
    // residual row w o r, the weights, and rWr
    double* R1p = R1 + static_cast<int64_t>(p) * (C + 1) * N;
    double acc = 0.0;
    for (int n = tid; n < N; n += kSetupThreads) {
        const double* xr = X + static_cast<int64_t>(n) * ldx;
        double fit = 0.0;
        for (int k = 0; k < C; ++k) fit = fma(xr[k], u[k], fit);
        const double w = 1.0 / (s[n] + delta);
        const double r = Y[static_cast<int64_t>(n) * ldy + p] - fit;
        W[static_cast<int64_t>(p) * N + n] = w;
        R1p[static_cast<int64_t>(C) * N + n] = w * r;
        acc = fma(w * r, r, acc);
    }
    acc = warp_sum(acc);
    if ((tid & 31) == 0) red[tid >> 5] = acc;
    for (int e = tid; e < CP; e += kSetupThreads) Lout[static_cast<int64_t>(p) * CP + e] = Ap[e];
    __syncthreads();
    if (tid == 0) {
        double tot = 0.0;
        for (int w = 0; w < kSetupThreads / 32; ++w) tot += red[w];
        rWr[p] = fmax(tot, 1e-300);
        if (fail) *info = 1;
    }
}

// Grid (ceil(N / T2), Pc), T2 threads, one sample each: q = L_p^-1 (w_n x_n) into rows 0..C-1 of phenotype p's
// block of R1.  Shared memory: packed L_p | q (C x T2, one column per thread).
__global__ void __launch_bounds__(128)
k_epi_q(const double* __restrict__ X, int64_t ldx, int C, int N, const double* __restrict__ L,
        const double* __restrict__ W, double* __restrict__ R1) {
    extern __shared__ double sm[];
    const int CP = tri(C);
    const int T2 = blockDim.x;
    double* Ls = sm;
    double* qs = sm + CP;
    const int p = blockIdx.y;
    for (int e = threadIdx.x; e < CP; e += T2) Ls[e] = L[static_cast<int64_t>(p) * CP + e];
    __syncthreads();
    const int t = threadIdx.x;
    const int n = blockIdx.x * T2 + t;
    if (n >= N) return;
    const double w = W[static_cast<int64_t>(p) * N + n];
    const double* xr = X + static_cast<int64_t>(n) * ldx;
    double* out = R1 + static_cast<int64_t>(p) * (C + 1) * N + n;
    for (int i = 0; i < C; ++i) {
        const double* li = Ls + tri(i);
        double acc = w * xr[i];
        for (int k = 0; k < i; ++k) acc = fma(-li[k], qs[k * T2 + t], acc);
        const double q = acc / li[i];
        qs[i * T2 + t] = q;
        out[static_cast<int64_t>(i) * N] = q;
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

extern "C" int flmm_epi_setup_f64(const double* s, int N, const double* X, int64_t ldx, int C, const double* Y,
                                  int64_t ldy, const double* log_delta, int Pc, double* R1, double* W, double* rWr,
                                  double* L, int* info, void* stream) {
    FLMM_REQUIRE(N >= 1 && C >= 1 && C <= kMaxEpiC && Pc >= 0 && Pc <= 65535 && ldx >= C && ldy >= Pc,
                 "flmm_epi_setup_f64: bad sizes (1 <= C <= 200, Pc <= 65535)");
    if (Pc == 0) return FLMM_OK;
    FLMM_REQUIRE(s && X && Y && log_delta && R1 && W && rWr && L && info, "flmm_epi_setup_f64: null pointer");
    cudaStream_t st = as_stream(stream);
    const size_t CP = static_cast<size_t>(C) * (C + 1) / 2;
    const size_t fixed = 8 * (CP + C + 32);
    const int T1 = static_cast<int>(std::min<size_t>(32, (kSetupSmemMax - fixed) / (8 * (C + 2))));
    const size_t smem1 = fixed + 8 * static_cast<size_t>(T1) * (C + 2);
    int T2 = 128;
    while (T2 > 32 && 8 * (CP + static_cast<size_t>(C) * T2) > kSetupSmemMax) T2 >>= 1;
    const size_t smem2 = 8 * (CP + static_cast<size_t>(C) * T2);
    // (function attributes are per device, so they are set on every call, to the same bound whatever the call's
    // sizes so that calls from other host threads never lower it under a launch; the call is cheap)
    FLMM_CUDA(cudaFuncSetAttribute(k_epi_normal, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(kSetupSmemMax)));
    FLMM_CUDA(cudaFuncSetAttribute(k_epi_q, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(kSetupSmemMax)));
    k_epi_normal<<<Pc, kSetupThreads, smem1, st>>>(s, N, X, ldx, C, Y, ldy, log_delta, T1, R1, W, rWr, L, info);
    int rc = check_launch("k_epi_normal");
    if (rc) return rc;
    k_epi_q<<<dim3((N + T2 - 1) / T2, Pc), T2, smem2, st>>>(X, ldx, C, N, L, W, R1);
    return check_launch("k_epi_q");
}
