// Split-precision form of the low-rank Wald scan (fasterlmm/lowrank.py:239-316): the operand preparation that lets
// the fused tensor-core Wald kernel (csrc/flmm_fast.cu) run it.
//
// In the low-rank basis (k eigenvectors U_eff of a rank-k kinship, eigenvalues s) every quadratic form has an
// on-rank part weighted by 1 / (s + delta) and an off-rank part weighted by 1 / delta, carried by the explicit
// residuals UUY = Y_r - U_eff UY and UUS = S_r - U_eff US as in the reference (lowrank.py:110, 289).  With the
// normalised weights w~_i = (shat + delta) / (s_i + delta) and c = (shat + delta) / delta (shat = mean s; F, beta
// and SE do not change when all weights are scaled together):
//
//     sWy = sum_i w~_i UY_i US_i + c sum_n UUY_n UUS_n      (one product over K = k + N)
//     sWs = sum_i w~_i US_i^2   + c ||UUS||^2               (a function of delta per variant: interpolated)
//     rWr = sum_i w~_i UY_i^2   + c ||UUY||^2.
//
// So sWy is the fused kernel's first product with the column row [w~ o UY | c UUY] and the variant row
// [US | UUS], and sWs its interpolated second product over [US^2 | ||UUS||^2] with node weights [w~(x_r) | c(x_r)].
// Forming the residuals first keeps the off-rank sums free of cancellation: where the kinship spans almost every
// direction both residuals are small and so is their product's error.  The F test's degrees of freedom are
// N - D - 1 (lowrank.py:270), not the product depth.
#include <math.h>

#include "flmm_common.cuh"
#include "flmm_split.cuh"

using namespace flmm;

namespace {

constexpr int kInterpPoints = 10;  // the Wald kernel's Lagrange stencil (csrc/flmm_fast.cu)
constexpr int kCols = 8;           // columns (warps) per block of the column preparation

// R (rows, ldr) FP64 = Y - C for Y (rows, ldy) FP64 and the FP32 product C (rows, ldc), and the row sums of squares
// of R into ss (rows,): one warp per row.  UUY = Y_r - U_eff UY.
__global__ void k_lr_residual(const double* __restrict__ Y, int64_t ldy, const float* __restrict__ Cm, int64_t ldc,
                              int rows, int N, double* __restrict__ R, int64_t ldr, double* __restrict__ ss) {
    const int lane = threadIdx.x & 31;
    const int64_t r = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    if (r >= rows) return;
    double acc = 0.0;
#pragma unroll 4
    for (int n = lane; n < N; n += 32) {
        const double v = Y[r * ldy + n] - static_cast<double>(Cm[r * ldc + n]);
        R[r * ldr + n] = v;
        acc = fma(v, v, acc);
    }
    acc = warp_sum(acc);
    if (lane == 0) ss[r] = acc;
}

// One warp per column p: A1 row = [w~ o UY | c UUY] split with one scale, the column's Lagrange weights over the R
// sWs nodes split, rWr = sum w~ UY^2 + c ||UUY||^2 and rWr0 = rWr / (shat + delta).
__global__ void __launch_bounds__(32 * kCols)
k_lr_prep_columns(const float* __restrict__ s32, int k, const float* __restrict__ UYt, int64_t ldu,
                  const double* __restrict__ UUYt, int64_t ldy, int N, const double* __restrict__ yy_off,
                  const double* __restrict__ ld, int P, const float* __restrict__ shat_p, double x0, double h,
                  double inv_h, int R, __half* __restrict__ A1h, __half* __restrict__ A1l, int64_t lda,
                  __half* __restrict__ Lh, __half* __restrict__ Ll, int64_t ldl, float* __restrict__ sa1,
                  float* __restrict__ sl, float* __restrict__ rWr, float* __restrict__ rWr0) {
    __shared__ float lw[kCols][kInterpPoints];
    __shared__ int lbase[kCols];
    const int64_t p0 = static_cast<int64_t>(blockIdx.x) * kCols;
    if (threadIdx.x < kCols * kInterpPoints) {  // Lagrange weights on nodes base .. base + 9 around x
        const int j = threadIdx.x / kInterpPoints, q = threadIdx.x % kInterpPoints;
        const int64_t p = p0 + j;
        if (p < P) {
            const double x = ld[p];
            int base = static_cast<int>(floor((x - x0) * inv_h)) - (kInterpPoints / 2 - 1);
            base = max(0, min(base, R - kInterpPoints));
            const double t = (x - (x0 + base * h)) * inv_h;
            double num = 1.0, den = 1.0;
#pragma unroll
            for (int m = 0; m < kInterpPoints; ++m) {
                if (m == q) continue;
                num *= t - m;
                den *= static_cast<double>(q - m);
            }
            lw[j][q] = static_cast<float>(num / den);
            if (q == 0) lbase[j] = base;
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, j = threadIdx.x >> 5;
    const int64_t p = p0 + j;
    if (p >= P) return;
    const double x = ld[p];
    const double delta = exp(x);
    const float shat = *shat_p;
    const float num = static_cast<float>(static_cast<double>(shat) + delta);
    const float c = static_cast<float>((static_cast<double>(shat) + delta) / delta);
    const float deltaf = static_cast<float>(delta);
    const float* u = UYt + p * ldu;
    const double* y = UUYt + p * ldy;
    // pass 1: the row's largest magnitude and the on-rank part of rWr
    float m1 = 0.0f, acc = 0.0f, comp = 0.0f;
    for (int i = lane; i < k; i += 32) {
        const float wt = num / (s32[i] + deltaf);
        const float ui = u[i];
        m1 = fmaxf(m1, fabsf(wt * ui));
        neumaier(acc, comp, wt * ui * ui);
    }
    float my = 0.0f;
#pragma unroll 4
    for (int n = lane; n < N; n += 32) my = fmaxf(my, fabsf(static_cast<float>(y[n])));
    m1 = fmaxf(m1, c * my);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, o));
    const float on_rank = warp_sum_pair(acc, comp);
    int e1;
    const float mul1 = row_scale_exp(m1, &e1);
    // pass 2: the split row
    for (int i = lane; i < k; i += 32) {
        const float wt = num / (s32[i] + deltaf);
        split_store(wt * u[i], mul1, A1h, A1l, p * lda + i);
    }
#pragma unroll 4
    for (int n = lane; n < N; n += 32) split_store(c * static_cast<float>(y[n]), mul1, A1h, A1l, p * lda + k + n);
    const int base = lbase[j];
    float lm = 0.0f;
#pragma unroll
    for (int q = 0; q < kInterpPoints; ++q) lm = fmaxf(lm, fabsf(lw[j][q]));
    int el;
    const float mull = row_scale_exp(lm, &el);
    for (int r = lane; r < R; r += 32) {
        const int q = r - base;
        const float v = (q >= 0 && q < kInterpPoints) ? lw[j][q] : 0.0f;
        split_store(v, mull, Lh, Ll, p * ldl + r);
    }
    if (lane == 0) {
        const double rwr = static_cast<double>(on_rank) + static_cast<double>(c) * fmax(yy_off[p], 0.0);
        sa1[p] = ldexpf(1.0f, -e1);
        sl[p] = ldexpf(1.0f, -el);
        rWr[p] = static_cast<float>(fmax(rwr, 0.0));
        rWr0[p] = static_cast<float>(fmax(rwr, 0.0) / static_cast<double>(num));
    }
}

// One warp per variant m: the off-rank residual UUS = S_r - U_eff US, S_r = S - sum_d q_d (q_d . s) for the
// orthonormal covariate basis rows q_d (Qt, D x N) and the FP32 product Ct = U_eff US (Mc, ldc); then
// B1 row = [US | UUS] split with one scale and B2 row = [US^2 | ||UUS||^2] split with its own.  The residual is formed
// in FP32 from the FP64 standardised variant (each element O(1), so FP32 keeps it to ~1e-7 absolute).
constexpr int kMaxD = 16;

__global__ void __launch_bounds__(256)
k_lr_prep_variants(const float* __restrict__ USt, int64_t ldus, const double* __restrict__ Zt, int64_t ldz,
                   const float* __restrict__ Ct, int64_t ldc, int Mc, int k, int N, const double* __restrict__ Qt,
                   int64_t ldq, int D, __half* __restrict__ B1h, __half* __restrict__ B1l, int64_t ldb,
                   float* __restrict__ sb1, __half* __restrict__ B2h, __half* __restrict__ B2l, int64_t ldb2,
                   float* __restrict__ sb2) {
    const int lane = threadIdx.x & 31;
    const int64_t m = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    if (m >= Mc) return;
    const float* u = USt + m * ldus;
    const double* z = Zt + m * ldz;
    const float* cu = Ct + m * ldc;
    // covariate coefficients q_d . s (compensated FP32 per lane, FP64 across the warp)
    float qh[kMaxD], qc[kMaxD];
#pragma unroll
    for (int d = 0; d < kMaxD; ++d) qh[d] = qc[d] = 0.0f;
    for (int n = lane; n < N; n += 32) {
        const float zn = static_cast<float>(z[n]);
#pragma unroll
        for (int d = 0; d < kMaxD; ++d)
            if (d < D) neumaier(qh[d], qc[d], static_cast<float>(Qt[d * ldq + n]) * zn);
    }
    float coef[kMaxD];
#pragma unroll
    for (int d = 0; d < kMaxD; ++d) coef[d] = d < D ? warp_sum_pair(qh[d], qc[d]) : 0.0f;
    auto resid = [&](int n) {
        float v = static_cast<float>(z[n]) - cu[n];
#pragma unroll
        for (int d = 0; d < kMaxD; ++d)
            if (d < D) v = fmaf(-coef[d], static_cast<float>(Qt[d * ldq + n]), v);
        return v;
    };
    float mu = 0.0f, mr = 0.0f, m2 = 0.0f, rr = 0.0f, rc = 0.0f;
    for (int i = lane; i < k; i += 32) {
        const float ui = u[i];
        mu = fmaxf(mu, fabsf(ui));
        m2 = fmaxf(m2, ui * ui);
    }
    for (int n = lane; n < N; n += 32) {
        const float v = resid(n);
        mr = fmaxf(mr, fabsf(v));
        neumaier(rr, rc, v * v);
    }
    float m1 = fmaxf(mu, mr);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, o));
        m2 = fmaxf(m2, __shfl_xor_sync(0xffffffffu, m2, o));
    }
    const float ssr = warp_sum_pair(rr, rc);
    m2 = fmaxf(m2, ssr);
    int e1, e2;
    const float mul1 = row_scale_exp(m1, &e1), mul2 = row_scale_exp(m2, &e2);
    for (int i = lane; i < k; i += 32) {
        const float ui = u[i];
        split_store(ui, mul1, B1h, B1l, m * ldb + i);
        split_store(ui * ui, mul2, B2h, B2l, m * ldb2 + i);
    }
    for (int n = lane; n < N; n += 32) split_store(resid(n), mul1, B1h, B1l, m * ldb + k + n);
    if (lane == 0) {
        split_store(ssr, mul2, B2h, B2l, m * ldb2 + k);
        sb1[m] = ldexpf(1.0f, -e1);
        sb2[m] = ldexpf(1.0f, -e2);
    }
}

// node weights W (R, ldw) FP64: W[r, i] = w~_i(x_r) for i < k, W[r, k] = c(x_r), x_r = x0 + r h
__global__ void k_lr_interp_nodes(const double* __restrict__ s, int k, const float* __restrict__ shat_p, double x0,
                                  double h, int R, double* __restrict__ W, int64_t ldw) {
    const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t >= static_cast<int64_t>(R) * (k + 1)) return;
    const int r = static_cast<int>(t / (k + 1)), i = static_cast<int>(t % (k + 1));
    const double delta = exp(x0 + r * h);
    const double num = static_cast<double>(*shat_p) + delta;
    W[r * ldw + i] = i < k ? num / (s[i] + delta) : num / delta;
}

// ---- strong-test re-evaluation of the low-rank scan ---------------------------------------------------------------
//
// The fused kernel's rss = rWr - sWy^2 / sWs cancels for strong associations (csrc/flmm_wald_refine.cu explains the
// error growth); here a listed test (m, p) is recomputed from the same operands with no cancelling subtraction, over
// the on-rank part (w_i = 1 / (s_i + delta), US and UY, k entries) and the off-rank part (w = 1 / delta, the
// residuals UUS = S_r - Ct and UUY, N entries): e = y - b u at the scan's beta b, rss0 = sum w e^2, sWs = sum w u^2,
// rWr = sum w y^2, g = sum w e u, beta = b + g / sWs, rss = rss0 - g^2 / sWs, on var_df degrees of freedom.

struct LrRefineArgs {
    const float* US;     // (Mc, ldus) FP32
    int64_t ldus;
    const float* UY;     // (P, lduy) FP32
    int64_t lduy;
    const double* Sr;    // (Mc, ldz) FP64 covariate-regressed variants
    int64_t ldz;
    const float* Ct;     // (Mc, ldc) FP32 U_eff US
    int64_t ldc;
    const double* UUY;   // (P, lduu) FP64 residuals
    int64_t lduu;
    const float* s32;    // (k,)
    const double* log_delta;
    int k, N, Mc, n_real, var_df;
    const int64_t* rows;
    double *f, *beta, *se, *sfve;
    int64_t ldo;
    double* max_F;
    float f_refine;
};

__device__ __forceinline__ void acc2(float& s, float& c, float x) {
    float t, e;
    two_sum(s, x, t, e);
    s = t;
    c += e;
}

__device__ void lr_refine_one(const LrRefineArgs& a, int m, int p) {
    const int lane = threadIdx.x & 31;
    const int64_t o = a.rows[m] * a.ldo + p;
    const float b = static_cast<float>(a.beta[o]);
    const double dld = exp(a.log_delta[p]);
    const float dl = static_cast<float>(dld);
    float s0 = 0.f, c0 = 0.f, s1 = 0.f, c1 = 0.f, s2 = 0.f, c2 = 0.f, s3 = 0.f, c3 = 0.f;
    const float* u = a.US + static_cast<int64_t>(m) * a.ldus;
    const float* r = a.UY + static_cast<int64_t>(p) * a.lduy;
    for (int i = lane; i < a.k; i += 32) {
        const float w = __frcp_rn(a.s32[i] + dl);
        const float un = u[i], rn = r[i];
        const float e = fmaf(-b, un, rn);
        acc2(s0, c0, (w * e) * e);
        acc2(s1, c1, (w * un) * un);
        acc2(s2, c2, (w * rn) * rn);
        acc2(s3, c3, (w * e) * un);
    }
    // off-rank: unit weights here, 1 / delta applied to the totals
    float t0 = 0.f, d0 = 0.f, t1 = 0.f, d1 = 0.f, t2 = 0.f, d2 = 0.f, t3 = 0.f, d3 = 0.f;
    const double* z = a.Sr + static_cast<int64_t>(m) * a.ldz;
    const float* cu = a.Ct + static_cast<int64_t>(m) * a.ldc;
    const double* y = a.UUY + static_cast<int64_t>(p) * a.lduu;
    for (int n = lane; n < a.N; n += 32) {
        const float un = static_cast<float>(z[n]) - cu[n];
        const float rn = static_cast<float>(y[n]);
        const float e = fmaf(-b, un, rn);
        acc2(t0, d0, e * e);
        acc2(t1, d1, un * un);
        acc2(t2, d2, rn * rn);
        acc2(t3, d3, e * un);
    }
    const double inv_d = 1.0 / dld;
    auto tot = [&](float sa, float ca, float sb, float cb) {
        const double v = static_cast<double>(sa) + static_cast<double>(ca) +
                         inv_d * (static_cast<double>(sb) + static_cast<double>(cb));
        return warp_sum(v);
    };
    const double rss0 = tot(s0, c0, t0, d0);
    const double sws = tot(s1, c1, t1, d1);
    const double rwr = tot(s2, c2, t2, d2);
    const double g = tot(s3, c3, t3, d3);
    if (lane != 0 || !(sws > 0.0)) return;
    const double df = static_cast<double>(a.var_df);
    const double bt = static_cast<double>(b) + g / sws;
    const double rss = fmax(rss0 - g * g / sws, kPosFloor);
    const double q = bt * bt * sws;
    const double F = q * df / rss;
    a.f[o] = F;
    a.beta[o] = bt;
    a.se[o] = sqrt(rss / df / sws);
    a.sfve[o] = sqrt(fmax(q / fmax(rwr, kPosFloor), 0.0));
    atomic_max_nonneg(a.max_F + p, F);
}

__global__ void __launch_bounds__(256) k_lr_refine_list(const int2* __restrict__ flags, const int* count, int cap,
                                                        LrRefineArgs a) {
    const int n = *count;
    if (n > cap) return;  // the list is incomplete: k_lr_refine_scan recomputes the block instead
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int e = wid; e < n; e += nw) {
        const int2 t = flags[e];
        lr_refine_one(a, t.x, t.y);
    }
}

__global__ void __launch_bounds__(256) k_lr_refine_scan(const int* count, int cap, LrRefineArgs a) {
    if (*count <= cap) return;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    for (int m = wid; m < a.Mc; m += nw) {
        const double* frow = a.f + a.rows[m] * a.ldo;
        for (int p0 = 0; p0 < a.n_real; p0 += 32) {
            const int p = p0 + lane;
            const bool hit = p < a.n_real && frow[p] > static_cast<double>(a.f_refine);
            unsigned mask = __ballot_sync(0xffffffffu, hit);
            while (mask) {
                const int bb = __ffs(mask) - 1;
                mask &= mask - 1;
                lr_refine_one(a, m, p0 + bb);
            }
        }
    }
}

}  // namespace

extern "C" int flmm_lr_wald_refine(const int32_t* flags, const int32_t* flag_count, int flag_cap, float f_refine,
                                   const float* USt, int64_t ldus, const float* UYt, int64_t lduy, const double* Sr,
                                   int64_t ldz, const float* Ct, int64_t ldc, const double* UUYt, int64_t lduu,
                                   const float* s32, const double* log_delta, int k, int N, int Mc, int n_real,
                                   int var_df, const int64_t* rows, double* f, double* beta, double* se, double* sfve,
                                   int64_t ldo, double* max_F, void* stream) {
    FLMM_REQUIRE(flag_count && flag_cap >= 0 && (flags || flag_cap == 0) && k > 0 && N > 0 && Mc >= 0 &&
                     n_real >= 0 && var_df > 0 && ldus >= k && lduy >= k && ldz >= N && ldc >= N && lduu >= N,
                 "flmm_lr_wald_refine: bad arguments");
    if (Mc == 0 || n_real == 0) return FLMM_OK;
    FLMM_REQUIRE(USt && UYt && Sr && Ct && UUYt && s32 && log_delta && rows && f && beta && se && sfve && max_F &&
                     ldo >= n_real,
                 "flmm_lr_wald_refine: operands or outputs missing");
    LrRefineArgs a{USt, ldus, UYt, lduy, Sr, ldz, Ct, ldc, UUYt, lduu, s32, log_delta, k, N, Mc, n_real, var_df,
                   rows, f, beta, se, sfve, ldo, max_F, f_refine};
    cudaStream_t st = as_stream(stream);
    if (flag_cap > 0) {
        k_lr_refine_list<<<64, 256, 0, st>>>(reinterpret_cast<const int2*>(flags), flag_count, flag_cap, a);
        int rc = check_launch("k_lr_refine_list");
        if (rc) return rc;
    }
    k_lr_refine_scan<<<64, 256, 0, st>>>(flag_count, flag_cap, a);
    return check_launch("k_lr_refine_scan");
}

extern "C" int flmm_lr_residual(const double* Y, int64_t ldy, const float* C, int64_t ldc, int rows, int N, double* R,
                                int64_t ldr, double* ss, void* stream) {
    FLMM_REQUIRE(Y && C && R && ss && rows >= 0 && N > 0 && ldy >= N && ldc >= N && ldr >= N,
                 "flmm_lr_residual: bad arguments");
    if (rows == 0) return FLMM_OK;
    k_lr_residual<<<ceil_div(static_cast<int64_t>(rows) * 32, 256), 256, 0, as_stream(stream)>>>(Y, ldy, C, ldc, rows,
                                                                                              N, R, ldr, ss);
    return check_launch("k_lr_residual");
}

extern "C" int flmm_lr_prep_columns(const float* s32, int k, const float* UYt, int64_t ldu, const double* UUYt,
                                    int64_t ldy, int N, const double* yy_off, const double* log_delta, int P,
                                    const float* shat, double x0, double h, int R, void* A1h, void* A1l, int64_t lda,
                                    void* Lh, void* Ll, int64_t ldl, float* sa1, float* sl, float* rWr, float* rWr0,
                                    void* stream) {
    FLMM_REQUIRE(s32 && UYt && UUYt && yy_off && log_delta && shat && A1h && A1l && Lh && Ll && sa1 && sl && rWr &&
                     rWr0 && k > 0 && N > 0 && ldu >= k && ldy >= N && lda >= static_cast<int64_t>(k) + N && ldl >= R &&
                     R >= kInterpPoints && h > 0 && P >= 0,
                 "flmm_lr_prep_columns: bad arguments");
    if (P == 0) return FLMM_OK;
    k_lr_prep_columns<<<ceil_div(P, kCols), 32 * kCols, 0, as_stream(stream)>>>(
        s32, k, UYt, ldu, UUYt, ldy, N, yy_off, log_delta, P, shat, x0, h, 1.0 / h, R, static_cast<__half*>(A1h),
        static_cast<__half*>(A1l), lda, static_cast<__half*>(Lh), static_cast<__half*>(Ll), ldl, sa1, sl, rWr, rWr0);
    return check_launch("k_lr_prep_columns");
}

extern "C" int flmm_lr_prep_variants(const float* USt, int64_t ldus, const double* Zt, int64_t ldz, const float* Ct,
                                     int64_t ldc, int Mc, int k, int N, const double* Qt, int64_t ldq, int D, void* B1h,
                                     void* B1l, int64_t ldb, float* sb1, void* B2h, void* B2l, int64_t ldb2, float* sb2,
                                     void* stream) {
    FLMM_REQUIRE(USt && Zt && Ct && B1h && B1l && sb1 && B2h && B2l && sb2 && k > 0 && N > 0 && Mc >= 0 &&
                     ldus >= k && ldz >= N && ldc >= N && ldb >= static_cast<int64_t>(k) + N && ldb2 >= k + 1 &&
                     D >= 0 && D <= kMaxD && (D == 0 || (Qt && ldq >= N)),
                 "flmm_lr_prep_variants: bad arguments (at most 16 covariate columns)");
    if (Mc == 0) return FLMM_OK;
    k_lr_prep_variants<<<ceil_div(static_cast<int64_t>(Mc) * 32, 256), 256, 0, as_stream(stream)>>>(
        USt, ldus, Zt, ldz, Ct, ldc, Mc, k, N, Qt, ldq, D, static_cast<__half*>(B1h), static_cast<__half*>(B1l), ldb,
        sb1, static_cast<__half*>(B2h), static_cast<__half*>(B2l), ldb2, sb2);
    return check_launch("k_lr_prep_variants");
}

extern "C" int flmm_lr_interp_nodes(const double* s, int k, const float* shat, double x0, double h, int R, double* W,
                                    int64_t ldw, void* stream) {
    FLMM_REQUIRE(s && shat && W && k > 0 && R > 0 && ldw >= k + 1 && h > 0, "flmm_lr_interp_nodes: bad arguments");
    k_lr_interp_nodes<<<ceil_div(static_cast<int64_t>(R) * (k + 1), 256), 256, 0, as_stream(stream)>>>(s, k, shat, x0,
                                                                                                     h, R, W, ldw);
    return check_launch("k_lr_interp_nodes");
}
