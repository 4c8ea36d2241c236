// The F(1, df2) tail in FP64 over an array of F statistics, as p or -log10 p (the CLI's post-scan step,
// fasterlmm/cli.py:405-406); the maths is in flmm_pvalue.cuh.
#include <math.h>

#include "flmm_common.cuh"
#include "flmm_pvalue.cuh"

using namespace flmm;

namespace {

__global__ void k_neglog10p_f64(const double* __restrict__ F, int64_t n, double df2, double lbeta,
                                double* __restrict__ out) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[i] = neglog10_fsf<double>(F[i], df2, lbeta);
}

__global__ void k_fsf_f64(const double* __restrict__ F, int64_t n, double df2, double lbeta,
                          double* __restrict__ out) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[i] = fsf<double>(F[i], df2, lbeta);
}

// 1-df chi-square quantile of each test's p-value, the input of the genomic inflation factor
// (fasterlmm/inflation.py:19-29): chi2.isf(p, 1) = (Phi^-1(1 - p / 2))^2 = 2 erfcinv(p)^2, p = P(F(1, df2) > F).
// NaN F gives NaN; p below the FP64 range gives +inf, as scipy's isf(0).
__global__ void k_chisq1_f64(const double* __restrict__ F, int64_t n, double df2, double lbeta,
                             double* __restrict__ out) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const double p = fsf<double>(F[i], df2, lbeta);
        const double z = erfcinv(p);
        out[i] = isnan(p) ? NAN : 2.0 * z * z;
    }
}

// Genome-wide threshold per phenotype (fasterlmm/cli.py:128): p = P(F(1, df2) > perm_max_F) for the row's n_perm
// permutation maxima, then numpy.quantile(p, q) with linear interpolation between order statistics.  p is
// decreasing in F, so the ascending p order is the descending F order: the row is sorted once (bitonic, shared
// memory) and only the two straddling order statistics are converted to p.  One block per phenotype.
__global__ void k_perm_threshold(const double* __restrict__ pmax, int B, int n_perm, int npow2, double df2,
                                 double lbeta, double q, double* __restrict__ thresh) {
    extern __shared__ double v[];
    const int b = blockIdx.x;
    const double* row = pmax + static_cast<int64_t>(b) * n_perm;
    for (int i = threadIdx.x; i < npow2; i += blockDim.x) v[i] = (i < n_perm) ? -row[i] : INFINITY;  // -F ascending
    __syncthreads();
    for (int size = 2; size <= npow2; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = threadIdx.x; i < npow2 / 2; i += blockDim.x) {
                const int lo = 2 * i - (i & (stride - 1));
                const int hi = lo + stride;
                const bool up = (lo & size) == 0;
                const double a = v[lo], c = v[hi];
                if ((a > c) == up) {
                    v[lo] = c;
                    v[hi] = a;
                }
            }
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) {
        // numpy's default ("linear"): position h = (n - 1) q, value = x[floor h] + (h - floor h)(x[floor h + 1] - x[floor h])
        const double h = (n_perm - 1) * q;
        const int j = static_cast<int>(floor(h));
        const double frac = h - j;
        const double p0 = fsf<double>(-v[j], df2, lbeta);
        double out = p0;
        if (frac > 0.0 && j + 1 < n_perm) {
            const double p1 = fsf<double>(-v[j + 1], df2, lbeta);
            out = p0 + frac * (p1 - p0);
        }
        thresh[b] = out;
    }
}

}  // namespace

extern "C" int flmm_perm_threshold_p(const double* perm_max_F, int B, int n_perm, int df2, double q, double* thresh,
                                     void* stream) {
    FLMM_REQUIRE((perm_max_F && thresh) || B == 0, "flmm_perm_threshold_p: NULL argument");
    FLMM_REQUIRE(n_perm >= 1 && n_perm <= 16384 && df2 >= 1 && q >= 0.0 && q <= 1.0,
                 "flmm_perm_threshold_p: need 1 <= n_perm <= 16384, df2 >= 1, 0 <= q <= 1");
    if (B == 0) return FLMM_OK;
    int npow2 = 1;
    while (npow2 < n_perm) npow2 <<= 1;
    const size_t smem = sizeof(double) * npow2;
    if (smem > 48 * 1024)
        FLMM_CUDA(cudaFuncSetAttribute(k_perm_threshold, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    const double a = 0.5 * df2;
    const double lbeta = lgamma(a) + lgamma(0.5) - lgamma(a + 0.5);
    k_perm_threshold<<<B, 256, smem, as_stream(stream)>>>(perm_max_F, B, n_perm, npow2, static_cast<double>(df2),
                                                          lbeta, q, thresh);
    return check_launch("k_perm_threshold");
}

extern "C" int flmm_neglog10_pvalue(const double* F, int64_t n, int df2, double* out, void* stream) {
    FLMM_REQUIRE((F && out) || n == 0, "flmm_neglog10_pvalue: NULL argument");
    FLMM_REQUIRE(df2 >= 1, "flmm_neglog10_pvalue: df2 must be >= 1 (got %d)", df2);
    if (n == 0) return FLMM_OK;
    const double a = 0.5 * df2;
    const double lbeta = lgamma(a) + lgamma(0.5) - lgamma(a + 0.5);
    const unsigned blocks = static_cast<unsigned>(n / 256 + 1 < 152 * 16 ? n / 256 + 1 : 152 * 16);
    k_neglog10p_f64<<<blocks, 256, 0, as_stream(stream)>>>(F, n, static_cast<double>(df2), lbeta, out);
    return check_launch("k_neglog10p_f64");
}

extern "C" int flmm_chisq1_from_f(const double* F, int64_t n, int df2, double* out, void* stream) {
    FLMM_REQUIRE((F && out) || n == 0, "flmm_chisq1_from_f: NULL argument");
    FLMM_REQUIRE(df2 >= 1, "flmm_chisq1_from_f: df2 must be >= 1 (got %d)", df2);
    if (n == 0) return FLMM_OK;
    const double a = 0.5 * df2;
    const double lbeta = lgamma(a) + lgamma(0.5) - lgamma(a + 0.5);
    const unsigned blocks = static_cast<unsigned>(n / 256 + 1 < 152 * 16 ? n / 256 + 1 : 152 * 16);
    k_chisq1_f64<<<blocks, 256, 0, as_stream(stream)>>>(F, n, static_cast<double>(df2), lbeta, out);
    return check_launch("k_chisq1_f64");
}

extern "C" int flmm_f_pvalue(const double* F, int64_t n, int df2, double* out, void* stream) {
    FLMM_REQUIRE((F && out) || n == 0, "flmm_f_pvalue: NULL argument");
    FLMM_REQUIRE(df2 >= 1, "flmm_f_pvalue: df2 must be >= 1 (got %d)", df2);
    if (n == 0) return FLMM_OK;
    const double a = 0.5 * df2;
    const double lbeta = lgamma(a) + lgamma(0.5) - lgamma(a + 0.5);
    const unsigned blocks = static_cast<unsigned>(n / 256 + 1 < 152 * 16 ? n / 256 + 1 : 152 * 16);
    k_fsf_f64<<<blocks, 256, 0, as_stream(stream)>>>(F, n, static_cast<double>(df2), lbeta, out);
    return check_launch("k_fsf_f64");
}
