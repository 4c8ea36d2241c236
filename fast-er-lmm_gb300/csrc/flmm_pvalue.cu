// -log10 p of the F(1, df2) tail in FP64 over an array of F statistics (the CLI's post-scan step,
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

}  // namespace

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
