// Accurate re-evaluation of the strongest real tests of the split-precision Wald scan.
//
// The fused tensor-core kernel forms rss = rWr - sWy^2 / sWs from FP32 sums (fasterlmm/core.py:651-655).  For a
// strong association q = sWy^2 / sWs approaches rWr, so rss cancels: a relative error e of the sums becomes a
// relative error of about e (1 + F / df) in rss and F, and -log10 p ~ F / (2 ln 10) moves by about
// F e (1 + F / df) / 4.6.  With e ~ 1e-6 that passes 1e-3 near F ~ 1,500 at N = 1,000 and near F ~ 700 at N = 5,000.
//
// The Wald epilogue therefore lists every real test whose F exceeds a cutoff, and this pass recomputes each listed
// test from the same FP32 operands the scan rotated (US row m, UY row p) with no cancelling subtraction:
//
//   e_n  = UY_pn - b US_mn                    (one FMA; b = the scan's beta, so e is the residual at b)
//   rss0 = sum w e^2,  sWs = sum w US^2,  rWr = sum w UY^2,  g = sum w e US     (w_n = 1 / (s_n + delta_p))
//   beta = b + g / sWs,  rss = rss0 - g^2 / sWs,  q = beta^2 sWs,  F = q df / rss
//
// rss(b) is the quadratic rss_min + sWs (b - beta)^2, so rss0 - g^2 / sWs is the exact minimum, and every sum has
// positive terms except g, which is small (b is within ~1e-6 of beta).  The sums are TwoSum-compensated FP32 per
// lane (the FP32 pipe; GB300's FP64 rate is a small fraction of it), combined in FP64 across the warp.  What is
// left is the operands' own rounding, which enters F only as ~2 e_op sqrt(1 + F / df) / sqrt(Neff): the statistic
// of slightly perturbed vectors rather than a cancelled difference.
//
// One warp per listed test.  When a chromosome has more such tests than the list holds, the list is not used and
// the scan mode visits every real test of the chromosome whose stored F exceeds the cutoff -- exactly the tests the
// epilogue counted, each recomputed once from the same inputs -- so both modes give the same bits and max_F always
// gets the recomputed maxima.
#include <math.h>

#include "flmm_common.cuh"

using namespace flmm;

namespace {

struct RefineArgs {
    const float* US;  // (Mc, ldus) rotated variants of the chromosome, FP32
    int64_t ldus;
    const float* UY;  // (P, lduy) rotated columns, FP32
    int64_t lduy;
    const float* s32;          // (Neff,) spectrum, FP32
    const double* log_delta;   // (P,)
    int Neff, Mc, n_real;
    const int64_t* rows;  // (Mc,) output row of each variant of the chromosome
    double* f;
    double* beta;
    double* se;
    double* sfve;
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

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Recompute test (m, p) of the chromosome; called by all 32 lanes of a warp with the same (m, p).
__device__ void refine_one(const RefineArgs& a, int m, int p) {
    const float* u = a.US + static_cast<int64_t>(m) * a.ldus;
    const float* r = a.UY + static_cast<int64_t>(p) * a.lduy;
    const int64_t o = a.rows[m] * a.ldo + p;
    const float b = static_cast<float>(a.beta[o]);
    const float dl = static_cast<float>(exp(a.log_delta[p]));
    float s0 = 0.f, c0 = 0.f, s1 = 0.f, c1 = 0.f, s2 = 0.f, c2 = 0.f, s3 = 0.f, c3 = 0.f;
    for (int n = threadIdx.x & 31; n < a.Neff; n += 32) {
        const float w = __frcp_rn(a.s32[n] + dl);
        const float un = u[n];
        const float rn = r[n];
        const float e = fmaf(-b, un, rn);
        const float we = w * e;
        const float wu = w * un;
        acc2(s0, c0, we * e);
        acc2(s1, c1, wu * un);
        acc2(s2, c2, (w * rn) * rn);
        acc2(s3, c3, we * un);
    }
    const double rss0 = warp_sum_d(static_cast<double>(s0) + static_cast<double>(c0));
    const double sws = warp_sum_d(static_cast<double>(s1) + static_cast<double>(c1));
    const double rwr = warp_sum_d(static_cast<double>(s2) + static_cast<double>(c2));
    const double g = warp_sum_d(static_cast<double>(s3) + static_cast<double>(c3));
    if ((threadIdx.x & 31) != 0 || !(sws > 0.0)) return;
    const double df = static_cast<double>(a.Neff - 1);
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

__global__ void __launch_bounds__(256) k_wald_refine_list(const int2* __restrict__ flags, const int* count, int cap,
                                                          RefineArgs a) {
    const int n = *count;
    if (n > cap) return;  // the list is incomplete: k_wald_refine_scan recomputes the chromosome instead
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int e = wid; e < n; e += nw) {
        const int2 t = flags[e];
        refine_one(a, t.x, t.y);
    }
}

// The list overflowed: every real test of the chromosome whose stored F exceeds the cutoff, one variant per warp,
// 32 columns at a time.
__global__ void __launch_bounds__(256) k_wald_refine_scan(const int* count, int cap, RefineArgs a) {
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
                const int b = __ffs(mask) - 1;
                mask &= mask - 1;
                refine_one(a, m, p0 + b);
            }
        }
    }
}

}  // namespace

int flmm_ctx_sm_count(flmm_context* ctx);

extern "C" int flmm_wald_refine_f32(flmm_context* ctx, const int32_t* flags, const int32_t* flag_count, int flag_cap,
                                    float f_refine, const float* USt, int64_t ldus, const float* UYt, int64_t lduy,
                                    const float* s32, const double* log_delta, int Neff, int Mc, int n_real,
                                    const int64_t* rows, double* f, double* beta, double* se, double* sfve,
                                    int64_t ldo, double* max_F, void* stream) {
    FLMM_REQUIRE(ctx && flag_count && flag_cap >= 0 && (flags || flag_cap == 0) && Neff > 1 && Mc >= 0 &&
                     n_real >= 0 && ldus >= Neff && lduy >= Neff,
                 "flmm_wald_refine_f32: bad arguments");
    if (Mc == 0 || n_real == 0) return FLMM_OK;
    FLMM_REQUIRE(USt && UYt && s32 && log_delta && rows && f && beta && se && sfve && max_F && ldo >= n_real,
                 "flmm_wald_refine_f32: operands or outputs missing");
    RefineArgs a;
    a.US = USt;
    a.ldus = ldus;
    a.UY = UYt;
    a.lduy = lduy;
    a.s32 = s32;
    a.log_delta = log_delta;
    a.Neff = Neff;
    a.Mc = Mc;
    a.n_real = n_real;
    a.rows = rows;
    a.f = f;
    a.beta = beta;
    a.se = se;
    a.sfve = sfve;
    a.ldo = ldo;
    a.max_F = max_F;
    a.f_refine = f_refine;
    cudaStream_t st = as_stream(stream);
    // A small grid: the launch usually finds few or no strong tests, and it must get onto the SMs quickly while the
    // next chromosome's delta fit runs beside it on another stream (a grid of several CTAs per SM waited there for
    // whole waves of that fit and held the Wald stream back ~1 ms per chromosome).
    const int sms = flmm_ctx_sm_count(ctx);
    const unsigned grid = static_cast<unsigned>(sms < 32 ? sms : 32);
    if (flag_cap > 0) {
        k_wald_refine_list<<<grid, 256, 0, st>>>(reinterpret_cast<const int2*>(flags), flag_count, flag_cap, a);
        int rc = check_launch("k_wald_refine_list");
        if (rc) return rc;
    }
    k_wald_refine_scan<<<grid, 256, 0, st>>>(flag_count, flag_cap, a);
    return check_launch("k_wald_refine_scan");
}
