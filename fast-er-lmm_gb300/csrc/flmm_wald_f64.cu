// Plain FP64 form of the compat Wald scan (fasterlmm/core.py:601-671), fused: the two per-chromosome products
// sWy = (w o UY)^T US and sWs = w^T (US o US) share one tile loop, and the epilogue (beta, var_beta, F, SE, SFVE,
// the per-column genome max) runs on the accumulators in registers.  Nothing of size (P, Mc) is written except
// the real columns' detail.
#include <math.h>

#include "flmm_common.cuh"

using namespace flmm;

namespace {

// W[p, n] = 1 / (s[n] + exp(ld[p])), A1 = W o UY, rWr[p] = max(sum_n (W UY) UY, floor)
// (fasterlmm/core.py:639-643); one warp per column
__global__ void k_wald_prep(const double* __restrict__ s, int Neff, const double* __restrict__ UYt, int64_t ldu,
                            const double* __restrict__ ld, int P, double* __restrict__ W, double* __restrict__ A1,
                            double* __restrict__ rWr) {
    const int lane = threadIdx.x & 31;
    const int64_t p = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    if (p >= P) return;
    const double delta = exp(ld[p]);
    const double* u = UYt + p * ldu;
    double acc = 0.0;
    for (int n = lane; n < Neff; n += 32) {
        double w = 1.0 / (s[n] + delta);
        double a = mul_rn(w, u[n]);
        W[p * Neff + n] = w;
        A1[p * Neff + n] = a;
        acc += mul_rn(a, u[n]);
    }
    acc = warp_sum(acc);
    if (lane == 0) rWr[p] = fmax(acc, kPosFloor);
}

constexpr int TP = 64, TM = 64, TK = 16, NT = 256;

// Thread (tx, ty) owns columns p0 + tx + 16 r and variants m0 + ty + 16 c, so the detail stores of consecutive tx
// (consecutive columns of one output row) coalesce.
__global__ void __launch_bounds__(NT)
k_wald_f64(const double* __restrict__ W, const double* __restrict__ A1, const double* __restrict__ rWr, int Neff,
           double var_df, int P, int n_real, const double* __restrict__ USt, int64_t ldus, int Mc,
           const int64_t* __restrict__ rows, double* __restrict__ f, double* __restrict__ beta, double* __restrict__ se,
           double* __restrict__ sfve, int64_t ldo, double* __restrict__ max_F) {
    __shared__ double Ws[TK][TP + 1];
    __shared__ double As[TK][TP + 1];
    __shared__ double Us[TK][TM + 1];
    __shared__ double U2s[TK][TM + 1];
    __shared__ double red[16][TP];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int p0 = blockIdx.y * TP, m0 = blockIdx.x * TM;
    double sy[4][4] = {}, ss[4][4] = {};
    for (int k0 = 0; k0 < Neff; k0 += TK) {
#pragma unroll
        for (int l = 0; l < (TP * TK) / NT; ++l) {
            int t = tid + l * NT, p = t / TK, k = t % TK;
            int gp = p0 + p, gk = k0 + k;
            bool ok = gp < P && gk < Neff;
            Ws[k][p] = ok ? W[static_cast<int64_t>(gp) * Neff + gk] : 0.0;
            As[k][p] = ok ? A1[static_cast<int64_t>(gp) * Neff + gk] : 0.0;
        }
#pragma unroll
        for (int l = 0; l < (TM * TK) / NT; ++l) {
            int t = tid + l * NT, m = t / TK, k = t % TK;
            int gm = m0 + m, gk = k0 + k;
            double v = (gm < Mc && gk < Neff) ? USt[static_cast<int64_t>(gm) * ldus + gk] : 0.0;
            Us[k][m] = v;
            U2s[k][m] = mul_rn(v, v);
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < TK; ++k) {
            double a[4], w[4], u[4], u2[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) { a[r] = As[k][tx + 16 * r]; w[r] = Ws[k][tx + 16 * r]; }
#pragma unroll
            for (int c = 0; c < 4; ++c) { u[c] = Us[k][ty + 16 * c]; u2[c] = U2s[k][ty + 16 * c]; }
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    sy[r][c] = fma(a[r], u[c], sy[r][c]);
                    ss[r][c] = fma(w[r], u2[c], ss[r][c]);
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int p = p0 + tx + 16 * r;
        const bool p_ok = p < P;
        const double rwr = p_ok ? rWr[p] : 1.0;
        double colmax = -INFINITY;
        bool col_nan = false;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int m = m0 + ty + 16 * c;
            if (!p_ok || m >= Mc) continue;
            // fasterlmm/core.py:651-655, in the reference's operation order
            const double swy = sy[r][c];
            const double denom = fmax(ss[r][c], kPosFloor);
            const double b = swy / denom;
            const double q = mul_rn(swy, swy);
            const double rss = fmax(add_rn(rwr, -(q / denom)), kPosFloor);
            const double var_b = (rss / var_df) / denom;
            const double F = mul_rn(b, b) / var_b;
            colmax = fmax(colmax, F);
            col_nan |= isnan(F);
            if (p < n_real) {
                const int64_t o = rows[m] * ldo + p;
                f[o] = F;
                beta[o] = b;
                se[o] = sqrt(var_b);
                sfve[o] = sqrt(fmax(q / mul_rn(denom, rwr), 0.0));
            }
        }
        red[ty][tx + 16 * r] = col_nan ? NAN : colmax;
    }
    __syncthreads();
    if (tid < TP && p0 + tid < P) {
        double v = -INFINITY;
        bool any_nan = false;
        for (int r = 0; r < 16; ++r) {
            double x = red[r][tid];
            any_nan |= isnan(x);
            v = fmax(v, x);
        }
        if (any_nan) v = NAN;
        if (v >= 0.0 || isnan(v)) atomic_max_nonneg(max_F + p0 + tid, v);
    }
}

size_t wald_ws(int P, int Neff) {
    return sizeof(double) * (2 * static_cast<size_t>(P) * Neff + static_cast<size_t>(P)) + 512;
}

}  // namespace

extern "C" int flmm_wald_f64_workspace_bytes(int P, int Neff, size_t* bytes) {
    FLMM_REQUIRE(bytes && P >= 0 && Neff > 0, "flmm_wald_f64_workspace_bytes: bad arguments");
    *bytes = wald_ws(P, Neff);
    return FLMM_OK;
}

namespace {

// rows of [A | B] (rows, ka + kb) from A (rows, ka) and B (rows, kb)
__global__ void k_concat_rows(const double* __restrict__ A, int64_t lda, int ka, const double* __restrict__ B,
                              int64_t ldb, int kb, int rows, double* __restrict__ C) {
    const int k = ka + kb;
    const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t >= static_cast<int64_t>(rows) * k) return;
    const int64_t r = t / k;
    const int c = static_cast<int>(t % k);
    C[t] = c < ka ? A[r * lda + c] : B[r * ldb + (c - ka)];
}

__global__ void k_spectrum_pad(const double* __restrict__ s, int k, int n0, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < k + n0) out[i] = i < k ? s[i] : 0.0;
}

int wald_impl(const double* s, int Neff, const double* UYt, int64_t ldu, const double* log_delta, int P, int n_real,
              const double* USt, int64_t ldus, int Mc, const int64_t* rows, double* f, double* beta, double* se,
              double* sfve, int64_t ldo, double* max_F, double var_df, void* work, cudaStream_t st) {
    double* W = static_cast<double*>(work);
    double* A1 = W + static_cast<size_t>(P) * Neff;
    double* rWr = A1 + static_cast<size_t>(P) * Neff;
    k_wald_prep<<<ceil_div(static_cast<int64_t>(P) * 32, 256), 256, 0, st>>>(s, Neff, UYt, ldu, log_delta, P, W, A1,
                                                                             rWr);
    int rc = check_launch("k_wald_prep");
    if (rc) return rc;
    dim3 grid(ceil_div(Mc, TM), ceil_div(P, TP));
    k_wald_f64<<<grid, NT, 0, st>>>(W, A1, rWr, Neff, var_df, P, n_real, USt, ldus, Mc, rows, f, beta, se, sfve, ldo,
                                    max_F);
    return check_launch("k_wald_f64");
}

size_t lowrank_cat_doubles(int k, int N, int P, int Mc) {
    return static_cast<size_t>(k + N) * (1 + static_cast<size_t>(P) + static_cast<size_t>(Mc));
}

}  // namespace

extern "C" int flmm_wald_f64(const double* s, int Neff, const double* UYt, int64_t ldu, const double* log_delta, int P,
                             int n_real, const double* USt, int64_t ldus, int Mc, const int64_t* rows, double* f,
                             double* beta, double* se, double* sfve, int64_t ldo, double* max_F, void* work,
                             size_t work_bytes, void* stream) {
    FLMM_REQUIRE(s && UYt && log_delta && max_F && work && Neff > 1 && P >= 0 && Mc >= 0 && ldu >= Neff &&
                     ldus >= Neff && n_real >= 0 && n_real <= P,
                 "flmm_wald_f64: bad arguments");
    FLMM_REQUIRE(n_real == 0 || Mc == 0 || (rows && f && beta && se && sfve && ldo >= n_real),
                 "flmm_wald_f64: real-column outputs missing");
    FLMM_REQUIRE(Mc == 0 || USt, "flmm_wald_f64: USt is NULL");
    if (work_bytes < wald_ws(P, Neff))
        return fail(FLMM_ERR_WORKSPACE, "flmm_wald_f64: need %zu bytes, got %zu", wald_ws(P, Neff), work_bytes);
    if (P == 0 || Mc == 0) return FLMM_OK;
    return wald_impl(s, Neff, UYt, ldu, log_delta, P, n_real, USt, ldus, Mc, rows, f, beta, se, sfve, ldo, max_F,
                     static_cast<double>(Neff - 1), work, as_stream(stream));
}

extern "C" int flmm_wald_lowrank_f64_workspace_bytes(int k, int N, int P, int Mc, size_t* bytes) {
    FLMM_REQUIRE(bytes && k > 0 && N > 0 && P >= 0 && Mc >= 0, "flmm_wald_lowrank_f64_workspace_bytes: bad arguments");
    *bytes = sizeof(double) * lowrank_cat_doubles(k, N, P, Mc) + 256 + wald_ws(P, k + N);
    return FLMM_OK;
}

extern "C" int flmm_wald_lowrank_f64(const double* s, int k, const double* UYt, int64_t ldu, const double* UUYt,
                                     int64_t lduu, int N, int Neff, const double* log_delta, int P, int n_real,
                                     const double* USt, int64_t ldus, const double* UUSt, int64_t lduus, int Mc,
                                     const int64_t* rows, double* f, double* beta, double* se, double* sfve,
                                     int64_t ldo, double* max_F, void* work, size_t work_bytes, void* stream) {
    FLMM_REQUIRE(s && UYt && UUYt && log_delta && max_F && work && k > 0 && N > 0 && Neff > 1 && P >= 0 && Mc >= 0 &&
                     ldu >= k && lduu >= N && ldus >= k && lduus >= N && n_real >= 0 && n_real <= P,
                 "flmm_wald_lowrank_f64: bad arguments");
    FLMM_REQUIRE(n_real == 0 || Mc == 0 || (rows && f && beta && se && sfve && ldo >= n_real),
                 "flmm_wald_lowrank_f64: real-column outputs missing");
    FLMM_REQUIRE(Mc == 0 || (USt && UUSt), "flmm_wald_lowrank_f64: variant operands missing");
    size_t need = 0;
    flmm_wald_lowrank_f64_workspace_bytes(k, N, P, Mc, &need);
    if (work_bytes < need)
        return fail(FLMM_ERR_WORKSPACE, "flmm_wald_lowrank_f64: need %zu bytes, got %zu", need, work_bytes);
    if (P == 0 || Mc == 0) return FLMM_OK;
    // The off-rank directions enter every form with weight 1 / delta, i.e. as eigen-directions with s = 0: the scan
    // is the compat scan over [on-rank | off-rank] = k + N directions with var_df = Neff - 1
    // (fasterlmm/lowrank.py:274-299).
    cudaStream_t st = as_stream(stream);
    const int kc = k + N;
    double* s_cat = static_cast<double*>(work);
    double* UY_cat = s_cat + kc;
    double* US_cat = UY_cat + static_cast<size_t>(P) * kc;
    void* rest = reinterpret_cast<char*>(work) + ((sizeof(double) * lowrank_cat_doubles(k, N, P, Mc) + 255) / 256) * 256;
    k_spectrum_pad<<<ceil_div(kc, 256), 256, 0, st>>>(s, k, N, s_cat);
    int rc = check_launch("k_spectrum_pad");
    if (rc) return rc;
    k_concat_rows<<<ceil_div(static_cast<int64_t>(P) * kc, 256), 256, 0, st>>>(UYt, ldu, k, UUYt, lduu, N, P, UY_cat);
    if ((rc = check_launch("k_concat_rows"))) return rc;
    k_concat_rows<<<ceil_div(static_cast<int64_t>(Mc) * kc, 256), 256, 0, st>>>(USt, ldus, k, UUSt, lduus, N, Mc,
                                                                                 US_cat);
    if ((rc = check_launch("k_concat_rows"))) return rc;
    return wald_impl(s_cat, kc, UY_cat, kc, log_delta, P, n_real, US_cat, kc, Mc, rows, f, beta, se, sfve, ldo, max_F,
                     static_cast<double>(Neff - 1), rest, st);
}
