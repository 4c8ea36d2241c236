// FP64 SIMT GEMM of the plain (FP64-faithful) form: the per-chromosome Gram that builds every LOCO kinship
// (fasterlmm/io.py:257-265) and the eigenbasis rotations (fasterlmm/core.py:518, :629).  GB300's FP64 pipe is the
// bound here, so a 64 x 64 register-blocked tile with 16-deep shared-memory stages is enough to keep it busy.
#include "flmm_common.cuh"

using namespace flmm;

namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 256;

// C (Mr, Nr) = alpha * sum_k A(i, k) B(j, k) + beta * C.  A(i, k) is A[i * lda + k] when AK (k contiguous), else
// A[k * lda + i]; likewise B.  Thread (tx, ty) of the 16 x 16 block owns rows i0 + ty + 16 r and columns
// j0 + tx + 16 c, so stores of consecutive tx hit consecutive columns.
template <bool AK, bool BK_CONTIG>
__global__ void __launch_bounds__(NT)
k_gemm_f64(const double* __restrict__ A, int64_t lda, const double* __restrict__ B, int64_t ldb, double* __restrict__ C,
           int64_t ldc, int Mr, int Nr, int K, double alpha, double beta) {
    __shared__ double As[BK][BM + 1];
    __shared__ double Bs[BK][BN + 1];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int i0 = blockIdx.y * BM, j0 = blockIdx.x * BN;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += BK) {
#pragma unroll
        for (int l = 0; l < (BM * BK) / NT; ++l) {
            int t = tid + l * NT;
            int i, k;
            if (AK) { i = t / BK; k = t % BK; } else { k = t / BM; i = t % BM; }
            int gi = i0 + i, gk = k0 + k;
            double v = 0.0;
            if (gi < Mr && gk < K) v = AK ? A[static_cast<int64_t>(gi) * lda + gk] : A[static_cast<int64_t>(gk) * lda + gi];
            As[k][i] = v;
        }
#pragma unroll
        for (int l = 0; l < (BN * BK) / NT; ++l) {
            int t = tid + l * NT;
            int j, k;
            if (BK_CONTIG) { j = t / BK; k = t % BK; } else { k = t / BN; j = t % BN; }
            int gj = j0 + j, gk = k0 + k;
            double v = 0.0;
            if (gj < Nr && gk < K) v = BK_CONTIG ? B[static_cast<int64_t>(gj) * ldb + gk] : B[static_cast<int64_t>(gk) * ldb + gj];
            Bs[k][j] = v;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < BK; ++k) {
            double a[4], b[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) a[r] = As[k][ty + 16 * r];
#pragma unroll
            for (int c = 0; c < 4; ++c) b[c] = Bs[k][tx + 16 * c];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        int gi = i0 + ty + 16 * r;
        if (gi >= Mr) continue;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            int gj = j0 + tx + 16 * c;
            if (gj >= Nr) continue;
            double* dst = C + static_cast<int64_t>(gi) * ldc + gj;
            double v = alpha * acc[r][c];
            *dst = (beta == 0.0) ? v : v + beta * (*dst);
        }
    }
}

}  // namespace

extern "C" int flmm_gemm_nt_f64(const double* A, int64_t lda, const double* B, int64_t ldb, double* C, int64_t ldc,
                                int Mr, int Nr, int K, double alpha, void* stream) {
    FLMM_REQUIRE(A && B && C && Mr >= 0 && Nr >= 0 && K >= 0 && lda >= K && ldb >= K && ldc >= Nr,
                 "flmm_gemm_nt_f64: bad arguments");
    if (Mr == 0 || Nr == 0) return FLMM_OK;
    dim3 grid(ceil_div(Nr, BN), ceil_div(Mr, BM));
    k_gemm_f64<true, true><<<grid, NT, 0, as_stream(stream)>>>(A, lda, B, ldb, C, ldc, Mr, Nr, K, alpha, 0.0);
    return check_launch("k_gemm_f64<nt>");
}

extern "C" int flmm_gram_f64(const double* Zt, int64_t ldzt, int M, int N, double beta, double* Gc, int64_t ldg,
                             void* stream) {
    FLMM_REQUIRE(Zt && Gc && M >= 0 && N > 0 && ldzt >= N && ldg >= N, "flmm_gram_f64: bad arguments");
    if (M == 0 && beta != 0.0) return FLMM_OK;
    dim3 grid(ceil_div(N, BN), ceil_div(N, BM));
    k_gemm_f64<false, false><<<grid, NT, 0, as_stream(stream)>>>(Zt, ldzt, Zt, ldzt, Gc, ldg, N, N, M, 1.0, beta);
    return check_launch("k_gemm_f64<gram>");
}
