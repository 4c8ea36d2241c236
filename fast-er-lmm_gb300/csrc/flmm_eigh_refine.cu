// One refinement step for FP32 eigendecompositions of FP64 symmetric matrices (the fast form's LOCO kinships).
//
// An FP32 eigensolver is ~3.5x faster than the FP64 one on GB300 for the scan's batch of N = 1,000 matrices, but
// its eigenvectors carry ~1e-7-relative errors that a flat likelihood turns into a visible shift of the fitted
// delta.  One step of the Ogita-Aishima iteration (T. Ogita, K. Aishima, "Iterative refinement for symmetric
// eigenvalue decomposition", Japan J. Indust. Appl. Math. 35, 2018) removes the first-order error: with rows u_j of
// U (approximate eigenvectors) and
//     lambda_j = u_j^T A u_j / u_j^T u_j,     r_j = A u_j - lambda_j u_j,
//     E_ij = u_i^T r_j / (lambda_j - lambda_i)  (i != j),   E_jj = (1 - u_j^T u_j) / 2,
// the update is u'_j = u_j + sum_i E_ij u_i.  Only A u_j needs high precision: r_j is ~1e-7 of A u_j and must keep
// ~4 digits, so W = U A is formed FP64-accurately -- by default on the FP16 tensor cores from exact digit planes
// (flmm_ozaki.cu; the step then works on the planes' rounding U~ of U, ~2^-46 relative), else in double-FP32
// arithmetic on the FP32 pipe (hi / lo pairs, exact products by FMA, TwoSum accumulation, ~2^-44 relative);
// u_i^T r_j and the update are small corrections and run in FP32.
// Pairs closer than tau = 1e-6 max|lambda| are left unrotated (their mixing does not change the likelihood).
#include <math.h>

#include <cstdlib>
#include <cstring>

#include "flmm_common.cuh"

using namespace flmm;

namespace {

// x = hi + lo with hi = fl32(x), lo = fl32(x - hi): 48 significant bits
__global__ void k_split_pairs(const double* __restrict__ x, int64_t n, float* __restrict__ hi, float* __restrict__ lo) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    const float h = static_cast<float>(v);
    hi[i] = h;
    lo[i] = static_cast<float>(v - static_cast<double>(h));
}

constexpr int DB = 64, DK = 16, DT = 256;  // 64 x 64 output tile, 16-deep k chunks, 16 x 16 threads of 4 x 4

// W[b] (N, N) FP64 = U[b] (N, N, FP32 rows) x A[b]^T with A given as FP32 pairs (Ah + Al); A symmetric, so row m of
// A is column m.  Double-FP32 accumulation per output.
__global__ void __launch_bounds__(DT)
k_df32_gemm_nt(const float* __restrict__ U, const float* __restrict__ Ah, const float* __restrict__ Al, int N,
               double* __restrict__ W) {
    __shared__ float Us[DK][DB + 1];
    __shared__ float Hs[DK][DB + 1];
    __shared__ float Ls[DK][DB + 1];
    const int64_t nn = static_cast<int64_t>(N) * N;
    const float* Ub = U + blockIdx.z * nn;
    const float* Hb = Ah + blockIdx.z * nn;
    const float* Lb = Al + blockIdx.z * nn;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int i0 = blockIdx.y * DB, m0 = blockIdx.x * DB;
    float hi[4][4] = {}, lo[4][4] = {};
    for (int k0 = 0; k0 < N; k0 += DK) {
#pragma unroll
        for (int l = 0; l < (DB * DK) / DT; ++l) {
            const int t = tid + l * DT, r = t / DK, k = t % DK;
            const int gk = k0 + k;
            const int gi = i0 + r, gm = m0 + r;
            Us[k][r] = (gi < N && gk < N) ? Ub[static_cast<int64_t>(gi) * N + gk] : 0.0f;
            const bool okm = gm < N && gk < N;
            Hs[k][r] = okm ? Hb[static_cast<int64_t>(gm) * N + gk] : 0.0f;
            Ls[k][r] = okm ? Lb[static_cast<int64_t>(gm) * N + gk] : 0.0f;
        }
        __syncthreads();
#pragma unroll 4
        for (int k = 0; k < DK; ++k) {
            float a[4], bh[4], bl[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) a[r] = Us[k][ty + 16 * r];
#pragma unroll
            for (int c = 0; c < 4; ++c) { bh[c] = Hs[k][tx + 16 * c]; bl[c] = Ls[k][tx + 16 * c]; }
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const float p = a[r] * bh[c];
                    const float e = fmaf(a[r], bh[c], -p);    // a bh = p + e exactly
                    const float t = fmaf(a[r], bl[c], e);
                    float s, err;
                    two_sum(hi[r][c], p, s, err);
                    hi[r][c] = s;
                    lo[r][c] += err + t;
                }
        }
        __syncthreads();
    }
    double* Wb = W + blockIdx.z * nn;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int i = i0 + ty + 16 * r;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int m = m0 + tx + 16 * c;
            if (i < N && m < N) Wb[static_cast<int64_t>(i) * N + m] = static_cast<double>(hi[r][c]) + lo[r][c];
        }
    }
}

// Per row j (one warp): lambda_j = (W_j . u_j) / (u_j . u_j), nrm_j = u_j . u_j, R_j = fl32(W_j - lambda_j u_j).
__global__ void k_rq_residual(const double* __restrict__ W, const float* __restrict__ U, int N, int rows,
                              double* __restrict__ lam, double* __restrict__ nrm, float* __restrict__ R) {
    const int lane = threadIdx.x & 31;
    const int64_t j = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    if (j >= rows) return;
    const double* w = W + j * N;
    const float* u = U + j * N;
    double q = 0.0, uu = 0.0;
    for (int n = lane; n < N; n += 32) {
        const double un = u[n];
        q = fma(w[n], un, q);
        uu = fma(un, un, uu);
    }
    q = warp_sum(q);
    uu = warp_sum(uu);
    const double l = q / uu;
    for (int n = lane; n < N; n += 32) R[j * N + n] = static_cast<float>(w[n] - l * static_cast<double>(u[n]));
    if (lane == 0) {
        lam[j] = l;
        nrm[j] = uu;
    }
}

constexpr int FB = 64, FK = 16, FT = 256;

// largest first-order rotation E_ij one refinement step applies to a pair of eigenvectors
constexpr double kMaxRotation = 0.25;

// FP32 batched products, C[b] = A[b] B[b]^T (NT) or A[b] B[b] (NN), (N, N) each; with ADD the result is added to
// D[b] and written to C[b].
template <bool NT, bool ADD>
__global__ void __launch_bounds__(FT)
k_f32_gemm(const float* __restrict__ A, const float* __restrict__ B, const float* __restrict__ D, int N,
           float* __restrict__ Cm) {
    __shared__ float As[FK][FB + 1];
    __shared__ float Bs[FK][FB + 1];
    const int64_t nn = static_cast<int64_t>(N) * N;
    const float* Ab = A + blockIdx.z * nn;
    const float* Bb = B + blockIdx.z * nn;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int i0 = blockIdx.y * FB, m0 = blockIdx.x * FB;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < N; k0 += FK) {
#pragma unroll
        for (int l = 0; l < (FB * FK) / FT; ++l) {
            const int t = tid + l * FT;
            {
                const int r = t / FK, k = t % FK, gi = i0 + r, gk = k0 + k;
                As[k][r] = (gi < N && gk < N) ? Ab[static_cast<int64_t>(gi) * N + gk] : 0.0f;
            }
            if (NT) {
                const int r = t / FK, k = t % FK, gm = m0 + r, gk = k0 + k;
                Bs[k][r] = (gm < N && gk < N) ? Bb[static_cast<int64_t>(gm) * N + gk] : 0.0f;
            } else {
                const int k = t / FB, c = t % FB, gm = m0 + c, gk = k0 + k;
                Bs[k][c] = (gm < N && gk < N) ? Bb[static_cast<int64_t>(gk) * N + gm] : 0.0f;
            }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < FK; ++k) {
            float a[4], b[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) a[r] = As[k][ty + 16 * r];
#pragma unroll
            for (int c = 0; c < 4; ++c) b[c] = Bs[k][tx + 16 * c];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[r][c] = fmaf(a[r], b[c], acc[r][c]);
        }
        __syncthreads();
    }
    float* Cb = Cm + blockIdx.z * nn;
    const float* Db = ADD ? D + blockIdx.z * nn : nullptr;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int i = i0 + ty + 16 * r;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int m = m0 + tx + 16 * c;
            if (i < N && m < N) {
                const int64_t o = static_cast<int64_t>(i) * N + m;
                Cb[o] = ADD ? Db[o] + acc[r][c] : acc[r][c];
            }
        }
    }
}

// T[j, i] = E_ij = M[i, j] / (lambda_j - lambda_i) where that first-order rotation is small, |E_ij| <= kMaxRotation,
// and the pair is not closer than tau = 1e-6 max |lambda| of the matrix; 0 otherwise.  T[j, j] = (1 - nrm_j) / 2;
// M[i, j] = u_i . r_j.  A pair whose coupling is not small against its gap is left as it is for this step: the
// first-order update is only valid for small rotations (applied to a large one it makes the vectors worse, which is
// what an FP32 decomposition of a 5,000 x 5,000 kinship gives for its closest pairs), the step's other corrections
// shrink the residuals, and a later step rotates the pair once its coupling is small.  A pair left unrotated moves
// the likelihood only by ~ M_ij / (s + delta), whatever the angle.
__global__ void k_refine_coeffs(const float* __restrict__ M, const double* __restrict__ lam,
                                const double* __restrict__ nrm, int N, float* __restrict__ T) {
    const int64_t nn = static_cast<int64_t>(N) * N;
    const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t >= nn) return;
    const int b = blockIdx.y;
    const double* lb = lam + static_cast<int64_t>(b) * N;
    const int j = static_cast<int>(t / N), i = static_cast<int>(t % N);
    float v;
    if (i == j) {
        v = static_cast<float>(0.5 * (1.0 - nrm[static_cast<int64_t>(b) * N + j]));
    } else {
        // the gap is formed in FP64 (close eigenvalues cancel), the rest in FP32: T is stored in FP32, and FP64 is
        // GB300's narrowest pipe (a division is many of its instructions)
        const float tau = 1e-6f * fmaxf(fabsf(static_cast<float>(lb[0])), fabsf(static_cast<float>(lb[N - 1])));
        const float gap = static_cast<float>(lb[j] - lb[i]);
        const float m = M[b * nn + static_cast<int64_t>(i) * N + j];
        v = (fabsf(gap) > tau && fabsf(m) <= static_cast<float>(kMaxRotation) * fabsf(gap)) ? m / gap : 0.0f;
    }
    T[b * nn + t] = v;
}

struct RefineWs {
    void* prod;  // the product's workspace: digit planes (tensor-core form) or the FP32 split of A (double-FP32 form)
    float *Ah, *Al, *Ut, *R, *Mt, *T;
    double *W, *nrm;
    size_t bytes;
};

RefineWs carve(void* base, int N, int batch) {
    RefineWs w{};
    const size_t nn = static_cast<size_t>(N) * N * batch;
    const uintptr_t b = reinterpret_cast<uintptr_t>(base);
    size_t off = 0;
    auto take = [&](size_t nbytes) {
        const uintptr_t p = b + off;
        off += (nbytes + 1023) / 1024 * 1024;
        return p;
    };
    const size_t split_bytes = 2 * ((sizeof(float) * nn + 1023) / 1024 * 1024);
    const size_t tc_bytes = refine_product_tc_bytes(N, batch);
    const uintptr_t prod = take(tc_bytes > split_bytes ? tc_bytes : split_bytes);
    w.prod = reinterpret_cast<void*>(prod);
    w.Ah = reinterpret_cast<float*>(prod);
    w.Al = reinterpret_cast<float*>(prod + split_bytes / 2);
    w.Ut = reinterpret_cast<float*>(take(sizeof(float) * nn));
    w.W = reinterpret_cast<double*>(take(sizeof(double) * nn));
    w.R = reinterpret_cast<float*>(take(sizeof(float) * nn));
    w.Mt = reinterpret_cast<float*>(take(sizeof(float) * nn));
    w.nrm = reinterpret_cast<double*>(take(sizeof(double) * static_cast<size_t>(N) * batch));
    w.T = reinterpret_cast<float*>(prod);  // the product's workspace is dead once W is formed
    w.bytes = off;
    return w;
}

// The product's form: tensor cores (digit planes, flmm_ozaki.cu) unless FLMM_REFINE_PRODUCT=df32 selects the
// double-FP32 kernel on the FP32 pipe (kept for cross-checks; both agree to ~2^-44 relative).
int default_form() {
    static int form = [] {
        const char* e = std::getenv("FLMM_REFINE_PRODUCT");
        return (e && std::strcmp(e, "df32") == 0) ? 1 : 0;
    }();
    return form;
}

// W = U~ A^T in the given form; U~ (the vectors the product is exact for) goes to Ut.
int product(const double* A, const float* U, int N, int batch, int form, const RefineWs& ws, cudaStream_t st) {
    const int64_t total = static_cast<int64_t>(N) * N * batch;
    if (form == 0) return refine_product_tc(U, A, N, batch, ws.Ut, ws.W, ws.prod, st);
    FLMM_CUDA(cudaMemcpyAsync(ws.Ut, U, sizeof(float) * total, cudaMemcpyDeviceToDevice, st));
    k_split_pairs<<<ceil_div(total, 256), 256, 0, st>>>(A, total, ws.Ah, ws.Al);
    int rc = check_launch("k_split_pairs");
    if (rc) return rc;
    const dim3 g64(ceil_div(N, DB), ceil_div(N, DB), batch);
    k_df32_gemm_nt<<<g64, DT, 0, st>>>(U, ws.Ah, ws.Al, N, ws.W);
    return check_launch("k_df32_gemm_nt");
}

}  // namespace

extern "C" int flmm_eigh_refine_workspace_bytes(int N, int batch, size_t* bytes) {
    FLMM_REQUIRE(bytes && N > 0 && batch > 0, "flmm_eigh_refine_workspace_bytes: bad arguments");
    *bytes = carve(nullptr, N, batch).bytes;
    return FLMM_OK;
}

extern "C" int flmm_refine_product_workspace_bytes(int N, int batch, size_t* bytes) {
    FLMM_REQUIRE(bytes && N > 0 && batch > 0, "flmm_refine_product_workspace_bytes: bad arguments");
    *bytes = carve(nullptr, N, batch).bytes;
    return FLMM_OK;
}

extern "C" int flmm_refine_product(const float* U, const double* A, int N, int batch, int form, float* Ut, double* W,
                                   void* work, size_t work_bytes, void* stream) {
    FLMM_REQUIRE(U && A && Ut && W && work && N > 0 && batch > 0 && batch <= 65535 && (form == 0 || form == 1),
                 "flmm_refine_product: bad arguments");
    RefineWs ws = carve(work, N, batch);
    if (work_bytes < ws.bytes)
        return fail(FLMM_ERR_WORKSPACE, "flmm_refine_product: need %zu bytes, got %zu", ws.bytes, work_bytes);
    cudaStream_t st = as_stream(stream);
    const int rc = product(A, U, N, batch, form, ws, st);
    if (rc) return rc;
    const int64_t total = static_cast<int64_t>(N) * N * batch;
    FLMM_CUDA(cudaMemcpyAsync(Ut, ws.Ut, sizeof(float) * total, cudaMemcpyDeviceToDevice, st));
    FLMM_CUDA(cudaMemcpyAsync(W, ws.W, sizeof(double) * total, cudaMemcpyDeviceToDevice, st));
    return FLMM_OK;
}

extern "C" int flmm_eigh_refine_f32(const double* A, float* U, float* U_out, double* evals, int N, int batch,
                                    void* work, size_t work_bytes, void* stream) {
    FLMM_REQUIRE(A && U && U_out && evals && work && N > 0 && batch > 0 && batch <= 65535 && U != U_out,
                 "flmm_eigh_refine_f32: bad arguments");
    RefineWs ws = carve(work, N, batch);
    if (work_bytes < ws.bytes)
        return fail(FLMM_ERR_WORKSPACE, "flmm_eigh_refine_f32: need %zu bytes, got %zu", ws.bytes, work_bytes);
    cudaStream_t st = as_stream(stream);
    // W = U~ A^T; from here on the step works on U~ (ws.Ut), the vectors the product is exact for
    int rc = product(A, U, N, batch, default_form(), ws, st);
    if (rc) return rc;
    const float* Uc = ws.Ut;
    const bool tc = default_form() == 0;
    const dim3 g64(ceil_div(N, DB), ceil_div(N, DB), batch);
    const int64_t rows = static_cast<int64_t>(N) * batch;
    k_rq_residual<<<ceil_div(rows * 32, 256), 256, 0, st>>>(ws.W, Uc, N, static_cast<int>(rows), evals, ws.nrm, ws.R);
    if ((rc = check_launch("k_rq_residual"))) return rc;
    // M[i, j] = u_i . r_j
    if (tc) {
        if ((rc = refine_m_tc(ws.R, N, batch, ws.Mt, ws.prod, st))) return rc;
    } else {
        k_f32_gemm<true, false><<<g64, FT, 0, st>>>(Uc, ws.R, nullptr, N, ws.Mt);
        if ((rc = check_launch("k_f32_gemm<nt>"))) return rc;
    }
    const dim3 gc(ceil_div(static_cast<int64_t>(N) * N, 256), batch);
    k_refine_coeffs<<<gc, 256, 0, st>>>(ws.Mt, evals, ws.nrm, N, ws.T);
    if ((rc = check_launch("k_refine_coeffs"))) return rc;
    // U' = U + T U
    if (tc) return refine_update_tc(ws.T, Uc, ws.Mt, N, batch, U_out, ws.prod, st);
    k_f32_gemm<false, true><<<g64, FT, 0, st>>>(ws.T, Uc, Uc, N, U_out);
    return check_launch("k_f32_gemm<nn>");
}
