// Input preparation and the small FP64 steps of the compat rotation: the unit standardiser, the LOCO kinship
// combine, the covariate projection of K + I, the kept spectrum, the OLS regress-out, the delta grid nodes and the
// fills of the result arrays.
#include <math.h>

#include "flmm_common.cuh"

using namespace flmm;

namespace {

// ---- standardiser from FP64 (N, M) sample-major input -------------------------------------------------------
// One block owns 32 consecutive variants; its 8 warps walk the samples.  Pass 1: NaN-aware sum and count; pass 2:
// sum of squared deviations; pass 3: write the transposed, standardised tile through shared memory so that both
// the read (32 variants of one sample) and the write (32 samples of one variant) are coalesced.
constexpr int kStdCols = 32;
constexpr int kStdRows = 8;

__global__ void __launch_bounds__(kStdCols * kStdRows)
k_standardise_f64(const double* __restrict__ Z, int64_t ldz, int N, int M, double* __restrict__ Zt, int64_t ldzt) {
    __shared__ double red_a[kStdRows][kStdCols];
    __shared__ double red_b[kStdRows][kStdCols];
    __shared__ double mean_s[kStdCols], std_s[kStdCols];
    __shared__ double tile[kStdCols][kStdCols + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int j = blockIdx.x * kStdCols + tx;
    const bool col_ok = j < M;

    double sum = 0.0, cnt = 0.0;
    for (int i = ty; i < N; i += kStdRows) {
        double a = col_ok ? Z[static_cast<int64_t>(i) * ldz + j] : 0.0;
        if (!isnan(a)) { sum += a; cnt += 1.0; }
    }
    red_a[ty][tx] = sum;
    red_b[ty][tx] = cnt;
    __syncthreads();
    if (ty == 0) {
        double s = 0.0, c = 0.0;
        for (int r = 0; r < kStdRows; ++r) { s += red_a[r][tx]; c += red_b[r][tx]; }
        mean_s[tx] = s / fmax(c, 1.0);
        red_b[0][tx] = fmax(c, 1.0);
    }
    __syncthreads();
    const double mean = mean_s[tx];
    const double n_nonnan = red_b[0][tx];
    __syncthreads();
    double ss = 0.0;
    for (int i = ty; i < N; i += kStdRows) {
        double a = col_ok ? Z[static_cast<int64_t>(i) * ldz + j] : 0.0;
        if (!isnan(a)) { double d = a - mean; ss += d * d; }
    }
    red_a[ty][tx] = ss;
    __syncthreads();
    if (ty == 0) {
        double s = 0.0;
        for (int r = 0; r < kStdRows; ++r) s += red_a[r][tx];
        double sd = sqrt(s / n_nonnan);
        std_s[tx] = (sd == 0.0) ? INFINITY : sd;
    }
    __syncthreads();
    // one reciprocal per variant and a multiply per element: FP64 division is a multi-instruction sequence on an
    // FP64 pipe with a small fraction of the FP32 rate (the result moves by at most one rounding)
    const double inv_sd = 1.0 / std_s[tx];
    for (int i0 = 0; i0 < N; i0 += kStdCols) {
        for (int r = ty; r < kStdCols; r += kStdRows) {
            int i = i0 + r;
            double v = 0.0;
            if (col_ok && i < N) {
                double a = Z[static_cast<int64_t>(i) * ldz + j];
                v = isnan(a) ? 0.0 : (a - mean) * inv_sd;
            }
            tile[r][tx] = v;  // tile[sample][variant]
        }
        __syncthreads();
        for (int r = ty; r < kStdCols; r += kStdRows) {
            int jj = blockIdx.x * kStdCols + r;  // variant
            int i = i0 + tx;                     // sample
            if (jj < M && i < N) Zt[static_cast<int64_t>(jj) * ldzt + i] = tile[tx][r];
        }
        __syncthreads();
    }
}

// ---- standardiser from int8 dosages (M, N) variant-major -------------------------------------------------------
// One warp per variant: exact integer count / sum / sum of squares, mean = sum / n (the same FP64 division the
// reference does on an exact integer sum), var = (n sumsq - sum^2) / n^2 from exact integers.
__global__ void k_standardise_dosage(const int8_t* __restrict__ Gt, int64_t ldg, int N, int M, double* __restrict__ Zt,
                                     int64_t ldzt) {
    const int lane = threadIdx.x & 31;
    const int64_t m = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    if (m >= M) return;
    const int8_t* g = Gt + m * ldg;
    long long n = 0, s = 0, q = 0;
    for (int i = lane; i < N; i += 32) {
        int v = g[i];
        if (v >= 0) { n += 1; s += v; q += v * v; }
    }
    n = warp_sum_ll(n);
    s = warp_sum_ll(s);
    q = warp_sum_ll(q);
    const long long nn = n > 0 ? n : 1;
    const double mean = static_cast<double>(s) / static_cast<double>(nn);
    const long long v_num = nn * q - s * s;  // n^2 var, exact
    double sd = sqrt(static_cast<double>(v_num)) / static_cast<double>(nn);
    if (sd == 0.0) sd = INFINITY;
    double* z = Zt + m * ldzt;
    for (int i = lane; i < N; i += 32) {
        int v = g[i];
        z[i] = (v >= 0) ? (static_cast<double>(v) - mean) / sd : 0.0;
    }
}

__global__ void k_transpose(const double* __restrict__ A, int64_t lda, int rows, int cols, double* __restrict__ At,
                            int64_t ldat) {
    __shared__ double tile[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += 8) {
        int r = r0 + k, c = c0 + threadIdx.x;
        if (r < rows && c < cols) tile[k][threadIdx.x] = A[static_cast<int64_t>(r) * lda + c];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += 8) {
        int c = c0 + k, r = r0 + threadIdx.x;
        if (r < rows && c < cols) At[static_cast<int64_t>(c) * ldat + r] = tile[threadIdx.x][k];
    }
}

__global__ void k_loco_kinship(const double* __restrict__ Gtot, const double* __restrict__ Gc, int64_t ld, int N,
                               double inv_m, double m_loco, double* __restrict__ K) {
    int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t >= static_cast<int64_t>(N) * N) return;
    int64_t i = t / N, j = t % N;
    double g = Gtot[i * ld + j];
    if (Gc) g -= Gc[i * ld + j];
    K[i * ld + j] = g / m_loco;
    (void)inv_m;
}

// ---- covariate projection of K + I -------------------------------------------------------------------------
// W (N, D): W[i, k] = sum_j (K + I)[i, j] Q[k, j]; one warp per (i, k).
__global__ void k_proj_W(const double* __restrict__ K, int64_t ldk, const double* __restrict__ Q, int N, int D,
                         double* __restrict__ W) {
    const int lane = threadIdx.x & 31;
    const int64_t w = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    if (w >= static_cast<int64_t>(N) * D) return;
    const int i = static_cast<int>(w / D), k = static_cast<int>(w % D);
    const double* krow = K + static_cast<int64_t>(i) * ldk;
    const double* q = Q + static_cast<int64_t>(k) * N;
    double acc = 0.0;
    for (int j = lane; j < N; j += 32) acc += krow[j] * q[j];
    acc = warp_sum(acc);
    if (lane == 0) W[static_cast<int64_t>(i) * D + k] = acc + q[i];
}

// C (D, D) = Q W, then V (N, D) = Q^T C; one block
__global__ void k_proj_C(const double* __restrict__ Q, const double* __restrict__ W, int N, int D,
                         double* __restrict__ C) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int e = warp; e < D * D; e += nw) {
        int k = e / D, l = e % D;
        double acc = 0.0;
        for (int i = lane; i < N; i += 32) acc += Q[static_cast<int64_t>(k) * N + i] * W[static_cast<int64_t>(i) * D + l];
        acc = warp_sum(acc);
        if (lane == 0) C[e] = acc;
    }
}

__global__ void k_proj_V(const double* __restrict__ Q, const double* __restrict__ C, const double* __restrict__ W,
                         int N, int D, double* __restrict__ VmW) {
    int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t >= static_cast<int64_t>(N) * D) return;
    int i = static_cast<int>(t / D), l = static_cast<int>(t % D);
    double acc = 0.0;
    for (int k = 0; k < D; ++k) acc += Q[static_cast<int64_t>(k) * N + i] * C[k * D + l];
    VmW[t] = acc - W[t];  // (Q^T C - W)[i, l]
}

// Kp[i, j] = (K + I)[i, j] - sum_k Q[k, i] W[j, k] + sum_k (V - W)[i, k] Q[k, j]
__global__ void k_proj_apply(const double* __restrict__ K, int64_t ldk, const double* __restrict__ Q,
                             const double* __restrict__ W, const double* __restrict__ VmW, int N, int D,
                             double* __restrict__ Kp, int64_t ldkp) {
    int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t >= static_cast<int64_t>(N) * N) return;
    int i = static_cast<int>(t / N), j = static_cast<int>(t % N);
    double a = K[static_cast<int64_t>(i) * ldk + j] + (i == j ? 1.0 : 0.0);
    double acc = 0.0;
    for (int k = 0; k < D; ++k) {
        const double qki = Q[static_cast<int64_t>(k) * N + i];
        const double qkj = Q[static_cast<int64_t>(k) * N + j];
        acc += VmW[static_cast<int64_t>(i) * D + k] * qkj - qki * W[static_cast<int64_t>(j) * D + k];
    }
    Kp[static_cast<int64_t>(i) * ldkp + j] = a + acc;
}

template <typename T>
__global__ void k_compat_spectrum(const T* __restrict__ evals, int N, int D, double* __restrict__ s) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N - D) return;
    s[i] = fmax(static_cast<double>(evals[D + i]) - 1.0, 0.0);
}

// R[r] = A[r] - X (Xpinv A[r]^T); one warp per row, D <= 64 coefficients held in shared memory per warp
constexpr int kMaxD = 64;
__global__ void k_regress_out(const double* __restrict__ A, int64_t lda, int rows, int N, const double* __restrict__ X,
                              int D, const double* __restrict__ Xpinv, double* __restrict__ R, int64_t ldr) {
    __shared__ double coef[8][kMaxD];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t r = blockIdx.x * static_cast<int64_t>(8) + warp;
    if (r >= rows) return;
    const double* a = A + r * lda;
    for (int d = 0; d < D; ++d) {
        const double* xp = Xpinv + static_cast<int64_t>(d) * N;
        double acc = 0.0;
        for (int i = lane; i < N; i += 32) acc += xp[i] * a[i];
        acc = warp_sum(acc);
        if (lane == 0) coef[warp][d] = acc;
    }
    __syncwarp();
    double* out = R + r * ldr;
    for (int i = lane; i < N; i += 32) {
        double xc = 0.0;
        for (int d = 0; d < D; ++d) xc += X[static_cast<int64_t>(i) * D + d] * coef[warp][d];
        out[i] = a[i] - xc;
    }
}

// torch.linspace's FP64 node values: fma(step, i, lo) below the midpoint, fma(-step, n-1-i, hi) above it
__global__ void k_grid_nodes(double lo, double hi, int n, double* __restrict__ grid) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (n == 1) { grid[0] = lo; return; }
    const double step = (hi - lo) / static_cast<double>(n - 1);
    const int half = n / 2;
    grid[i] = (i < half) ? fma(step, static_cast<double>(i), lo) : fma(-step, static_cast<double>(n - 1 - i), hi);
}

// nullh2 = 1 / (1 + exp(log delta)) broadcast over a chromosome's variant rows.  The FP64 exp is evaluated once per
// column and thread (GB300's FP64 rate is low); each thread then writes its column in kNullh2Rows rows, so the
// stores of a warp are contiguous.
constexpr int kNullh2Rows = 64;

__global__ void k_fill_nullh2(const double* __restrict__ ld, int n_real, const int64_t* __restrict__ rows, int Mc,
                              double* __restrict__ out, int64_t ldo) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_real) return;
    const double h2 = 1.0 / (1.0 + exp(ld[p]));
    for (int64_t m0 = static_cast<int64_t>(blockIdx.y) * kNullh2Rows; m0 < Mc;
         m0 += static_cast<int64_t>(gridDim.y) * kNullh2Rows) {
        const int64_t m1 = m0 + kNullh2Rows < Mc ? m0 + kNullh2Rows : Mc;
        for (int64_t m = m0; m < m1; ++m) out[rows[m] * ldo + p] = h2;
    }
}

__global__ void k_axpy(int64_t n, double alpha, const double* __restrict__ x, double* __restrict__ y) {
    int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t < n) y[t] += alpha * x[t];
}

__global__ void k_pack_perms(const double* __restrict__ Yr, int64_t ldy, int B, int N, const int32_t* __restrict__ ord,
                             int n_perm, double* __restrict__ Ya, int64_t lda) {
    const int64_t rows = static_cast<int64_t>(B) * (1 + n_perm);
    const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t >= rows * N) return;
    const int64_t r = t / N;
    const int n = static_cast<int>(t % N);
    double v;
    if (r < B) {
        v = Yr[r * ldy + n];
    } else {
        const int64_t q = r - B;  // = b * n_perm + j
        const int64_t b = q / n_perm;
        const int src = ord[q * N + n];
        v = (src >= 0 && src < N) ? Yr[b * ldy + src] : NAN;
    }
    Ya[r * lda + n] = v;
}

__global__ void k_fill(double* __restrict__ x, int64_t n, double v) {
    int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t < n) x[t] = v;
}

}  // namespace

extern "C" int flmm_standardise_f64(const double* Z, int64_t ldz, int N, int M, double* Zt, int64_t ldzt,
                                    void* stream) {
    FLMM_REQUIRE(Z && Zt && N > 0 && M >= 0 && ldz >= M && ldzt >= N, "flmm_standardise_f64: bad arguments");
    if (M == 0) return FLMM_OK;
    k_standardise_f64<<<ceil_div(M, kStdCols), dim3(kStdCols, kStdRows), 0, as_stream(stream)>>>(Z, ldz, N, M, Zt,
                                                                                                  ldzt);
    return check_launch("k_standardise_f64");
}

extern "C" int flmm_standardise_dosage(const int8_t* Gt, int64_t ldg, int N, int M, double* Zt, int64_t ldzt,
                                       void* stream) {
    FLMM_REQUIRE(Gt && Zt && N > 0 && M >= 0 && ldg >= N && ldzt >= N, "flmm_standardise_dosage: bad arguments");
    if (M == 0) return FLMM_OK;
    k_standardise_dosage<<<ceil_div(static_cast<int64_t>(M) * 32, 256), 256, 0, as_stream(stream)>>>(Gt, ldg, N, M,
                                                                                                     Zt, ldzt);
    return check_launch("k_standardise_dosage");
}

extern "C" int flmm_transpose_f64(const double* A, int64_t lda, int rows, int cols, double* At, int64_t ldat,
                                  void* stream) {
    FLMM_REQUIRE(A && At && rows >= 0 && cols >= 0 && lda >= cols && ldat >= rows, "flmm_transpose_f64: bad arguments");
    if (rows == 0 || cols == 0) return FLMM_OK;
    dim3 grid(ceil_div(cols, 32), ceil_div(rows, 32));
    k_transpose<<<grid, dim3(32, 8), 0, as_stream(stream)>>>(A, lda, rows, cols, At, ldat);
    return check_launch("k_transpose");
}

extern "C" int flmm_loco_kinship(const double* Gtot, const double* Gc, int64_t ld, int N, double m_loco, double* K,
                                 void* stream) {
    FLMM_REQUIRE(Gtot && K && N > 0 && ld >= N && m_loco > 0, "flmm_loco_kinship: bad arguments");
    int64_t nn = static_cast<int64_t>(N) * N;
    k_loco_kinship<<<ceil_div(nn, 256), 256, 0, as_stream(stream)>>>(Gtot, Gc, ld, N, 1.0 / m_loco, m_loco, K);
    return check_launch("k_loco_kinship");
}

extern "C" int flmm_project_kinship_workspace_bytes(int N, int D, size_t* bytes) {
    FLMM_REQUIRE(bytes && N > 0 && D > 0, "flmm_project_kinship_workspace_bytes: bad arguments");
    *bytes = sizeof(double) * (2 * static_cast<size_t>(N) * D + static_cast<size_t>(D) * D);
    return FLMM_OK;
}

extern "C" int flmm_project_kinship(const double* K, int64_t ldk, const double* Qx, int N, int D, double* Kp,
                                    int64_t ldkp, void* work, size_t work_bytes, void* stream) {
    FLMM_REQUIRE(K && Qx && Kp && work && N > 0 && D > 0 && ldk >= N && ldkp >= N,
                 "flmm_project_kinship: bad arguments");
    size_t need = 0;
    flmm_project_kinship_workspace_bytes(N, D, &need);
    if (work_bytes < need)
        return fail(FLMM_ERR_WORKSPACE, "flmm_project_kinship: need %zu bytes, got %zu", need, work_bytes);
    double* W = static_cast<double*>(work);
    double* VmW = W + static_cast<size_t>(N) * D;
    double* C = VmW + static_cast<size_t>(N) * D;
    cudaStream_t st = as_stream(stream);
    int64_t nd = static_cast<int64_t>(N) * D;
    int rc;
    k_proj_W<<<ceil_div(nd * 32, 256), 256, 0, st>>>(K, ldk, Qx, N, D, W);
    if ((rc = check_launch("k_proj_W"))) return rc;
    k_proj_C<<<1, 512, 0, st>>>(Qx, W, N, D, C);
    if ((rc = check_launch("k_proj_C"))) return rc;
    k_proj_V<<<ceil_div(nd, 256), 256, 0, st>>>(Qx, C, W, N, D, VmW);
    if ((rc = check_launch("k_proj_V"))) return rc;
    k_proj_apply<<<ceil_div(static_cast<int64_t>(N) * N, 256), 256, 0, st>>>(K, ldk, Qx, W, VmW, N, D, Kp, ldkp);
    return check_launch("k_proj_apply");
}

extern "C" int flmm_compat_spectrum(const double* evals, int N, int D, double* s, void* stream) {
    FLMM_REQUIRE(evals && s && N > D && D >= 0, "flmm_compat_spectrum: need N > D");
    k_compat_spectrum<double><<<ceil_div(N - D, 256), 256, 0, as_stream(stream)>>>(evals, N, D, s);
    return check_launch("k_compat_spectrum");
}

extern "C" int flmm_compat_spectrum_f32(const float* evals, int N, int D, double* s, void* stream) {
    FLMM_REQUIRE(evals && s && N > D && D >= 0, "flmm_compat_spectrum_f32: need N > D");
    k_compat_spectrum<float><<<ceil_div(N - D, 256), 256, 0, as_stream(stream)>>>(evals, N, D, s);
    return check_launch("k_compat_spectrum");
}

extern "C" int flmm_regress_out(const double* A, int64_t lda, int rows, int N, const double* X, int D,
                                const double* Xpinv, double* R, int64_t ldr, void* stream) {
    FLMM_REQUIRE(A && X && Xpinv && R && N > 0 && D > 0 && D <= kMaxD && lda >= N && ldr >= N,
                 "flmm_regress_out: bad arguments (D must be in 1..%d)", kMaxD);
    if (rows <= 0) return FLMM_OK;
    k_regress_out<<<ceil_div(rows, 8), 256, 0, as_stream(stream)>>>(A, lda, rows, N, X, D, Xpinv, R, ldr);
    return check_launch("k_regress_out");
}

extern "C" int flmm_delta_grid_nodes(double lo, double hi, int n_grid, double* grid, void* stream) {
    FLMM_REQUIRE(grid && n_grid > 0, "flmm_delta_grid_nodes: bad arguments");
    k_grid_nodes<<<ceil_div(n_grid, 256), 256, 0, as_stream(stream)>>>(lo, hi, n_grid, grid);
    return check_launch("k_grid_nodes");
}

extern "C" int flmm_fill_nullh2(const double* log_delta, int n_real, const int64_t* rows, int Mc, double* nullh2,
                                int64_t ldo, void* stream) {
    FLMM_REQUIRE(log_delta && rows && nullh2 && ldo >= n_real, "flmm_fill_nullh2: bad arguments");
    if (n_real <= 0 || Mc <= 0) return FLMM_OK;
    const int64_t row_blocks = ceil_div(static_cast<int64_t>(Mc), kNullh2Rows);
    const dim3 grid(static_cast<unsigned>(ceil_div(n_real, 128)),
                    static_cast<unsigned>(row_blocks < 65535 ? row_blocks : 65535));
    k_fill_nullh2<<<grid, 128, 0, as_stream(stream)>>>(log_delta, n_real, rows, Mc, nullh2, ldo);
    return check_launch("k_fill_nullh2");
}

extern "C" int flmm_fill_f64(double* x, int64_t n, double value, void* stream) {
    FLMM_REQUIRE(x || n == 0, "flmm_fill_f64: bad arguments");
    if (n == 0) return FLMM_OK;
    k_fill<<<ceil_div(n, 256), 256, 0, as_stream(stream)>>>(x, n, value);
    return check_launch("k_fill");
}

extern "C" int flmm_axpy_f64(int64_t n, double alpha, const double* x, double* y, void* stream) {
    FLMM_REQUIRE((x && y) || n == 0, "flmm_axpy_f64: NULL argument");
    if (n == 0) return FLMM_OK;
    k_axpy<<<ceil_div(n, 256), 256, 0, as_stream(stream)>>>(n, alpha, x, y);
    return check_launch("k_axpy");
}

extern "C" int flmm_pack_perm_columns(const double* Yt_real, int64_t ldy, int B, int N, const int32_t* orders,
                                      int n_perm, double* Yt_all, int64_t lda, void* stream) {
    FLMM_REQUIRE(Yt_real && Yt_all && B >= 0 && N > 0 && n_perm >= 0 && ldy >= N && lda >= N,
                 "flmm_pack_perm_columns: bad arguments");
    FLMM_REQUIRE(n_perm == 0 || B == 0 || orders, "flmm_pack_perm_columns: orders is NULL");
    const int64_t total = static_cast<int64_t>(B) * (1 + n_perm) * N;
    if (total == 0) return FLMM_OK;
    k_pack_perms<<<ceil_div(total, 256), 256, 0, as_stream(stream)>>>(Yt_real, ldy, B, N, orders, n_perm, Yt_all, lda);
    return check_launch("k_pack_perms");
}

namespace {

__global__ void k_f64_to_f32(int64_t n, const double* __restrict__ x, float* __restrict__ y) {
    int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t < n) y[t] = static_cast<float>(x[t]);
}

__global__ void k_acc_f32_f64(int64_t n, const float* __restrict__ x, double* __restrict__ y) {
    int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t < n) y[t] += static_cast<double>(x[t]);
}

__global__ void k_loco_kinship_f32(const double* __restrict__ Gtot, const float* __restrict__ Gc, int64_t nn,
                                   double m_loco, double* __restrict__ K) {
    int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t < nn) K[t] = (Gtot[t] - (Gc ? static_cast<double>(Gc[t]) : 0.0)) / m_loco;
}

}  // namespace

// out[r] = sum_c A[r, c]^2, one warp per row
__global__ void k_row_sumsq(const double* __restrict__ A, int64_t lda, int rows, int cols, double* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t r = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    if (r >= rows) return;
    double acc = 0.0;
    for (int c = lane; c < cols; c += 32) acc = fma(A[r * lda + c], A[r * lda + c], acc);
    acc = warp_sum(acc);
    if (lane == 0) out[r] = acc;
}

extern "C" int flmm_row_sumsq_f64(const double* A, int64_t lda, int rows, int cols, double* out, void* stream) {
    FLMM_REQUIRE((A && out && lda >= cols && cols >= 0) || rows == 0, "flmm_row_sumsq_f64: bad arguments");
    if (rows == 0) return FLMM_OK;
    k_row_sumsq<<<ceil_div(static_cast<int64_t>(rows) * 32, 256), 256, 0, as_stream(stream)>>>(A, lda, rows, cols, out);
    return check_launch("k_row_sumsq");
}

extern "C" int flmm_convert_f64_f32(int64_t n, const double* x, float* y, void* stream) {
    FLMM_REQUIRE((x && y) || n == 0, "flmm_convert_f64_f32: NULL argument");
    if (n == 0) return FLMM_OK;
    k_f64_to_f32<<<ceil_div(n, 256), 256, 0, as_stream(stream)>>>(n, x, y);
    return check_launch("k_f64_to_f32");
}

extern "C" int flmm_accumulate_f32_f64(int64_t n, const float* x, double* y, void* stream) {
    FLMM_REQUIRE((x && y) || n == 0, "flmm_accumulate_f32_f64: NULL argument");
    if (n == 0) return FLMM_OK;
    k_acc_f32_f64<<<ceil_div(n, 256), 256, 0, as_stream(stream)>>>(n, x, y);
    return check_launch("k_acc_f32_f64");
}

extern "C" int flmm_loco_kinship_f32(const double* Gtot, const float* Gc, int N, double m_loco, double* K,
                                     void* stream) {
    FLMM_REQUIRE(Gtot && K && N > 0 && m_loco > 0, "flmm_loco_kinship_f32: bad arguments");
    const int64_t nn = static_cast<int64_t>(N) * N;
    k_loco_kinship_f32<<<ceil_div(nn, 256), 256, 0, as_stream(stream)>>>(Gtot, Gc, nn, m_loco, K);
    return check_launch("k_loco_kinship_f32");
}
