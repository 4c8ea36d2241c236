// Plain GLS form of the scan (fasterlmm/core.py:89-375), in FP64: the covariates stay in the model, so every
// delta needs the (C, C) Gram A = X~^T W X~ and its Cholesky, and every test carries the quadratic form
// B^T A^-1 B with B = X~^T W s.
//
//   * grid losses: A_g, its Cholesky and log det once per grid node (k_gls_grid_prep); per (node, column) the
//     weighted products u = X~^T W y and yWy (k_gls_grid_loss); first argmin per column (k_gls_argmin);
//   * per-column evaluations (golden section, the per-phenotype loss): one warp forms the Gram of the augmented
//     columns [X~ | y] at the column's own delta in a few passes over the samples, then one lane factors it;
//   * Wald: per column the null fit (A, beta_x, r, rWr) and the left operands w o r, w o x_c, w (k_gls_wald_prep),
//     then a tiled kernel accumulates num = (w o r)^T s, B_c = (w o x_c)^T s and sWs = w^T (s o s) per (column,
//     variant) and runs the reference's epilogue (k_gls_wald).
// Loss formulas and golden-section updates use non-contracting FP64 intrinsics in the reference's order; sums over
// samples are warp / tile sums, so refined log delta agrees with the reference to its FP64 noise.
#include <math.h>

#include "flmm_common.cuh"

using namespace flmm;

namespace {

constexpr int kMaxGlsC = 30;                       // covariate columns supported by the GLS kernels
constexpr double kLog2Pi = 1.8378770664093453;     // log(2 pi) in FP64
constexpr int kPairChunk = 8;                      // weighted products accumulated per pass over the samples
constexpr int kEvalWarps = 4;                      // warps per block of the per-column evaluation kernels

// -2 log L from yWy, uAu, sum log(s + delta) and log det A (fasterlmm/core.py:180-186 / 216-222)
__device__ double gls_loss(double yWy, double uAu, double sum_log_sd, double logdet_a, int N, int C, bool reml) {
    const double rWr = fmax(add_rn(yWy, -uAu), kPosFloor);
    if (reml) {
        const double nc = static_cast<double>(N - C);
        const double t = add_rn(add_rn(kLog2Pi, log(rWr / nc)), 1.0);
        return add_rn(add_rn(mul_rn(nc, t), sum_log_sd), logdet_a);
    }
    const double n = static_cast<double>(N);
    const double t = add_rn(add_rn(kLog2Pi, log(rWr / n)), 1.0);
    return add_rn(mul_rn(n, t), sum_log_sd);
}

// In-place lower Cholesky of the row-major (C, C) matrix A (lower triangle read).  False when a pivot is not
// positive, where torch.linalg.cholesky_ex reports info > 0; the caller then uses the identity, as the reference does.
__device__ bool chol_lower(double* A, int C) {
    for (int j = 0; j < C; ++j) {
        double d = A[j * C + j];
        for (int k = 0; k < j; ++k) d -= A[j * C + k] * A[j * C + k];
        if (!(d > 0.0)) return false;
        d = sqrt(d);
        A[j * C + j] = d;
        for (int i = j + 1; i < C; ++i) {
            double v = A[i * C + j];
            for (int k = 0; k < j; ++k) v -= A[i * C + k] * A[j * C + k];
            A[i * C + j] = v / d;
        }
    }
    for (int i = 0; i < C; ++i)
        for (int j = i + 1; j < C; ++j) A[i * C + j] = 0.0;
    return true;
}

__device__ void set_identity(double* A, int C) {
    for (int i = 0; i < C; ++i)
        for (int j = 0; j < C; ++j) A[i * C + j] = (i == j) ? 1.0 : 0.0;
}

// z = L^-1 b in place (forward substitution), L row-major lower
__device__ void forward_solve(const double* L, int C, double* z) {
    for (int i = 0; i < C; ++i) {
        double v = z[i];
        for (int k = 0; k < i; ++k) v -= L[i * C + k] * z[k];
        z[i] = v / L[i * C + i];
    }
}

// x = L^-T z in place (back substitution)
__device__ void back_solve(const double* L, int C, double* x) {
    for (int i = C - 1; i >= 0; --i) {
        double v = x[i];
        for (int k = i + 1; k < C; ++k) v -= L[k * C + i] * x[k];
        x[i] = v / L[i * C + i];
    }
}

// Weighted Gram of the augmented columns a_0..a_C = (x~_0 .. x~_{C-1}, y) at one delta, by one warp:
// Gs[i * (C + 1) + j] = sum_n a_i[n] a_j[n] / (s[n] + delta) for j <= i.  Returns sum_n log(s[n] + delta).
__device__ double warp_gram(const double* __restrict__ s, int N, const double* __restrict__ Xrt, int64_t ldx, int C,
                            const double* __restrict__ y, double delta, double* Gs) {
    const int lane = threadIdx.x & 31;
    const int K = C + 1;
    const int pairs = K * (K + 1) / 2;
    double sl = 0.0;
    int i0 = 0, j0 = 0;  // pair at the start of the chunk
    for (int q0 = 0; q0 < pairs; q0 += kPairChunk) {
        int pi[kPairChunk], pj[kPairChunk];
        int i = i0, j = j0;
#pragma unroll
        for (int k = 0; k < kPairChunk; ++k) {
            pi[k] = i;
            pj[k] = j;
            if (j < i) { ++j; } else { ++i; j = 0; }
        }
        i0 = i;
        j0 = j;
        double acc[kPairChunk] = {};
        for (int n = lane; n < N; n += 32) {
            const double sd = s[n] + delta;
            const double w = 1.0 / sd;
            if (q0 == 0) sl += log(sd);
#pragma unroll
            for (int k = 0; k < kPairChunk; ++k) {
                if (q0 + k < pairs) {
                    const double ai = pi[k] < C ? Xrt[pi[k] * ldx + n] : y[n];
                    const double aj = pj[k] < C ? Xrt[pj[k] * ldx + n] : y[n];
                    acc[k] += mul_rn(mul_rn(w, ai), aj);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < kPairChunk; ++k) {
            const double v = warp_sum(acc[k]);
            if (lane == 0 && q0 + k < pairs) Gs[pi[k] * K + pj[k]] = v;
        }
    }
    __syncwarp();
    return warp_sum(sl);
}

// One column's -2 log L at its own delta (fasterlmm/core.py:190-224), by one warp; A is per-warp scratch (C * C)
// and z (C).  The result is valid in lane 0.
__device__ double warp_pheno_loss(const double* __restrict__ s, int N, const double* __restrict__ Xrt, int64_t ldx,
                                  int C, const double* __restrict__ y, double ld, bool reml, double* Gs, double* A,
                                  double* z) {
    const int lane = threadIdx.x & 31;
    const double sum_log = warp_gram(s, N, Xrt, ldx, C, y, exp(ld), Gs);
    double loss = 0.0;
    if (lane == 0) {
        const int K = C + 1;
        for (int i = 0; i < C; ++i) {
            for (int j = 0; j <= i; ++j) A[i * C + j] = Gs[i * K + j];
            z[i] = Gs[C * K + i];
        }
        const bool ok = chol_lower(A, C);
        if (!ok) set_identity(A, C);
        double logdet = 0.0;
        for (int i = 0; i < C; ++i) logdet += log(A[i * C + i]);
        logdet = 2.0 * logdet;
        forward_solve(A, C, z);
        double uAu = 0.0;
        for (int i = 0; i < C; ++i) uAu += z[i] * z[i];
        loss = ok ? gls_loss(Gs[C * K + C], uAu, sum_log, logdet, N, C, reml) : INFINITY;
    }
    __syncwarp();
    return __shfl_sync(0xffffffffu, loss, 0);
}

// ---- grid ----------------------------------------------------------------------------------------------------

// Per grid node g (one block): W[g, n] = 1 / (s[n] + delta_g), sum log(s + delta_g), A_g, its Cholesky L_g (identity
// and bad[g] = 1 when it fails) and log det A_g.
__global__ void k_gls_grid_prep(const double* __restrict__ s, int N, const double* __restrict__ Xrt, int64_t ldx,
                                int C, const double* __restrict__ grid, double* __restrict__ W,
                                double* __restrict__ sum_log, double* __restrict__ Lg, double* __restrict__ logdet,
                                int32_t* __restrict__ bad) {
    __shared__ double A[kMaxGlsC * kMaxGlsC];
    __shared__ double red[32];
    const int g = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const double delta = exp(grid[g]);
    double sl = 0.0;
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        const double sd = s[n] + delta;
        W[static_cast<int64_t>(g) * N + n] = 1.0 / sd;
        sl += log(sd);
    }
    sl = warp_sum(sl);
    if (lane == 0) red[warp] = sl;
    __syncthreads();  // W row complete
    const double* w = W + static_cast<int64_t>(g) * N;
    const int pairs = C * (C + 1) / 2;
    for (int q = warp; q < pairs; q += nwarps) {
        int i = 0, r = q;
        while (r > i) { r -= i + 1; ++i; }
        const int j = r;
        double acc = 0.0;
        for (int n = lane; n < N; n += 32) acc += mul_rn(mul_rn(w[n], Xrt[i * ldx + n]), Xrt[j * ldx + n]);
        acc = warp_sum(acc);
        if (lane == 0) A[i * C + j] = acc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < nwarps; ++k) t += red[k];
        sum_log[g] = t;
        const bool ok = chol_lower(A, C);
        if (!ok) set_identity(A, C);
        double ld = 0.0;
        for (int i = 0; i < C; ++i) ld += log(A[i * C + i]);
        logdet[g] = 2.0 * ld;
        bad[g] = ok ? 0 : 1;
        double* L = Lg + static_cast<int64_t>(g) * C * C;
        for (int i = 0; i < C * C; ++i) L[i] = A[i];
    }
}

// loss[g, p] (fasterlmm/core.py:148-187): one warp per (g, column), u_c = sum_n W[g, n] x~_c[n] y[n] in chunks
__global__ void k_gls_grid_loss(const double* __restrict__ W, const double* __restrict__ Xrt, int64_t ldx, int C,
                                const double* __restrict__ Yrt, int64_t ldy, int N, int P,
                                const double* __restrict__ sum_log, const double* __restrict__ Lg,
                                const double* __restrict__ logdet, const int32_t* __restrict__ bad, int reml,
                                double* __restrict__ loss) {
    __shared__ double zs[kEvalWarps][kMaxGlsC + 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = blockIdx.y;
    const int64_t p = static_cast<int64_t>(blockIdx.x) * kEvalWarps + warp;
    if (p >= P) return;
    const double* w = W + static_cast<int64_t>(g) * N;
    const double* y = Yrt + p * ldy;
    double* z = zs[warp];
    for (int c0 = 0; c0 <= C; c0 += kPairChunk) {
        double acc[kPairChunk] = {};
        for (int n = lane; n < N; n += 32) {
            const double yy = mul_rn(y[n], y[n]);  // yWy = w @ (Y o Y), fasterlmm/core.py:177
#pragma unroll
            for (int k = 0; k < kPairChunk; ++k) {
                const int c = c0 + k;
                if (c < C) acc[k] += mul_rn(mul_rn(w[n], Xrt[c * ldx + n]), y[n]);
                else if (c == C) acc[k] += mul_rn(w[n], yy);
            }
        }
#pragma unroll
        for (int k = 0; k < kPairChunk; ++k) {
            const double v = warp_sum(acc[k]);
            if (lane == 0 && c0 + k <= C) z[c0 + k] = v;
        }
    }
    __syncwarp();
    if (lane == 0) {
        const double yWy = z[C];
        forward_solve(Lg + static_cast<int64_t>(g) * C * C, C, z);
        double uAu = 0.0;
        for (int i = 0; i < C; ++i) uAu += z[i] * z[i];
        loss[static_cast<int64_t>(g) * P + p] =
            bad[g] ? INFINITY : gls_loss(yWy, uAu, sum_log[g], logdet[g], N, C, reml != 0);
    }
}

// first argmin over g of loss (G, P), as torch.argmin
__global__ void k_gls_argmin(const double* __restrict__ loss, int G, int P, int32_t* __restrict__ idx) {
    const int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (p >= P) return;
    double best = loss[p];
    int bi = 0;
    for (int g = 1; g < G; ++g) {
        const double v = loss[static_cast<int64_t>(g) * P + p];
        if (v < best) { best = v; bi = g; }
    }
    idx[p] = bi;
}

// ---- per-column evaluations -----------------------------------------------------------------------------------

__device__ __forceinline__ size_t eval_smem_doubles(int C) {
    return static_cast<size_t>(C + 1) * (C + 1) + static_cast<size_t>(C) * C + (C + 1);
}

// loss[p] at log_delta[p], one warp per column
__global__ void k_gls_pheno_loss(const double* __restrict__ s, int N, const double* __restrict__ Xrt, int64_t ldx,
                                 int C, const double* __restrict__ Yrt, int64_t ldy, int P,
                                 const double* __restrict__ ld, int reml, double* __restrict__ loss) {
    extern __shared__ double sm[];
    const int warp = threadIdx.x >> 5;
    const int64_t p = static_cast<int64_t>(blockIdx.x) * kEvalWarps + warp;
    if (p >= P) return;
    double* Gs = sm + warp * eval_smem_doubles(C);
    double* A = Gs + (C + 1) * (C + 1);
    double* z = A + C * C;
    const double v = warp_pheno_loss(s, N, Xrt, ldx, C, Yrt + p * ldy, ld[p], reml != 0, Gs, A, z);
    if ((threadIdx.x & 31) == 0) loss[p] = v;
}

// golden-section search on [grid[i-1], grid[i+1]], one warp per column (fasterlmm/core.py:245-264)
__global__ void k_gls_golden(const double* __restrict__ s, int N, const double* __restrict__ Xrt, int64_t ldx, int C,
                             const double* __restrict__ Yrt, int64_t ldy, int P, const double* __restrict__ grid,
                             int G, const int32_t* __restrict__ idx, int refine, int reml, double lo, double hi,
                             double* __restrict__ log_delta) {
    extern __shared__ double sm[];
    const int warp = threadIdx.x >> 5;
    const int64_t p = static_cast<int64_t>(blockIdx.x) * kEvalWarps + warp;
    if (p >= P) return;
    const int i = idx[p];
    if (!refine) {
        if ((threadIdx.x & 31) == 0) log_delta[p] = grid[i];
        return;
    }
    double* Gs = sm + warp * eval_smem_doubles(C);
    double* A = Gs + (C + 1) * (C + 1);
    double* z = A + C * C;
    const double* y = Yrt + p * ldy;
    const bool rm = reml != 0;
    double a = grid[max(i - 1, 0)], b = grid[min(i + 1, G - 1)];
    const double inv_phi = 2.0 / (1.0 + sqrt(5.0));
    const double inv_phi2 = mul_rn(inv_phi, inv_phi);
    double c = add_rn(a, mul_rn(inv_phi2, add_rn(b, -a)));
    double d = add_rn(a, mul_rn(inv_phi, add_rn(b, -a)));
    double fc = warp_pheno_loss(s, N, Xrt, ldx, C, y, c, rm, Gs, A, z);
    double fd = warp_pheno_loss(s, N, Xrt, ldx, C, y, d, rm, Gs, A, z);
    for (int it = 0; it < 50; ++it) {
        const bool cond = fc < fd;
        b = cond ? d : b;
        a = cond ? a : c;
        c = add_rn(a, mul_rn(inv_phi2, add_rn(b, -a)));
        d = add_rn(a, mul_rn(inv_phi, add_rn(b, -a)));
        fc = warp_pheno_loss(s, N, Xrt, ldx, C, y, c, rm, Gs, A, z);
        fd = warp_pheno_loss(s, N, Xrt, ldx, C, y, d, rm, Gs, A, z);
    }
    if ((threadIdx.x & 31) == 0) log_delta[p] = fmin(fmax(mul_rn(0.5, add_rn(a, b)), lo), hi);
}

// ---- Wald ------------------------------------------------------------------------------------------------------

// Null fit of column p at its log delta (fasterlmm/core.py:328-341): A_p, L_p (identity when the Cholesky fails),
// beta_x = A^-1 u, r = y~ - X~ beta_x, rWr = sum w r^2, and the left operands of the scan
// Lv[p] = (w o r, w o x~_0 .. w o x~_{C-1}, w), each of N entries.
__global__ void k_gls_wald_prep(const double* __restrict__ s, int N, const double* __restrict__ Xrt, int64_t ldx,
                                int C, const double* __restrict__ Yrt, int64_t ldy, int P,
                                const double* __restrict__ ld, double* __restrict__ Lv, double* __restrict__ Lp,
                                double* __restrict__ rWr) {
    extern __shared__ double sm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t p = static_cast<int64_t>(blockIdx.x) * kEvalWarps + warp;
    if (p >= P) return;
    double* Gs = sm + warp * eval_smem_doubles(C);
    double* A = Gs + (C + 1) * (C + 1);
    double* z = A + C * C;
    const double* y = Yrt + p * ldy;
    const double delta = exp(ld[p]);
    warp_gram(s, N, Xrt, ldx, C, y, delta, Gs);
    if (lane == 0) {
        const int K = C + 1;
        for (int i = 0; i < C; ++i) {
            for (int j = 0; j <= i; ++j) A[i * C + j] = Gs[i * K + j];
            z[i] = Gs[C * K + i];
        }
        if (!chol_lower(A, C)) set_identity(A, C);
        forward_solve(A, C, z);
        back_solve(A, C, z);  // z = beta_x
        double* L = Lp + p * C * C;
        for (int i = 0; i < C * C; ++i) L[i] = A[i];
    }
    __syncwarp();
    double* lv = Lv + p * static_cast<int64_t>(C + 2) * N;
    double acc = 0.0;
    for (int n = lane; n < N; n += 32) {
        const double w = 1.0 / (s[n] + delta);
        double fit = 0.0;
        for (int c = 0; c < C; ++c) fit = fma(Xrt[c * ldx + n], z[c], fit);
        const double r = add_rn(y[n], -fit);
        const double wr = mul_rn(w, r);
        acc += mul_rn(wr, r);
        lv[n] = wr;
        for (int c = 0; c < C; ++c) lv[static_cast<int64_t>(1 + c) * N + n] = mul_rn(w, Xrt[c * ldx + n]);
        lv[static_cast<int64_t>(C + 1) * N + n] = w;
    }
    acc = warp_sum(acc);
    if (lane == 0) rWr[p] = acc;
}

constexpr int WP = 16, WM = 16, WK = 8, WT = 256;

// Tile of 16 columns x 16 variants, thread = one (column, variant): num, B_0..B_{C-1} in acc[0..C] and sWs in
// acc[KOPS - 1], accumulated over the samples in chunks of 8, then fasterlmm/core.py:346-371 on the sums.
// KOPS >= C + 2 is the register budget (8, 16 or 32 operands).
template <int KOPS>
__global__ void __launch_bounds__(WT)
k_gls_wald(const double* __restrict__ Lv, const double* __restrict__ Lp, const double* __restrict__ rWr, int N,
           int C, int P, int n_real, const double* __restrict__ Srt, int64_t lds, int M,
           const int64_t* __restrict__ rows, double* __restrict__ f, double* __restrict__ beta, double* __restrict__ se,
           double* __restrict__ sfve, int64_t ldo, double* __restrict__ max_F) {
    extern __shared__ double sm[];
    const int nops = C + 2;
    double* Ls = sm;                                   // [WP][nops][WK]
    double* Ss = Ls + WP * nops * WK;                  // [WM][WK]
    const int tid = threadIdx.x;
    const int pi = tid >> 4, mi = tid & 15;            // 16 consecutive threads share a column
    const int p0 = blockIdx.y * WP, m0 = blockIdx.x * WM;
    const int p = p0 + pi, m = m0 + mi;
    double acc[KOPS];
#pragma unroll
    for (int k = 0; k < KOPS; ++k) acc[k] = 0.0;
    for (int n0 = 0; n0 < N; n0 += WK) {
        for (int t = tid; t < WP * nops * WK; t += WT) {
            const int q = t / (nops * WK), rem = t % (nops * WK), op = rem / WK, k = rem % WK;
            const int gp = p0 + q, gn = n0 + k;
            Ls[t] = (gp < P && gn < N) ? Lv[(static_cast<int64_t>(gp) * nops + op) * N + gn] : 0.0;
        }
        for (int t = tid; t < WM * WK; t += WT) {
            const int q = t / WK, k = t % WK;
            const int gm = m0 + q, gn = n0 + k;
            Ss[t] = (gm < M && gn < N) ? Srt[static_cast<int64_t>(gm) * lds + gn] : 0.0;
        }
        __syncthreads();
        const double* lrow = Ls + pi * nops * WK;
        const double* srow = Ss + mi * WK;
#pragma unroll
        for (int k = 0; k < WK; ++k) {
            const double sv = srow[k];
#pragma unroll
            for (int op = 0; op < KOPS - 1; ++op)
                if (op < C + 1) acc[op] = fma(lrow[op * WK + k], sv, acc[op]);
            acc[KOPS - 1] = fma(lrow[(C + 1) * WK + k], mul_rn(sv, sv), acc[KOPS - 1]);
        }
        __syncthreads();
    }
    double F = -INFINITY;
    if (p < P && m < M) {
        // quad = B^T A^-1 B = |L^-1 B|^2
        const double* L = Lp + static_cast<int64_t>(p) * C * C;
        double quad = 0.0;
#pragma unroll
        for (int i = 0; i < KOPS - 2; ++i) {
            if (i < C) {
                double v = acc[1 + i];
#pragma unroll
                for (int k = 0; k < KOPS - 2; ++k)
                    if (k < i) v -= L[i * C + k] * acc[1 + k];
                v = v / L[i * C + i];
                acc[1 + i] = v;
                quad += v * v;
            }
        }
        const double num = acc[0];
        const double denom = fmax(add_rn(acc[KOPS - 1], -quad), kPosFloor);
        const double b = num / denom;
        const double q = mul_rn(num, num);
        const double rwr = rWr[p];
        const double rss = fmax(add_rn(rwr, -(q / denom)), kPosFloor);
        const double var_b = (rss / static_cast<double>(N - C - 1)) / denom;
        F = mul_rn(b, b) / var_b;
        if (p < n_real) {
            const int64_t o = rows[m] * ldo + p;
            f[o] = F;
            beta[o] = b;
            se[o] = sqrt(var_b);
            sfve[o] = sqrt(fmax(q / mul_rn(denom, rwr), 0.0));
        }
    }
    // column max over this tile's 16 variants (a half-warp), NaN kept
    bool nan_f = isnan(F);
    double v = nan_f ? -INFINITY : F;
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) {
        v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
        nan_f |= __shfl_xor_sync(0xffffffffu, static_cast<int>(nan_f), o) != 0;
    }
    if (mi == 0 && p < P) {
        if (nan_f) v = NAN;
        if (v >= 0.0 || isnan(v)) atomic_max_nonneg(max_F + p, v);
    }
}

// Workspace of the grid stage: grid nodes, W (G, N), sum log, log det, L_g (G, C, C), bad (G), loss (G, P)
struct GridWs {
    double *grid, *W, *sum_log, *logdet, *Lg, *loss;
    int32_t* bad;
    size_t bytes;
};

GridWs carve_grid(void* base, int N, int C, int P, int G) {
    GridWs w{};
    size_t off = 0;
    const uintptr_t b = reinterpret_cast<uintptr_t>(base);
    auto take = [&](size_t nbytes) {
        const uintptr_t p = b + off;
        off += (nbytes + 255) / 256 * 256;
        return p;
    };
    w.grid = reinterpret_cast<double*>(take(sizeof(double) * G));  // (addresses only when base is non-null)
    w.W = reinterpret_cast<double*>(take(sizeof(double) * static_cast<size_t>(G) * N));
    w.sum_log = reinterpret_cast<double*>(take(sizeof(double) * G));
    w.logdet = reinterpret_cast<double*>(take(sizeof(double) * G));
    w.Lg = reinterpret_cast<double*>(take(sizeof(double) * static_cast<size_t>(G) * C * C));
    w.bad = reinterpret_cast<int32_t*>(take(sizeof(int32_t) * G));
    w.loss = reinterpret_cast<double*>(take(sizeof(double) * static_cast<size_t>(G) * P));
    w.bytes = off;
    return w;
}

constexpr int kWaldChunk = 4096;  // columns prepared per pass of the Wald scan

size_t wald_ws(int N, int C, int P) {
    const size_t pc = static_cast<size_t>(P < kWaldChunk ? P : kWaldChunk);
    return sizeof(double) * (pc * (C + 2) * N + pc * C * C + pc) + 1024;
}

__global__ void k_shift_diagonal(double* __restrict__ A, int N, int64_t lda, double v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) A[static_cast<int64_t>(i) * lda + i] += v;
}

__global__ void k_clamp_nonneg(const double* __restrict__ x, int64_t n, double* __restrict__ y) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i < n) y[i] = fmax(x[i], 0.0);
}

size_t eval_smem_bytes(int C) {
    return sizeof(double) * kEvalWarps *
           (static_cast<size_t>(C + 1) * (C + 1) + static_cast<size_t>(C) * C + (C + 1));
}

int check_c(int C, const char* fn) {
    if (C < 1 || C > kMaxGlsC) return fail(FLMM_ERR_ARG, "%s: covariate columns must be in 1..%d", fn, kMaxGlsC);
    return FLMM_OK;
}

}  // namespace

extern "C" int flmm_gls_loss_workspace_bytes(int N, int C, int P, int n_ld, size_t* bytes) {
    FLMM_REQUIRE(bytes && N > 0 && C > 0 && P >= 0 && n_ld > 0, "flmm_gls_loss_workspace_bytes: bad arguments");
    *bytes = carve_grid(nullptr, N, C, P, n_ld).bytes;
    return FLMM_OK;
}

extern "C" int flmm_gls_loss_f64(const double* s, int N, const double* Xrt, int64_t ldx, int C, const double* Yrt,
                                 int64_t ldy, int P, const double* log_delta, int n_ld, int per_column, int reml,
                                 double* loss, void* work, size_t work_bytes, void* stream) {
    FLMM_REQUIRE(s && Xrt && Yrt && log_delta && loss && N > C && ldx >= N && ldy >= N && P >= 0 && n_ld > 0,
                 "flmm_gls_loss_f64: bad arguments");
    int rc = check_c(C, "flmm_gls_loss_f64");
    if (rc) return rc;
    if (P == 0) return FLMM_OK;
    cudaStream_t st = as_stream(stream);
    const size_t smem = eval_smem_bytes(C);
    if (per_column) {
        FLMM_REQUIRE(n_ld == P, "flmm_gls_loss_f64: per-column mode needs one log delta per column");
        if (smem > 48 * 1024)
            FLMM_CUDA(cudaFuncSetAttribute(k_gls_pheno_loss, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_gls_pheno_loss<<<ceil_div(P, kEvalWarps), 32 * kEvalWarps, smem, st>>>(s, N, Xrt, ldx, C, Yrt, ldy, P,
                                                                                  log_delta, reml, loss);
        return check_launch("k_gls_pheno_loss");
    }
    FLMM_REQUIRE(work, "flmm_gls_loss_f64: grid mode needs a workspace");
    GridWs ws = carve_grid(work, N, C, P, n_ld);
    if (work_bytes < ws.bytes)
        return fail(FLMM_ERR_WORKSPACE, "flmm_gls_loss_f64: need %zu bytes, got %zu", ws.bytes, work_bytes);
    k_gls_grid_prep<<<n_ld, 256, 0, st>>>(s, N, Xrt, ldx, C, log_delta, ws.W, ws.sum_log, ws.Lg, ws.logdet, ws.bad);
    if ((rc = check_launch("k_gls_grid_prep"))) return rc;
    dim3 grid(ceil_div(P, kEvalWarps), n_ld);
    k_gls_grid_loss<<<grid, 32 * kEvalWarps, 0, st>>>(ws.W, Xrt, ldx, C, Yrt, ldy, N, P, ws.sum_log, ws.Lg, ws.logdet,
                                                       ws.bad, reml, loss);
    return check_launch("k_gls_grid_loss");
}

extern "C" int flmm_fit_delta_gls_workspace_bytes(int N, int C, int P, int n_grid, size_t* bytes) {
    FLMM_REQUIRE(bytes && N > 0 && C > 0 && P >= 0 && n_grid > 0, "flmm_fit_delta_gls_workspace_bytes: bad arguments");
    *bytes = carve_grid(nullptr, N, C, P, n_grid).bytes;
    return FLMM_OK;
}

extern "C" int flmm_fit_delta_gls_f64(const double* s, int N, const double* Xrt, int64_t ldx, int C,
                                      const double* Yrt, int64_t ldy, int P, int n_grid, double lo, double hi,
                                      int refine, int reml, double* log_delta, int32_t* grid_idx, void* work,
                                      size_t work_bytes, void* stream) {
    FLMM_REQUIRE(s && Xrt && Yrt && log_delta && grid_idx && work && N > C && ldx >= N && ldy >= N && P >= 0 &&
                     n_grid > 0,
                 "flmm_fit_delta_gls_f64: bad arguments");
    int rc = check_c(C, "flmm_fit_delta_gls_f64");
    if (rc) return rc;
    GridWs ws = carve_grid(work, N, C, P, n_grid);
    if (work_bytes < ws.bytes)
        return fail(FLMM_ERR_WORKSPACE, "flmm_fit_delta_gls_f64: need %zu bytes, got %zu", ws.bytes, work_bytes);
    if (P == 0) return FLMM_OK;
    cudaStream_t st = as_stream(stream);
    if ((rc = flmm_delta_grid_nodes(lo, hi, n_grid, ws.grid, stream))) return rc;
    k_gls_grid_prep<<<n_grid, 256, 0, st>>>(s, N, Xrt, ldx, C, ws.grid, ws.W, ws.sum_log, ws.Lg, ws.logdet, ws.bad);
    if ((rc = check_launch("k_gls_grid_prep"))) return rc;
    dim3 g2(ceil_div(P, kEvalWarps), n_grid);
    k_gls_grid_loss<<<g2, 32 * kEvalWarps, 0, st>>>(ws.W, Xrt, ldx, C, Yrt, ldy, N, P, ws.sum_log, ws.Lg, ws.logdet,
                                                     ws.bad, reml, ws.loss);
    if ((rc = check_launch("k_gls_grid_loss"))) return rc;
    k_gls_argmin<<<ceil_div(P, 256), 256, 0, st>>>(ws.loss, n_grid, P, grid_idx);
    if ((rc = check_launch("k_gls_argmin"))) return rc;
    const size_t smem = eval_smem_bytes(C);
    if (smem > 48 * 1024)
        FLMM_CUDA(cudaFuncSetAttribute(k_gls_golden, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_gls_golden<<<ceil_div(P, kEvalWarps), 32 * kEvalWarps, smem, st>>>(s, N, Xrt, ldx, C, Yrt, ldy, P, ws.grid,
                                                                          n_grid, grid_idx, refine, reml, lo, hi,
                                                                          log_delta);
    return check_launch("k_gls_golden");
}

extern "C" int flmm_wald_gls_workspace_bytes(int N, int C, int P, size_t* bytes) {
    FLMM_REQUIRE(bytes && N > 0 && C > 0 && P >= 0, "flmm_wald_gls_workspace_bytes: bad arguments");
    *bytes = wald_ws(N, C, P);
    return FLMM_OK;
}

extern "C" int flmm_wald_gls_f64(const double* s, int N, const double* Xrt, int64_t ldx, int C, const double* Yrt,
                                 int64_t ldy, const double* log_delta, int P, int n_real, const double* Srt,
                                 int64_t lds, int M, const int64_t* rows, double* f, double* beta, double* se,
                                 double* sfve, int64_t ldo, double* max_F, void* work, size_t work_bytes,
                                 void* stream) {
    FLMM_REQUIRE(s && Xrt && Yrt && log_delta && max_F && work && N > C + 1 && ldx >= N && ldy >= N && lds >= N &&
                     P >= 0 && M >= 0 && n_real >= 0 && n_real <= P,
                 "flmm_wald_gls_f64: bad arguments");
    FLMM_REQUIRE(n_real == 0 || M == 0 || (rows && f && beta && se && sfve && ldo >= n_real),
                 "flmm_wald_gls_f64: real-column outputs missing");
    FLMM_REQUIRE(M == 0 || Srt, "flmm_wald_gls_f64: Srt is NULL");
    int rc = check_c(C, "flmm_wald_gls_f64");
    if (rc) return rc;
    if (work_bytes < wald_ws(N, C, P))
        return fail(FLMM_ERR_WORKSPACE, "flmm_wald_gls_f64: need %zu bytes, got %zu", wald_ws(N, C, P), work_bytes);
    if (P == 0 || M == 0) return FLMM_OK;
    cudaStream_t st = as_stream(stream);
    const size_t smem_prep = eval_smem_bytes(C);
    if (smem_prep > 48 * 1024)
        FLMM_CUDA(cudaFuncSetAttribute(k_gls_wald_prep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_prep));
    const size_t smem_wald = sizeof(double) * (static_cast<size_t>(WP) * (C + 2) * WK + WM * WK);
    for (int q0 = 0; q0 < P; q0 += kWaldChunk) {
        const int pc = (P - q0 < kWaldChunk) ? P - q0 : kWaldChunk;
        double* Lv = static_cast<double*>(work);
        double* Lp = Lv + static_cast<size_t>(pc) * (C + 2) * N;
        double* rWr = Lp + static_cast<size_t>(pc) * C * C;
        k_gls_wald_prep<<<ceil_div(pc, kEvalWarps), 32 * kEvalWarps, smem_prep, st>>>(
            s, N, Xrt, ldx, C, Yrt + static_cast<int64_t>(q0) * ldy, ldy, pc, log_delta + q0, Lv, Lp, rWr);
        if ((rc = check_launch("k_gls_wald_prep"))) return rc;
        const int nr = n_real - q0 > 0 ? (n_real - q0 < pc ? n_real - q0 : pc) : 0;
        dim3 grid(ceil_div(M, WM), ceil_div(pc, WP));
        // detail outputs exist (and are offset) only for chunks holding real columns
        double* fo = nr > 0 ? f + q0 : nullptr;
        double* bo = nr > 0 ? beta + q0 : nullptr;
        double* so = nr > 0 ? se + q0 : nullptr;
        double* vo = nr > 0 ? sfve + q0 : nullptr;
        auto launch = [&](auto kernel) {
            kernel<<<grid, WT, smem_wald, st>>>(Lv, Lp, rWr, N, C, pc, nr, Srt, lds, M, rows, fo, bo, so, vo, ldo,
                                                max_F + q0);
        };
        if (C + 2 <= 8) launch(k_gls_wald<8>);
        else if (C + 2 <= 16) launch(k_gls_wald<16>);
        else launch(k_gls_wald<32>);
        if ((rc = check_launch("k_gls_wald"))) return rc;
    }
    return FLMM_OK;
}

extern "C" int flmm_shift_diagonal_f64(double* A, int N, int64_t lda, double value, void* stream) {
    FLMM_REQUIRE(A && N > 0 && lda >= N, "flmm_shift_diagonal_f64: bad arguments");
    k_shift_diagonal<<<ceil_div(N, 256), 256, 0, as_stream(stream)>>>(A, N, lda, value);
    return check_launch("k_shift_diagonal");
}

extern "C" int flmm_clamp_nonneg_f64(const double* x, int64_t n, double* y, void* stream) {
    FLMM_REQUIRE((x && y) || n == 0, "flmm_clamp_nonneg_f64: bad arguments");
    if (n == 0) return FLMM_OK;
    k_clamp_nonneg<<<ceil_div(n, 256), 256, 0, as_stream(stream)>>>(x, n, y);
    return check_launch("k_clamp_nonneg");
}
