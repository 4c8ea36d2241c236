// Plain FP64 form of the null-model delta fit (fasterlmm/core.py:525-595): the (G, P) grid of ML -2 log L, its
// first argmin per column, and the reference's 50-step golden-section refinement on [grid[i-1], grid[i+1]].
//
// The loss is evaluated with the reference's operation order, and every a + k * (b - a) bracket update uses
// non-contracting FP64 intrinsics, so each step rounds like the reference's separate tensor operations.  Summation
// order over the eigenvalues differs (warp / tile sums), which is why the refined value agrees with the reference
// to its own FP64 noise rather than bit for bit.
#include <math.h>

#include "flmm_common.cuh"

using namespace flmm;

namespace {

constexpr double kLog2Pi = 1.8378770664093453;  // log(2 pi) in FP64, the reference's log2pi constant

// The low-rank model (fasterlmm/lowrank.py:131-151) adds, per column, the off-rank quadratic form yy_off / delta
// and (Neff - k) log delta to the log determinant, and its Neff is N - D rather than the spectrum length k.  The
// compat fit is the special case yy = NULL, n_logd = 0, neff = k.
struct OffRank {
    const double* yy;  // (P,) off-rank residual sum of squares, or NULL
    double neff;       // sample count of the variance estimate
    double n_logd;     // count of extra log(delta) terms in log det V
};

// ML -2 log L from the weighted sum yWy and log det V (fasterlmm/core.py:538-542, fasterlmm/lowrank.py:144-151)
__device__ __forceinline__ double ml_loss(double yWy, double sum_log_sd, double delta, double yy_off,
                                          const OffRank& o) {
    double rWr = fmax(o.yy ? add_rn(yWy, yy_off / delta) : yWy, kPosFloor);
    double sigma2 = rWr / o.neff;
    double t = add_rn(add_rn(kLog2Pi, log(sigma2)), 1.0);
    const double logdet = o.n_logd != 0.0 ? add_rn(sum_log_sd, mul_rn(o.n_logd, log(delta))) : sum_log_sd;
    return add_rn(mul_rn(o.neff, t), logdet);
}

// Wg[g, n] = 1 / (s[n] + exp(grid[g])), sum_log[g] = sum_n log(s[n] + exp(grid[g])); one block per grid node
__global__ void k_grid_weights(const double* __restrict__ s, int Neff, const double* __restrict__ grid,
                               double* __restrict__ Wg, double* __restrict__ sum_log) {
    __shared__ double red[32];
    const int g = blockIdx.x;
    const double delta = exp(grid[g]);
    double acc = 0.0;
    for (int n = threadIdx.x; n < Neff; n += blockDim.x) {
        double sd = s[n] + delta;
        Wg[static_cast<int64_t>(g) * Neff + n] = 1.0 / sd;
        acc += log(sd);
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) sum_log[g] = v;
    }
}

// Grid loss and first argmin over g for a tile of 64 columns; g is walked in tiles of 64.  yWy[g, p] =
// sum_n Wg[g, n] UY[p, n]^2 is the (G x Neff) x (Neff x P) product of fasterlmm/core.py:537.
constexpr int TG = 64, TP = 64, TK = 16, NT = 256;

__global__ void __launch_bounds__(NT)
k_grid_argmin(const double* __restrict__ Wg, const double* __restrict__ sum_log, const double* __restrict__ grid,
              const double* __restrict__ UYt, int64_t ldu, int Neff, int P, int G, OffRank off,
              int32_t* __restrict__ idx_out) {
    __shared__ double Ws[TK][TG + 1];
    __shared__ double Us[TK][TP + 1];
    __shared__ double red_v[16][TP];
    __shared__ int red_i[16][TP];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int p0 = blockIdx.x * TP;
    double best = INFINITY;
    int best_g = 0;
    for (int g0 = 0; g0 < G; g0 += TG) {
        double acc[4][4] = {};
        for (int k0 = 0; k0 < Neff; k0 += TK) {
#pragma unroll
            for (int l = 0; l < (TG * TK) / NT; ++l) {
                int t = tid + l * NT, g = t / TK, k = t % TK;
                int gg = g0 + g, gk = k0 + k;
                Ws[k][g] = (gg < G && gk < Neff) ? Wg[static_cast<int64_t>(gg) * Neff + gk] : 0.0;
            }
#pragma unroll
            for (int l = 0; l < (TP * TK) / NT; ++l) {
                int t = tid + l * NT, p = t / TK, k = t % TK;
                int gp = p0 + p, gk = k0 + k;
                double u = (gp < P && gk < Neff) ? UYt[static_cast<int64_t>(gp) * ldu + gk] : 0.0;
                Us[k][p] = u * u;
            }
            __syncthreads();
#pragma unroll
            for (int k = 0; k < TK; ++k) {
                double a[4], b[4];
#pragma unroll
                for (int r = 0; r < 4; ++r) a[r] = Ws[k][ty + 16 * r];
#pragma unroll
                for (int c = 0; c < 4; ++c) b[c] = Us[k][tx + 16 * c];
#pragma unroll
                for (int r = 0; r < 4; ++r)
#pragma unroll
                    for (int c = 0; c < 4; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
            }
            __syncthreads();
        }
        // this thread's nodes are g0 + ty + 16 r, ascending in r: keep the first minimum per column
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            double bv = INFINITY;
            int bi = G;
            const int pc = p0 + tx + 16 * c;
            const double yy = (off.yy && pc < P) ? off.yy[pc] : 0.0;
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                int g = g0 + ty + 16 * r;
                if (g < G) {
                    const double dg = (off.yy || off.n_logd != 0.0) ? exp(grid[g]) : 1.0;  // compat needs no delta
                    double v = ml_loss(acc[r][c], sum_log[g], dg, yy, off);
                    if (v < bv) { bv = v; bi = g; }
                }
            }
            red_v[ty][tx + 16 * c] = bv;
            red_i[ty][tx + 16 * c] = bi;
        }
        __syncthreads();
        if (tid < TP) {
            for (int r = 0; r < 16; ++r) {
                double v = red_v[r][tid];
                int gi = red_i[r][tid];
                if (v < best || (v == best && gi < best_g)) { best = v; best_g = gi; }
            }
        }
        __syncthreads();
    }
    if (tid < TP && p0 + tid < P) idx_out[p0 + tid] = best_g;
}

// Per-column loss at its own log delta (fasterlmm/core.py:545-558), by one warp.
__device__ double pheno_loss(const double* __restrict__ s, const double* __restrict__ u, int Neff, double ld,
                             double yy, const OffRank& off) {
    const int lane = threadIdx.x & 31;
    const double delta = exp(ld);
    double ywy = 0.0, sl = 0.0;
    for (int n = lane; n < Neff; n += 32) {
        double sd = s[n] + delta;
        double w = 1.0 / sd;
        ywy += mul_rn(mul_rn(w, u[n]), u[n]);
        sl += log(sd);
    }
    ywy = warp_sum(ywy);
    sl = warp_sum(sl);
    return ml_loss(ywy, sl, delta, yy, off);
}

// golden-section search, one warp per column (fasterlmm/core.py:577-595)
__global__ void k_golden(const double* __restrict__ s, int Neff, const double* __restrict__ UYt, int64_t ldu, int P,
                         const double* __restrict__ grid, int G, const int32_t* __restrict__ idx, int refine,
                         double lo, double hi, OffRank off, double* __restrict__ log_delta) {
    const int64_t p = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    if (p >= P) return;
    const int i = idx[p];
    if (!refine) {
        if ((threadIdx.x & 31) == 0) log_delta[p] = grid[i];
        return;
    }
    const double* u = UYt + p * ldu;
    const double yy = off.yy ? off.yy[p] : 0.0;
    const int lo_i = max(i - 1, 0), hi_i = min(i + 1, G - 1);
    double a = grid[lo_i], b = grid[hi_i];
    const double inv_phi = 2.0 / (1.0 + sqrt(5.0));
    const double inv_phi2 = mul_rn(inv_phi, inv_phi);
    double c = add_rn(a, mul_rn(inv_phi2, add_rn(b, -a)));
    double d = add_rn(a, mul_rn(inv_phi, add_rn(b, -a)));
    double fc = pheno_loss(s, u, Neff, c, yy, off);
    double fd = pheno_loss(s, u, Neff, d, yy, off);
    for (int it = 0; it < 50; ++it) {
        const bool cond = fc < fd;
        b = cond ? d : b;
        a = cond ? a : c;
        c = add_rn(a, mul_rn(inv_phi2, add_rn(b, -a)));
        d = add_rn(a, mul_rn(inv_phi, add_rn(b, -a)));
        fc = pheno_loss(s, u, Neff, c, yy, off);
        fd = pheno_loss(s, u, Neff, d, yy, off);
    }
    if ((threadIdx.x & 31) == 0) log_delta[p] = fmin(fmax(mul_rn(0.5, add_rn(a, b)), lo), hi);
}

size_t fit_ws(int Neff, int G) {
    return sizeof(double) * (static_cast<size_t>(G) * Neff + 2 * static_cast<size_t>(G)) + 256;
}

}  // namespace

extern "C" int flmm_fit_delta_f64_workspace_bytes(int Neff, int n_grid, size_t* bytes) {
    FLMM_REQUIRE(bytes && Neff > 0 && n_grid > 0, "flmm_fit_delta_f64_workspace_bytes: bad arguments");
    *bytes = fit_ws(Neff, n_grid);
    return FLMM_OK;
}

namespace {

int fit_delta_impl(const double* s, int Neff, const double* UYt, int64_t ldu, int P, int n_grid, double lo, double hi,
                   int refine, const OffRank& off, double* log_delta, int32_t* grid_idx, void* work, size_t work_bytes,
                   void* stream, const char* fn) {
    if (work_bytes < fit_ws(Neff, n_grid))
        return fail(FLMM_ERR_WORKSPACE, "%s: need %zu bytes, got %zu", fn, fit_ws(Neff, n_grid), work_bytes);
    if (P == 0) return FLMM_OK;
    cudaStream_t st = as_stream(stream);
    double* Wg = static_cast<double*>(work);
    double* sum_log = Wg + static_cast<size_t>(n_grid) * Neff;
    double* grid = sum_log + n_grid;
    int rc = flmm_delta_grid_nodes(lo, hi, n_grid, grid, stream);
    if (rc) return rc;
    k_grid_weights<<<n_grid, 256, 0, st>>>(s, Neff, grid, Wg, sum_log);
    if ((rc = check_launch("k_grid_weights"))) return rc;
    k_grid_argmin<<<ceil_div(P, TP), NT, 0, st>>>(Wg, sum_log, grid, UYt, ldu, Neff, P, n_grid, off, grid_idx);
    if ((rc = check_launch("k_grid_argmin"))) return rc;
    k_golden<<<ceil_div(static_cast<int64_t>(P) * 32, 256), 256, 0, st>>>(s, Neff, UYt, ldu, P, grid, n_grid,
                                                                          grid_idx, refine, lo, hi, off, log_delta);
    return check_launch("k_golden");
}

}  // namespace

extern "C" int flmm_fit_delta_f64(const double* s, int Neff, const double* UYt, int64_t ldu, int P, int n_grid,
                                  double lo, double hi, int refine, double* log_delta, int32_t* grid_idx, void* work,
                                  size_t work_bytes, void* stream) {
    FLMM_REQUIRE(s && UYt && log_delta && grid_idx && work && Neff > 0 && n_grid > 0 && ldu >= Neff && P >= 0,
                 "flmm_fit_delta_f64: bad arguments");
    const OffRank off{nullptr, static_cast<double>(Neff), 0.0};
    return fit_delta_impl(s, Neff, UYt, ldu, P, n_grid, lo, hi, refine, off, log_delta, grid_idx, work, work_bytes,
                          stream, "flmm_fit_delta_f64");
}

extern "C" int flmm_fit_delta_lowrank_f64(const double* s, int k, const double* UYt, int64_t ldu, const double* yy_off,
                                          int Neff, int P, int n_grid, double lo, double hi, int refine,
                                          double* log_delta, int32_t* grid_idx, void* work, size_t work_bytes,
                                          void* stream) {
    FLMM_REQUIRE(s && UYt && yy_off && log_delta && grid_idx && work && k > 0 && Neff > 0 && n_grid > 0 && ldu >= k &&
                     P >= 0,
                 "flmm_fit_delta_lowrank_f64: bad arguments");
    // Neff - k may be negative: with k >= N the reference's basis can keep O(1e-17) directions of the projected-out
    // space, each adding log(s + delta) ~ log(delta), which the negative count cancels (fasterlmm/lowrank.py:88-94)
    const OffRank off{yy_off, static_cast<double>(Neff), static_cast<double>(Neff - k)};
    return fit_delta_impl(s, k, UYt, ldu, P, n_grid, lo, hi, refine, off, log_delta, grid_idx, work, work_bytes,
                          stream, "flmm_fit_delta_lowrank_f64");
}
