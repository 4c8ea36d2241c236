// Learned delta proposal for the fast delta fit (no counterpart in the reference, which searches a grid).
//
// A small MLP maps cheap per-column features of the rotated phenotype to log delta:
//   f_b = log(e_b / E + 1e-12), e_b = sum of UY^2 over the b-th of 32 equal-count bins of the ascending spectrum,
//   g_b = log(mean of s over bin b + 1e-4)   (the spectrum's shape, shared by all columns of a chromosome),
//   log(Neff) / 10,
// 65 inputs -> 128 -> 128 -> 1 with tanh-GELU.  The proposal collapses the fit's grid search to a narrow bracket:
// each column evaluates the FP32 grid loss only at the 2 h + 1 grid nodes nearest its proposal and takes their
// argmin.  The full grid stays both the fallback and the check on the proposal:
//   * a column whose window argmin sits on the window's edge (the minimum may lie outside it) is put on a list whose
//     columns then get the full grid argmin;
//   * every audit_stride-th column also evaluates the full grid; if a node outside the window beats the window's
//     argmin there, every column of the call falls back to the full grid.
// The exact refinement (the fast fit's bracketed Newton iteration) then runs from the chosen node, as in the grid
// path, so the answer is the same stationary point of the same loss; the proposal saves grid evaluations.
#include <math.h>

#include "flmm_common.cuh"
#include "flmm_delta_eval.cuh"
#include "flmm_mlp.cuh"

using namespace flmm;
using namespace flmm::dfit;

namespace {

constexpr int kBins = 32;
constexpr int kIn = 2 * kBins + 1;
constexpr int kHid = 128;

// Features of one column per warp: feats[p, b] = f_b, feats[p, 32 + b] = g_b, feats[p, 64] = log(Neff) / 10.
__global__ void k_delta_features(const double* __restrict__ s, int Neff, const float* __restrict__ UYt, int64_t ldu,
                                 int P, float* __restrict__ feats) {
    const int lane = threadIdx.x & 31;
    const int64_t p = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    if (p >= P) return;
    const float* u = UYt + p * ldu;
    // bin `lane` covers eigen-indices [lane Neff / 32, (lane + 1) Neff / 32)
    const int n0 = static_cast<int>((static_cast<int64_t>(lane) * Neff) / kBins);
    const int n1 = static_cast<int>((static_cast<int64_t>(lane + 1) * Neff) / kBins);
    float e = 0.0f, sm = 0.0f;
    for (int n = n0; n < n1; ++n) {
        e += u[n] * u[n];
        sm += static_cast<float>(s[n]);
    }
    const float E = warp_sum(e);
    float* f = feats + p * kIn;
    f[lane] = logf((E > 0.0f ? e / E : 0.0f) + 1e-12f);
    f[kBins + lane] = logf((n1 > n0 ? sm / static_cast<float>(n1 - n0) : 0.0f) + 1e-4f);
    if (lane == 0) f[2 * kBins] = logf(static_cast<float>(Neff)) * 0.1f;
}

// The MLP over tiles of 16 columns: a persistent CTA holds both weight matrices in shared memory (thread j = hidden
// unit j, the forward pass of flmm_mlp.cuh in FP32) and writes x = clamp(out, lo, hi).
__global__ void __launch_bounds__(mlp::kMlpThreads)
k_delta_mlp(const float* __restrict__ feats, int P, const float* __restrict__ W1, const float* __restrict__ b1,
            const float* __restrict__ W2, const float* __restrict__ b2, const float* __restrict__ w3, float b3,
            double lo, double hi, double* __restrict__ x_out) {
    using namespace flmm::mlp;
    extern __shared__ float sm[];
    float* W1s = sm;
    float* W2s = W1s + kHid * kIn;
    float* xs = W2s + kHid * kLdW2;
    float* a1s = xs + kMlpRows * kIn;
    float* red = a1s + kMlpRows * kHid;
    auto same = [](float v) { return v; };
    load_weights(W1, W2, W1s, W2s, same);
    const int j = threadIdx.x;
    const float b1j = b1[j], b2j = b2[j], w3j = w3[j];
    const int n_tiles = (P + kMlpRows - 1) / kMlpRows;
    for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const int r0 = tile * kMlpRows;
        __syncthreads();  // the previous tile is done with xs, a1s and red (and the weights are in place)
        for (int t = j; t < kMlpRows * kIn; t += kMlpThreads) {
            const int r = t / kIn;
            xs[t] = (r0 + r < P) ? feats[static_cast<int64_t>(r0 + r) * kIn + t % kIn] : 0.0f;
        }
        __syncthreads();
        float z1[kMlpRows], z2[kMlpRows], a2[kMlpRows];
        forward_tile(W1s, W2s, xs, a1s, b1j, b2j, z1, z2, a2, same);
        output_partials(w3j, a2, red);
        __syncthreads();
        if (j < kMlpRows && r0 + j < P) x_out[r0 + j] = fmin(fmax(static_cast<double>(row_output(red, j, b3)), lo), hi);
    }
}

constexpr size_t kMlpSmem =
    sizeof(float) * (static_cast<size_t>(mlp::kHid) * mlp::kIn + static_cast<size_t>(mlp::kHid) * mlp::kLdW2 +
                     mlp::kMlpRows * mlp::kIn + mlp::kMlpRows * mlp::kHid + 4 * mlp::kMlpRows);

int launch_delta_mlp(const float* feats, int P, const float* W1, const float* b1, const float* W2, const float* b2,
                     const float* w3, float b3, double lo, double hi, double* x_out, cudaStream_t st) {
    FLMM_CUDA(cudaFuncSetAttribute(k_delta_mlp, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(kMlpSmem)));
    int dev = 0, sms = 0;
    FLMM_CUDA(cudaGetDevice(&dev));
    FLMM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int n_tiles = (P + mlp::kMlpRows - 1) / mlp::kMlpRows;
    const int grid = n_tiles < 2 * sms ? n_tiles : 2 * sms;
    k_delta_mlp<<<grid, mlp::kMlpThreads, kMlpSmem, st>>>(feats, P, W1, b1, W2, b2, w3, b3, lo, hi, x_out);
    return check_launch("k_delta_mlp");
}

// Grid loss of one column at node g (the FP32 grid path's formula): Neff log(sum_n Wg[g, n] u_n^2) + sum_log[g]
__device__ __forceinline__ float window_loss(const float* __restrict__ Wg, const float* __restrict__ sum_log,
                                             const float* __restrict__ u, int Neff, int g, int lane) {
    const float* w = Wg + static_cast<int64_t>(g) * Neff;
    float acc = 0.0f;
    for (int n = lane; n < Neff; n += 32) acc = fmaf(w[n], u[n] * u[n], acc);
    acc = warp_sum(acc);
    return static_cast<float>(Neff) * logf(fmaxf(acc, 1e-30f)) + sum_log[g];
}

// stats: [0] columns on the fallback list, [1] audited columns, [2] audits lost, [3] grid nodes evaluated here
__global__ void k_delta_window(const float* __restrict__ Wg, const float* __restrict__ sum_log,
                               const double* __restrict__ grid, int G, const float* __restrict__ UYt, int64_t ldu,
                               int Neff, int P, const double* __restrict__ x_prop, int half, int audit_stride,
                               int32_t* __restrict__ idx, int32_t* __restrict__ fb_cols, int32_t* __restrict__ stats) {
    const int lane = threadIdx.x & 31;
    const int64_t p = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    if (p >= P) return;
    const float* u = UYt + p * ldu;
    const double h = G > 1 ? (grid[G - 1] - grid[0]) / (G - 1) : 1.0;
    const double t = (x_prop[p] - grid[0]) / h;
    const int c = t <= 0.0 ? 0 : (t >= G - 1 ? G - 1 : static_cast<int>(llrint(t)));
    const int wlo = max(c - half, 0), whi = min(c + half, G - 1);
    float best = INFINITY;
    int bi = wlo;
    for (int g = wlo; g <= whi; ++g) {
        const float v = window_loss(Wg, sum_log, u, Neff, g, lane);
        if (v < best) { best = v; bi = g; }
    }
    int evals = whi - wlo + 1;
    bool edge = (bi == wlo && wlo > 0) || (bi == whi && whi < G - 1);
    if (audit_stride > 0 && p % audit_stride == 0) {
        float fbest = INFINITY;
        int fi = 0;
        for (int g = 0; g < G; ++g) {
            const float v = (g >= wlo && g <= whi) ? INFINITY : window_loss(Wg, sum_log, u, Neff, g, lane);
            if (v < fbest) { fbest = v; fi = g; }
        }
        evals += G - (whi - wlo + 1);
        if (lane == 0) {
            atomicAdd(&stats[1], 1);
            if (!edge && fbest < best) atomicAdd(&stats[2], 1);  // a node outside the window is lower
        }
        if (fbest < best || (fbest == best && fi < bi)) bi = fi;  // the audited column keeps the full-grid argmin
        edge = false;
    }
    if (lane == 0) {
        if (edge) fb_cols[atomicAdd(&stats[0], 1)] = static_cast<int32_t>(p);
        else idx[p] = bi;
        atomicAdd(&stats[3], evals);
    }
}

// After a lost audit every column goes on the fallback list.
__global__ void k_window_fallback_all(int P, int32_t* __restrict__ fb_cols, int32_t* __restrict__ stats) {
    if (stats[2] == 0) return;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < P) fb_cols[p] = p;
    if (p == 0) stats[0] = P;
}

inline size_t pad256(size_t x) { return (x + 255) / 256 * 256; }

size_t learned_ws(int Neff, int G, int P) {
    return pad256(fast_ws(Neff, G)) + pad256(sizeof(float) * static_cast<size_t>(P) * kIn) +
           pad256(sizeof(double) * static_cast<size_t>(P)) + pad256(sizeof(int32_t) * static_cast<size_t>(P));
}

}  // namespace

extern "C" int flmm_delta_features_f32(const double* s, int Neff, const float* UYt, int64_t ldu, int P, float* feats,
                                       void* stream) {
    FLMM_REQUIRE(s && UYt && feats && Neff >= kBins && ldu >= Neff && P >= 0,
                 "flmm_delta_features_f32: bad arguments (Neff must be >= 32)");
    if (P == 0) return FLMM_OK;
    k_delta_features<<<ceil_div(static_cast<int64_t>(P) * 32, 256), 256, 0, as_stream(stream)>>>(s, Neff, UYt, ldu,
                                                                                                 P, feats);
    return check_launch("k_delta_features");
}

extern "C" int flmm_delta_mlp_f32(const float* feats, int P, const float* W1, const float* b1, const float* W2,
                                  const float* b2, const float* w3, float b3, double lo, double hi, double* x_out,
                                  void* stream) {
    FLMM_REQUIRE(feats && W1 && b1 && W2 && b2 && w3 && x_out && P >= 0, "flmm_delta_mlp_f32: bad arguments");
    if (P == 0) return FLMM_OK;
    return launch_delta_mlp(feats, P, W1, b1, W2, b2, w3, b3, lo, hi, x_out, as_stream(stream));
}

extern "C" int flmm_fit_delta_learned_workspace_bytes(int Neff, int n_grid, int P, size_t* bytes) {
    FLMM_REQUIRE(bytes && Neff > 0 && n_grid > 0 && P >= 0, "flmm_fit_delta_learned_workspace_bytes: bad arguments");
    *bytes = learned_ws(Neff, n_grid, P);
    return FLMM_OK;
}

extern "C" int flmm_fit_delta_learned(const double* s, int Neff, const float* UYt, int64_t ldu, int P, int n_grid,
                                      double lo, double hi, int refine, const float* W1, const float* b1,
                                      const float* W2, const float* b2, const float* w3, float b3, int half_width,
                                      int audit_stride, double* log_delta, int32_t* grid_idx, int32_t* stats,
                                      void* work, size_t work_bytes, void* stream) {
    FLMM_REQUIRE(s && UYt && W1 && b1 && W2 && b2 && w3 && log_delta && grid_idx && stats && work && n_grid > 0 &&
                     ldu >= Neff && P >= 0 && half_width >= 1 && audit_stride >= 0,
                 "flmm_fit_delta_learned: bad arguments");
    FLMM_REQUIRE(Neff >= kBins, "flmm_fit_delta_learned: Neff must be >= %d (the proposal's features)", kBins);
    const size_t need = learned_ws(Neff, n_grid, P);
    if (work_bytes < need)
        return fail(FLMM_ERR_WORKSPACE, "flmm_fit_delta_learned: need %zu bytes, got %zu", need, work_bytes);
    cudaStream_t st = as_stream(stream);
    FLMM_CUDA(cudaMemsetAsync(stats, 0, 4 * sizeof(int32_t), st));
    if (P == 0) return FLMM_OK;
    char* base = static_cast<char*>(work);
    const FastWs w = carve_fast(base, Neff, n_grid);
    size_t off = pad256(fast_ws(Neff, n_grid));
    float* feats = reinterpret_cast<float*>(base + off);
    off += pad256(sizeof(float) * static_cast<size_t>(P) * kIn);
    double* x_prop = reinterpret_cast<double*>(base + off);
    off += pad256(sizeof(double) * static_cast<size_t>(P));
    int32_t* fb_cols = reinterpret_cast<int32_t*>(base + off);

    int rc = launch_grid_tables(s, Neff, lo, hi, n_grid, w, st);
    if (rc) return rc;
    const unsigned warps_grid = ceil_div(static_cast<int64_t>(P) * 32, 256);
    k_delta_features<<<warps_grid, 256, 0, st>>>(s, Neff, UYt, ldu, P, feats);
    if ((rc = check_launch("k_delta_features"))) return rc;
    if ((rc = launch_delta_mlp(feats, P, W1, b1, W2, b2, w3, b3, lo, hi, x_prop, st))) return rc;
    k_delta_window<<<warps_grid, 256, 0, st>>>(w.Wg, w.sum_log, w.grid, n_grid, UYt, ldu, Neff, P, x_prop, half_width,
                                               audit_stride, grid_idx, fb_cols, stats);
    if ((rc = check_launch("k_delta_window"))) return rc;
    k_window_fallback_all<<<ceil_div(P, 256), 256, 0, st>>>(P, fb_cols, stats);
    if ((rc = check_launch("k_window_fallback_all"))) return rc;
    if ((rc = launch_grid_argmin_list(w, UYt, ldu, Neff, P, n_grid, fb_cols, stats, grid_idx, st))) return rc;
    return launch_refine(s, Neff, UYt, ldu, P, n_grid, grid_idx, refine, w, log_delta, st);
}
