// Fast form of the null-model delta fit (fasterlmm/core.py:561-595).
//
// Grid: the (G, P) ML loss in FP32 from w[g, n] = 1 / (s_n + delta_g) and UY^2 (a tiled (G x Neff) x (Neff x P)
// product), first argmin per column.  The bracket is the reference's [grid[i-1], grid[i+1]].
//
// Refinement: where the reference runs 50 golden-section steps on the loss, this finds the stationary point of the
// loss in the bracket directly.  With x = log delta, r_n = 1 / (s_n + delta), S_k = sum u_n^2 r_n^k, T_k = sum r_n^k,
//     dL/dx = delta (T1 - Neff S2 / S1),  d/dx (T1 - Neff S2 / S1) = delta (-T2 + Neff (2 S3 / S1 - S2^2 / S1^2)),
// and a sign-safeguarded Newton iteration on g = T1 - Neff S2 / S1 keeps g(lo) < 0 < g(hi), so it always converges
// to a local minimum of the loss in the bracket (never a maximum).  When g does not change sign the minimum is a
// bracket edge, which is where the golden-section search converges as well.  The sums are accumulated in FP32 in a
// centred form (newton_eval) with Neumaier compensation and combined across lanes with TwoSum, so g is accurate to
// the rounding of the individual terms (~1e-7 relative each, averaging out over Neff); log delta comes out within
// ~1e-7 of the exact stationary point, well inside the FP64 noise of the reference's own search on flat likelihoods.
#include <math.h>

#include <mutex>

#include "flmm_common.cuh"
#include "flmm_delta_eval.cuh"

using namespace flmm;
using namespace flmm::dfit;

namespace {

__global__ void k_grid_weights_f32(const double* __restrict__ s, int Neff, const double* __restrict__ grid,
                                   float* __restrict__ Wg, float* __restrict__ sum_log) {
    __shared__ double red[32];
    const int g = blockIdx.x;
    const double delta = exp(grid[g]);
    double acc = 0.0;
    for (int n = threadIdx.x; n < Neff; n += blockDim.x) {
        const double sd = s[n] + delta;
        Wg[static_cast<int64_t>(g) * Neff + n] = static_cast<float>(1.0 / sd);
        acc += log(sd);
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) sum_log[g] = static_cast<float>(v);
    }
}

// Tiles of the grid product: 64 grid nodes x 128 columns per block, 32-deep k steps, 128 threads of 8 x 8
// accumulators (nodes 8 ty .. +7 against columns 4 tx .. +3 and 64 + 4 tx .. +3, so the quarter-warps' 128-bit shared
// loads fall in distinct banks).  Shared rows are padded by 4 floats for the same reason on the transposing stores.
constexpr int TG = 64, TP = 128, TK = 32, NT = 128;
constexpr int WS_LD = TG + 4, US_LD = TP + 4;

// loss[g, p] = Neff log(yWy) + sum_log[g] (+ constants that do not move the argmin), first argmin over g.  Every
// accumulator adds its k terms in order with one FMA each, as a plain loop over n would.
// kList: the CTA's columns are entries [128 b, 128 b + 128) of the column list cols[0 .. *count) instead of columns
// [128 b, 128 b + 128); CTAs past the list's end return at once (the grid is sized for the longest list, P).
template <bool kList>
__global__ void __launch_bounds__(NT)
k_grid_argmin_f32(const float* __restrict__ Wg, const float* __restrict__ sum_log, const float* __restrict__ UYt,
                  int64_t ldu, int Neff, int P, int G, int32_t* __restrict__ idx_out, const int32_t* __restrict__ cols,
                  const int32_t* __restrict__ count) {
    __shared__ __align__(16) float Ws[TK * WS_LD];
    __shared__ __align__(16) float Us[TK * US_LD];
    __shared__ float red_v[8][TP];
    __shared__ int red_i[8][TP];
    __shared__ int col_s[TP];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int lane = tid & 31, warp = tid >> 5;
    const int p0 = blockIdx.x * TP;
    if (kList) {
        const int n = min(*count, P);
        if (p0 >= n) return;
    }
    for (int q = tid; q < TP; q += NT) {
        if (kList) {
            const int n = min(*count, P);
            col_s[q] = (p0 + q < n) ? cols[p0 + q] : -1;
        } else {
            col_s[q] = (p0 + q < P) ? p0 + q : -1;
        }
    }
    __syncthreads();
    const float neff = static_cast<float>(Neff);
    float best = INFINITY;
    int best_g = 0;
    for (int g0 = 0; g0 < G; g0 += TG) {
        float acc[8][8];
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int c = 0; c < 8; ++c) acc[r][c] = 0.0f;
        // register prefetch: the next k tile's entries are loaded while the current one is multiplied
        float wv[16], uv[32];
        auto load_tile = [&](int k0) {
            const int gk = k0 + lane;
            const bool kok = gk < Neff;
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int gg = g0 + 16 * warp + i;
                wv[i] = (gg < G && kok) ? Wg[static_cast<int64_t>(gg) * Neff + gk] : 0.0f;
            }
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                const int col = col_s[32 * warp + i];
                const float u = (col >= 0 && kok) ? UYt[static_cast<int64_t>(col) * ldu + gk] : 0.0f;
                uv[i] = u * u;
            }
        };
        load_tile(0);
        for (int k0 = 0; k0 < Neff; k0 += TK) {
            // weights: warp w stores nodes 16 w .. +15 of k = lane, squared column entries columns 32 w .. +31, four
            // per 128-bit store
#pragma unroll
            for (int i = 0; i < 16; i += 4)
                *reinterpret_cast<float4*>(&Ws[lane * WS_LD + 16 * warp + i]) =
                    make_float4(wv[i], wv[i + 1], wv[i + 2], wv[i + 3]);
#pragma unroll
            for (int i = 0; i < 32; i += 4)
                *reinterpret_cast<float4*>(&Us[lane * US_LD + 32 * warp + i]) =
                    make_float4(uv[i], uv[i + 1], uv[i + 2], uv[i + 3]);
            __syncthreads();
            if (k0 + TK < Neff) load_tile(k0 + TK);
#pragma unroll 4
            for (int k = 0; k < TK; ++k) {
                const float4 a0 = *reinterpret_cast<const float4*>(&Ws[k * WS_LD + 8 * ty]);
                const float4 a1 = *reinterpret_cast<const float4*>(&Ws[k * WS_LD + 8 * ty + 4]);
                const float4 b0 = *reinterpret_cast<const float4*>(&Us[k * US_LD + 4 * tx]);
                const float4 b1 = *reinterpret_cast<const float4*>(&Us[k * US_LD + 64 + 4 * tx]);
                const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
                for (int r = 0; r < 8; ++r)
#pragma unroll
                    for (int c = 0; c < 8; ++c) acc[r][c] = fmaf(a[r], b[c], acc[r][c]);
            }
            __syncthreads();
        }
        // per column: the first minimum over this thread's 8 nodes, then over the 8 threads of the column
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int q = (c < 4) ? 4 * tx + c : 64 + 4 * tx + (c - 4);
            float bv = INFINITY;
            int bi = G;
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const int g = g0 + 8 * ty + r;
                if (g < G) {
                    const float v = neff * logf(fmaxf(acc[r][c], 1e-30f)) + sum_log[g];
                    if (v < bv) { bv = v; bi = g; }
                }
            }
            red_v[ty][q] = bv;
            red_i[ty][q] = bi;
        }
        __syncthreads();
        for (int q = tid; q < TP; q += NT) {
            // one thread per column (NT == TP)
            for (int r = 0; r < 8; ++r) {
                const float v = red_v[r][q];
                const int gi = red_i[r][q];
                if (v < best || (v == best && gi < best_g)) { best = v; best_g = gi; }
            }
        }
        __syncthreads();
    }
    static_assert(NT == TP, "one thread per column in the final reduction");
    const int col = col_s[tid];
    if (col >= 0) idx_out[col] = best_g;
}

// The spectrum as the evaluations read it, once per fit: s32 = fl32(s), dsb = sbar - s32, sbar = mean(s).
__global__ void k_spectrum_prep(const double* __restrict__ s, int Neff, float* __restrict__ s32,
                                float* __restrict__ dsb, float* __restrict__ sbar_out) {
    __shared__ double red[32];
    double acc = 0.0;
    for (int n = threadIdx.x; n < Neff; n += blockDim.x) acc += s[n];
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) red[0] = v;
    }
    __syncthreads();
    const float sbar = static_cast<float>(red[0] / Neff);
    for (int n = threadIdx.x; n < Neff; n += blockDim.x) {
        const float sn = static_cast<float>(s[n]);
        s32[n] = sn;
        dsb[n] = sbar - sn;
    }
    if (threadIdx.x == 0) *sbar_out = sbar;
}

// Lanes per column of the refinement: two columns per warp (see group_sum).
constexpr int kNewtonLanes = 16;

// One group of kNewtonLanes lanes per column; the spectrum arrays are shared by every group of the grid through
// L1 / L2.
__global__ void k_newton_refine(const float* __restrict__ s32, const float* __restrict__ dsb,
                                const float* __restrict__ sbar_p, int Neff, const float* __restrict__ UYt, int64_t ldu,
                                int P, const double* __restrict__ grid, int G, const int32_t* __restrict__ idx,
                                int refine, double* __restrict__ log_delta) {
    constexpr int W = kNewtonLanes;
    const int lane = threadIdx.x & (W - 1);
    const int64_t p = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) / W;
    if (p >= P) return;
    const float* u = UYt + p * ldu;
    const float sbar = *sbar_p;
    const int i = idx[p];
    // one pass gives the column's sum of squares and the evaluations at the grid argmin and its two neighbours (the
    // bracket test of the usual case), sharing the loads of the column and the spectrum
    const bool inner = refine && i > 0 && i < G - 1;
    const EvalPoint pt = eval_point(grid[i], sbar);
    const EvalPoint pa = eval_point(grid[inner ? i - 1 : i], sbar);
    const EvalPoint pb = eval_point(grid[inner ? i + 1 : i], sbar);
    EvalSums t, ta, tb;
    float uh = 0.f, uc = 0.f;
#pragma unroll 4
    for (int n = lane; n < Neff; n += W) {
        const float un = u[n];
        const float uu = un * un;
        const float sn = s32[n], dn = dsb[n];
        neumaier(uh, uc, uu);
        t.add(sn, dn, uu, pt, false);
        if (inner) {
            ta.add(sn, dn, uu, pa, false);
            tb.add(sn, dn, uu, pb, false);
        }
    }
    const float U = group_sum_pair<W>(uh, uc);
    FirstEvals first;
    first.at = finish_eval<W>(t, U, Neff, pt, false);
    first.have_at = true;
    if (inner) {
        first.lo = finish_eval<W>(ta, U, Neff, pa, false);
        first.hi = finish_eval<W>(tb, U, Neff, pb, false);
        first.have_nb = true;
    }
    const GlobalColumn<W> ev{s32, dsb, u, Neff, sbar, U};
    const double out = refine_column(ev, grid, G, i, refine, &first);
    if (lane == 0) log_delta[p] = out;
}

int launch_fast_fit(const double* s, int Neff, const float* UYt, int64_t ldu, int P, int n_grid, double lo,
                    double hi, int refine, double* log_delta, int32_t* grid_idx, void* scratch, cudaStream_t st) {
    const FastWs w = carve_fast(scratch, Neff, n_grid);
    int rc = flmm_delta_grid_nodes(lo, hi, n_grid, w.grid, st);
    if (rc) return rc;
    k_grid_weights_f32<<<n_grid, 256, 0, st>>>(s, Neff, w.grid, w.Wg, w.sum_log);
    if ((rc = check_launch("k_grid_weights_f32"))) return rc;
    k_grid_argmin_f32<false><<<ceil_div(P, TP), NT, 0, st>>>(w.Wg, w.sum_log, UYt, ldu, Neff, P, n_grid, grid_idx,
                                                             nullptr, nullptr);
    if ((rc = check_launch("k_grid_argmin_f32"))) return rc;
    k_spectrum_prep<<<1, 256, 0, st>>>(s, Neff, w.s32, w.dsb, w.sbar);
    if ((rc = check_launch("k_spectrum_prep"))) return rc;
    k_newton_refine<<<ceil_div(static_cast<int64_t>(P) * kNewtonLanes, 256), 256, 0, st>>>(
        w.s32, w.dsb, w.sbar, Neff, UYt, ldu, P, w.grid, n_grid, grid_idx, refine, log_delta);
    return check_launch("k_newton_refine");
}

}  // namespace

// Pieces of the fit for the learned-proposal path (flmm_delta_learned.cu), declared in flmm_delta_eval.cuh.
namespace flmm {
namespace dfit {

size_t fast_ws(int Neff, int G) {
    return sizeof(float) * (static_cast<size_t>(G) * Neff + static_cast<size_t>(G) + 2 * static_cast<size_t>(Neff) + 4) +
           sizeof(double) * G + 512;
}

FastWs carve_fast(void* base, int Neff, int G) {
    FastWs w;
    w.grid = static_cast<double*>(base);
    w.Wg = reinterpret_cast<float*>(w.grid + G);
    w.sum_log = w.Wg + static_cast<size_t>(G) * Neff;
    w.s32 = w.sum_log + G;
    w.dsb = w.s32 + Neff;
    w.sbar = w.dsb + Neff;
    return w;
}

int launch_grid_tables(const double* s, int Neff, double lo, double hi, int G, const FastWs& w, cudaStream_t st) {
    int rc = flmm_delta_grid_nodes(lo, hi, G, w.grid, st);
    if (rc) return rc;
    k_grid_weights_f32<<<G, 256, 0, st>>>(s, Neff, w.grid, w.Wg, w.sum_log);
    return check_launch("k_grid_weights_f32");
}

int launch_grid_argmin_list(const FastWs& w, const float* UYt, int64_t ldu, int Neff, int P, int G,
                            const int32_t* cols, const int32_t* count, int32_t* idx, cudaStream_t st) {
    k_grid_argmin_f32<true><<<ceil_div(P, TP), NT, 0, st>>>(w.Wg, w.sum_log, UYt, ldu, Neff, P, G, idx, cols, count);
    return check_launch("k_grid_argmin_f32 (column list)");
}

int launch_refine(const double* s, int Neff, const float* UYt, int64_t ldu, int P, int G, const int32_t* idx,
                  int refine, const FastWs& w, double* log_delta, cudaStream_t st) {
    k_spectrum_prep<<<1, 256, 0, st>>>(s, Neff, w.s32, w.dsb, w.sbar);
    int rc = check_launch("k_spectrum_prep");
    if (rc) return rc;
    k_newton_refine<<<ceil_div(static_cast<int64_t>(P) * kNewtonLanes, 256), 256, 0, st>>>(
        w.s32, w.dsb, w.sbar, Neff, UYt, ldu, P, w.grid, G, idx, refine, log_delta);
    return check_launch("k_newton_refine");
}

}  // namespace dfit
}  // namespace flmm

extern "C" int flmm_fit_delta_fast_workspace_bytes(int Neff, int n_grid, size_t* bytes) {
    FLMM_REQUIRE(bytes && Neff > 0 && n_grid > 0, "flmm_fit_delta_fast_workspace_bytes: bad arguments");
    *bytes = fast_ws(Neff, n_grid);
    return FLMM_OK;
}

extern "C" int flmm_fit_delta_fast(const double* s, int Neff, const float* UYt, int64_t ldu, int P, int n_grid,
                                   double lo, double hi, int refine, double* log_delta, int32_t* grid_idx, void* work,
                                   size_t work_bytes, void* stream) {
    FLMM_REQUIRE(s && UYt && log_delta && grid_idx && work && Neff > 0 && n_grid > 0 && ldu >= Neff && P >= 0,
                 "flmm_fit_delta_fast: bad arguments");
    if (work_bytes < fast_ws(Neff, n_grid))
        return fail(FLMM_ERR_WORKSPACE, "flmm_fit_delta_fast: need %zu bytes, got %zu", fast_ws(Neff, n_grid), work_bytes);
    if (P == 0) return FLMM_OK;
    return launch_fast_fit(s, Neff, UYt, ldu, P, n_grid, lo, hi, refine, log_delta, grid_idx, work, as_stream(stream));
}

// ---- allocation-free variant ------------------------------------------------------------------------------------
//
// Some callers cannot hand this library any device memory: a host whose device memory is entirely owned by another
// memory pool (a framework that reserved all of it up front), or a call site in a latency-critical loop that may not
// call cudaMalloc, which can synchronise the device and has no bounded latency.  flmm_fit_delta_fast_noalloc serves
// them: its scratch (grid nodes, the (n_grid, Neff) weight table and the per-node log determinants) lives in the
// fixed array below, which every GPU that loads this library holds until the process exits.
//
// The array is shared by every call of this entry point on a device and keeps the previous call's contents; each
// call overwrites every byte it reads before reading it, so nothing has to start at zero.  Calls whose kernels
// overlap on the GPU (other streams, other host threads) race on the array: serialise them.

// 4 MiB: fits every call with fast_ws(Neff, n_grid) <= 4 MiB (n_grid * Neff a little under 2^20)
constexpr size_t kNoAllocScratchBytes = size_t(4) << 20;
static __device__ __align__(256) unsigned char g_fit_scratch[kNoAllocScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void* g_scratch_addr[kMaxDevices] = {};
void* g_scratch_ctx[kMaxDevices] = {};  // the driver context each address was looked up in

// the driver's cuCtxGetCurrent, from the runtime's entry-point table (no link-time dependency on the driver library)
using CtxGetCurrentFn = int (*)(void**);
CtxGetCurrentFn ctx_get_current() {
    static CtxGetCurrentFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<CtxGetCurrentFn>(f);
    }();
    return fn;
}

// Device address of g_fit_scratch in the current context.  In host code the array's name is only a host-side
// stand-in, so the address comes from the runtime; it is kept per device together with the driver context it was
// looked up in, and looked up again when the current context differs (after cudaDeviceReset, which reloads the
// module, or in a non-primary context).  The lookup itself does not allocate once the module is loaded.
int scratch_address(void** out) {
    int dev = 0;
    FLMM_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(FLMM_ERR_DEVICE, "device index %d out of range", dev);
    void* ctx = nullptr;
    if (CtxGetCurrentFn f = ctx_get_current()) {
        if (f(&ctx) != 0) ctx = nullptr;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev] || ctx == nullptr || ctx != g_scratch_ctx[dev]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_fit_scratch);
        if (e != cudaSuccess || !ptr)
            return fail(FLMM_ERR_CUDA, "cudaGetSymbolAddress(g_fit_scratch) on device %d: %s", dev,
                        cudaGetErrorString(e));
        g_scratch_addr[dev] = ptr;
        g_scratch_ctx[dev] = ctx;
    }
    *out = g_scratch_addr[dev];
    return FLMM_OK;
}

}  // namespace

extern "C" int flmm_fit_delta_fast_noalloc(const double* s, int Neff, const float* UYt, int64_t ldu, int P, int n_grid,
                                           double lo, double hi, int refine, double* log_delta, int32_t* grid_idx,
                                           void* stream) {
    FLMM_REQUIRE(s && UYt && log_delta && grid_idx && Neff > 0 && n_grid > 0 && ldu >= Neff && P >= 0,
                 "flmm_fit_delta_fast_noalloc: bad arguments");
    const size_t need = fast_ws(Neff, n_grid);
    if (need > kNoAllocScratchBytes)
        return fail(FLMM_ERR_WORKSPACE,
                    "flmm_fit_delta_fast_noalloc: n_grid * Neff = %lld needs %zu bytes of scratch, more than the fixed "
                    "%zu; use flmm_fit_delta_fast with caller-provided workspace",
                    static_cast<long long>(n_grid) * Neff, need, kNoAllocScratchBytes);
    void* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    if (P == 0) return FLMM_OK;
    return launch_fast_fit(s, Neff, UYt, ldu, P, n_grid, lo, hi, refine, log_delta, grid_idx, scratch,
                           as_stream(stream));
}
