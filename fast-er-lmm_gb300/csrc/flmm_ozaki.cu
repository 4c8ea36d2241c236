// FP64-accurate product of the eigenvector refinement on the FP16 tensor cores: W[b] = U~[b] A[b]^T (A symmetric,
// so row m of A is column m), for the residuals r_j = A u_j - lambda_j u_j of the Ogita-Aishima step
// (flmm_eigh_refine.cu).
//
// Method: the error-free splitting of Ozaki, Ogita, Oishi and Rump ("Error-free transformations of matrix
// multiplication by using fast routines of matrix multiplication and its applications", Numer. Algorithms 59, 2012)
// run on FP16 tensor cores with FP32 accumulation, as in Mukunoki, Ozaki, Ogita and Imamura ("DGEMM using Tensor
// Cores, and Its Accurate and Reproducible Versions", ISC 2020).  Every row of both operands becomes a sum of digit
// planes on one exponent per row,
//     x = 2^(e - 6) (d_0 + d_1 2^-7 + d_2 2^-14 + ...),   d_t integers, |d_t| <= 64,
// e the binary exponent of the row's largest |x| (so |x| 2^(6 - e) < 64).  A digit is exact in FP16 and the product
// of two digits is an integer of at most 12 bits, so a sum of up to 4,096 such products -- four plane pairs over a
// reduction of 1,024 -- stays within 2^24 and the tensor core's FP32 accumulation adds it without rounding.
// U (FP32) takes 4 planes (28 bits below its row's leading bit, which holds every element within 2^-3 of the row
// maximum exactly and rounds smaller ones to the same absolute grid); the product is the exact product of that
// rounded U~, which the refinement then uses in place of U (it is an equally good iterate, and the residuals must
// belong to the vectors they correct).  A (FP64) takes 7 planes (48 bits).  Plane pairs (i, j) of equal level
// l = i + j carry the same weight 2^(-7 l) and share one accumulator in tensor memory; levels 0..7 are kept (25
// pairs; the first dropped level weighs 2^-56).  Levels 0..3 are exact by the bound above; levels 4..7 weigh at
// most 2^-28 and round at 2^-18 of themselves over 1,024 terms.  The leading digits of most elements are small
// (off-diagonal kinship entries and most eigenvector entries lie well below their row's maximum), so the
// lower levels carry more than their nominal weight: on a 600 x 600 kinship-like test the product's error was
// 1.3e-14 of sum |u||a| with eight levels and 8e-14 with seven, against 3.2e-13 for double-FP32.  Per output,
//     W = 2^(e_i + e_m - 12) sum_l 2^(-7 l) C_l
// is combined in double-FP32 (TwoSum) and stored in FP64.  Reductions longer than 1,024 run as several launches
// that add into W.
//
// Kernel: persistent, one CTA per SM, 320 threads -- warp 0 issues the TMA loads (per 32-deep k-block the 4 U
// planes of 128 rows and the 7 A planes of 64 rows, 60 KB, three stages), warp 1 owns tensor memory and issues the
// 50 MMAs of a k-block (M = 128, N = 64, K = 16, kind::f16), warps 2..9 combine the 8 level accumulators of a tile
// (all 512 columns) and store it.  Tiles are (matrix, 128 U rows, 64 A rows).
#include <cuda.h>
#include <cuda_fp16.h>
#include <math.h>

#include <cstdlib>
#include <cstring>
#include <mutex>

#include "flmm_common.cuh"
#include "flmm_tc.cuh"

using namespace flmm;
using namespace flmm::tc;

namespace {

constexpr int kDigitShift = 7;    // bits per digit below the first
constexpr int kMaxChunk = 1024;   // reduction of one launch (exact accumulation bound)
constexpr int kBM = 128;          // A-side rows per tile (TMEM lanes)
constexpr int kBN = 64;           // B-side rows per tile (columns of one level accumulator)
constexpr int kBK = 32;           // reduction depth of one stage (64-byte rows, 64-byte swizzle)
constexpr int kATile = kBM * kBK * 2;                                   // 8 KB: one A-side plane
constexpr int kBTile = kBN * kBK * 2;                                   // 4 KB: one B-side plane
constexpr uint32_t kSBO = 8u * kBK * 2u;                                // bytes between 8-row groups
constexpr uint32_t kSwizzle64 = 4u;
constexpr int kThreads = 320;
constexpr int kEpilogueThreads = 256;

// One configuration of the digit-plane product: PA planes on the A side (128 rows per tile), PB on the B side (64),
// levels 0 .. LV - 1 kept, FP64 output (the refinement's A U) or FP32 output (its corrections).
template <int PA, int PB, int LV, bool F64>
struct OzCfg {
    static constexpr int kStageBytes = PA * kATile + PB * kBTile;
    static constexpr int kStages = (192 * 1024) / kStageBytes < 4 ? (192 * 1024) / kStageBytes : 4;
    static constexpr int kTmemCols = LV * kBN <= 256 ? 256 : 512;
    static constexpr int kSmemBytes = kStages * kStageBytes + 256 + 1024;
    static_assert(LV * kBN <= kTmemCols && kTmemCols <= 512, "tensor memory budget");
    static_assert(kStages >= 2, "pipeline depth");
    static_assert(kSmemBytes <= 227 * 1024, "shared memory budget");
};
// Configurations used: the refinement's A U as <4, 7, 8, FP64> (U~ in 4 planes, A in 7, levels 0..7, 25 pairs); the
// corrections u_i . r_j as <3, 3, 3, FP32> (6 pairs on planes 0..2 of either side: the coefficients E_ij are
// themselves corrections and need ~1e-3 relative accuracy) and T U~ as <4, 4, 5, FP32> (13 pairs: FP32 accuracy against the row's largest rotation, which
// reaches 0.25 for nearly degenerate pairs).
constexpr int kUPlanes = 4;
constexpr int kAPlanes = 7;
static_assert(kMaxChunk % kBK == 0, "chunks must start on a k-block");

struct OzMaps {
    CUtensorMap u, a;
};

struct OzArgs {
    int N, batch;
    int k0, klen;        // reduction range of this launch
    const int* eU;       // (batch N) row exponents of the A side
    const int* eA;       // (batch N) row exponents of the B side
    double* W;           // (batch, N, N), FP64 output
    float* C;            // (batch, N, N), FP32 output
    const float* D;      // (batch, N, N) added to the FP32 output, or null
    int accumulate;      // add into the output (launches after the first)
    int* err;
};

// ---- digit planes -------------------------------------------------------------------------------------------

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// U rows (FP32, pitch N): planes[t][row][n] = d_t, expo[row] = e, Ut = U~ (the value the planes represent).  One
// warp per row.  y = u 2^(6 - e) is exact and every remainder step (y - rint(y)) 128 is exact in FP32.
__global__ void k_digits_u(const float* __restrict__ U, int64_t rows, int N, __half* __restrict__ planes,
                           int64_t ldp, int64_t plane_rows, int* __restrict__ expo, float* __restrict__ Ut) {
    const int lane = threadIdx.x & 31;
    const int64_t j = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    if (j >= rows) return;
    const float* u = U + j * N;
    float mx = 0.0f;
    for (int n = lane; n < N; n += 32) mx = fmaxf(mx, fabsf(u[n]));
    mx = warp_max(mx);
    int e = 0;
    frexpf(mx, &e);  // mx = f 2^e with f in [0.5, 1); 0 for an all-zero row
    for (int n = lane; n < N; n += 32) {
        float y = ldexpf(u[n], 6 - e);
        float d[kUPlanes];
#pragma unroll
        for (int t = 0; t < kUPlanes; ++t) {
            d[t] = rintf(y);
            y = (y - d[t]) * 128.0f;
        }
#pragma unroll
        for (int t = 0; t < kUPlanes; ++t) planes[(t * plane_rows + j) * ldp + n] = __float2half_rn(d[t]);
        float r = d[kUPlanes - 1];
#pragma unroll
        for (int t = kUPlanes - 2; t >= 0; --t) r = d[t] + r * (1.0f / 128.0f);
        if (Ut) Ut[j * N + n] = ldexpf(r, e - 6);
    }
    if (lane == 0) expo[j] = e;
}

// A rows (FP64, pitch N): planes and exponents as above, from the double-FP32 pair (fl32(a), fl32(a - fl32(a)))
// (48 bits of each element); the pair is renormalised by TwoSum after every digit, so it stays the exact remainder.
__global__ void k_digits_a(const double* __restrict__ A, int64_t rows, int N, __half* __restrict__ planes,
                           int64_t ldp, int64_t plane_rows, int* __restrict__ expo) {
    const int lane = threadIdx.x & 31;
    const int64_t j = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    if (j >= rows) return;
    const double* a = A + j * N;
    float mx = 0.0f;
    for (int n = lane; n < N; n += 32) mx = fmaxf(mx, fabsf(static_cast<float>(a[n])));
    mx = warp_max(mx);
    int e = 0;
    frexpf(mx, &e);
    for (int n = lane; n < N; n += 32) {
        const double v = a[n];
        const float h = static_cast<float>(v);
        const float l = static_cast<float>(v - static_cast<double>(h));
        float yh = ldexpf(h, 6 - e), yl = ldexpf(l, 6 - e);
#pragma unroll
        for (int t = 0; t < kAPlanes; ++t) {
            const float d = rintf(yh);
            planes[(t * plane_rows + j) * ldp + n] = __float2half_rn(d);
            float s, err;
            two_sum(yh - d, yl, s, err);
            yh = s * 128.0f;
            yl = err * 128.0f;
        }
    }
    if (lane == 0) expo[j] = e;
}

// ---- the tensor-core product ----------------------------------------------------------------------------------

template <int PA, int PB, int LV, bool F64>
__global__ void __launch_bounds__(kThreads, 1) k_ozaki(const __grid_constant__ OzMaps maps, const OzArgs args) {
    using Cfg = OzCfg<PA, PB, LV, F64>;
    constexpr int kStages = Cfg::kStages;
    constexpr int kStageBytes = Cfg::kStageBytes;
    constexpr int kTmemCols = Cfg::kTmemCols;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023u)) & 1023u);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kStages * kStageBytes);
    uint64_t* full = bars;                  // [kStages]
    uint64_t* empty = bars + kStages;       // [kStages]
    uint64_t* acc_full = empty + kStages;   // tile accumulated (MMA -> epilogue)
    uint64_t* acc_empty = acc_full + 1;     // tile combined (epilogue -> MMA)
    uint64_t* final_bar = acc_empty + 1;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(final_bar + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int N = args.N;
    const int tiles_i = (N + kBM - 1) / kBM, tiles_m = (N + kBN - 1) / kBN;
    const int per = tiles_i * tiles_m;
    const int n_tiles = args.batch * per;
    const int n_kb = (args.klen + kBK - 1) / kBK;
    constexpr uint32_t idesc = idesc_f16_f32(kBM, kBN);

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(acc_full, 1);
        mbar_init(acc_empty, kEpilogueThreads);
        mbar_init(final_bar, 1);
        fence_barrier_init();
    }
    if (warp == 0 && lane == 0) {
        tma_prefetch_desc(&maps.u);
        tma_prefetch_desc(&maps.a);
    }
    if (warp == 1) {
        tmem_alloc(tmem_slot, kTmemCols);
        tmem_relinquish();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem_base = *tmem_slot;

    if (warp == 0) {
        // ---- TMA producer ----
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            bool armed[kStages] = {};
            uint32_t armed_phase[kStages] = {};
            bool ok = true;
            for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x) {
                const int b = t / per, rem = t - b * per;
                const int ti = rem / tiles_m, tm = rem - ti * tiles_m;
                for (int kb = 0; kb < n_kb; ++kb) {
                    if (!mbar_wait(&empty[stage], phase ^ 1u, args.err, 11)) { ok = false; break; }
                    mbar_arrive_expect_tx(&full[stage], kStageBytes);
                    armed[stage] = true;
                    armed_phase[stage] = phase;
                    uint8_t* base = smem + stage * kStageBytes;
                    const int x = args.k0 + kb * kBK;
#pragma unroll
                    for (int p = 0; p < PA; ++p)
                        tma_load_2d(base + p * kATile, &maps.u, x, (p * args.batch + b) * N + ti * kBM, &full[stage]);
#pragma unroll
                    for (int p = 0; p < PB; ++p)
                        tma_load_2d(base + PA * kATile + p * kBTile, &maps.a, x,
                                    (p * args.batch + b) * N + tm * kBN, &full[stage]);
                    if (++stage == kStages) { stage = 0; phase ^= 1u; }
                }
            }
            for (int s = 0; s < kStages; ++s)
                if (armed[s]) mbar_drain(&full[s], armed_phase[s]);
        }
    } else if (warp == 1) {
        // ---- MMA issuer: the plane pairs (i, j) with i + j < LV of every 16-deep step, each into its level's
        // accumulator ----
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            uint32_t tphase = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x) {
                if (!mbar_wait(acc_empty, tphase ^ 1u, args.err, 12)) break;
                fence_after_sync();
                for (int kb = 0; kb < n_kb; ++kb) {
                    if (!mbar_wait(&full[stage], phase, args.err, 13)) { ok = false; break; }
                    fence_after_sync();
                    const uint32_t sbase = smem_u32(smem + stage * kStageBytes);
#pragma unroll
                    for (int kk = 0; kk < kBK / 16; ++kk) {
#pragma unroll
                        for (int l = 0; l < LV; ++l) {
                            const int i_lo = l - (PB - 1) > 0 ? l - (PB - 1) : 0;
                            const int i_hi = l < PA - 1 ? l : PA - 1;
#pragma unroll
                            for (int i = i_lo; i <= i_hi; ++i) {
                                const int j = l - i;
                                const uint64_t ad = smem_desc(sbase + i * kATile, kSBO, kSwizzle64) + 2u * kk;
                                const uint64_t bd =
                                    smem_desc(sbase + PA * kATile + j * kBTile, kSBO, kSwizzle64) + 2u * kk;
                                const uint32_t acc = (kb > 0 || kk > 0 || i > i_lo) ? 1u : 0u;
                                mma_f16(tmem_base + static_cast<uint32_t>(l * kBN), ad, bd, idesc, acc);
                            }
                        }
                    }
                    mma_commit(&empty[stage]);
                    if (++stage == kStages) { stage = 0; phase ^= 1u; }
                }
                if (!ok) break;
                mma_commit(acc_full);
                tphase ^= 1u;
            }
            mma_commit(final_bar);
            mbar_drain(final_bar, 0);
        }
    } else {
        // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 (thread = one U row) and half (w - 2) / 4 of the
        // tile's 64 columns, in two groups of 16 ----
        const int q = warp & 3;
        const int half = (warp - 2) >> 2;
        const int r = q * 32 + lane;
        const uint32_t tl0 =
            tmem_base + (static_cast<uint32_t>(q * 32) << 16) + static_cast<uint32_t>(half * (kBN / 2));
        uint32_t tphase = 0;
        for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
            if (!mbar_wait(acc_full, tphase, args.err, 14)) break;
            fence_after_sync();
            const int b = t / per, rem = t - b * per;
            const int ti = rem / tiles_m, tm = rem - ti * tiles_m;
            const int i = ti * kBM + r;
            const bool row_ok = i < N;
            const int eu = row_ok ? args.eU[static_cast<int64_t>(b) * N + i] : 0;
            const int64_t orow = (static_cast<int64_t>(b) * N + (row_ok ? i : 0)) * N;
#pragma unroll 1
            for (int g = 0; g < 2; ++g) {
                const int c0 = tm * kBN + half * (kBN / 2) + g * 16;
                const uint32_t ta = tl0 + static_cast<uint32_t>(g * 16);
                float hi[16], lo[16], v[16];
                if constexpr (F64) {
                    // double-FP32 sum of the levels, stored in FP64
                    tmem_ld16_wait(ta, hi);
#pragma unroll
                    for (int c = 0; c < 16; ++c) lo[c] = 0.0f;
#pragma unroll
                    for (int l = 1; l < LV; ++l) {
                        tmem_ld16_wait(ta + static_cast<uint32_t>(l * kBN), v);
                        const float w = ldexpf(1.0f, -kDigitShift * l);
#pragma unroll
                        for (int c = 0; c < 16; ++c) {
                            float s, err;
                            two_sum(hi[c], v[c] * w, s, err);
                            hi[c] = s;
                            lo[c] += err;
                        }
                    }
                } else {
                    // FP32 sum of the levels, smallest first
                    tmem_ld16_wait(ta + static_cast<uint32_t>((LV - 1) * kBN), hi);
                    const float wl = ldexpf(1.0f, -kDigitShift * (LV - 1));
#pragma unroll
                    for (int c = 0; c < 16; ++c) hi[c] *= wl;
#pragma unroll
                    for (int l = LV - 2; l >= 0; --l) {
                        tmem_ld16_wait(ta + static_cast<uint32_t>(l * kBN), v);
                        const float w = ldexpf(1.0f, -kDigitShift * l);
#pragma unroll
                        for (int c = 0; c < 16; ++c) hi[c] = fmaf(v[c], w, hi[c]);
                    }
                }
                if (row_ok) {
#pragma unroll
                    for (int c = 0; c < 16; ++c) {
                        const int m = c0 + c;
                        if (m < N) {
                            const int ex = eu + args.eA[static_cast<int64_t>(b) * N + m] - 12;
                            if constexpr (F64) {
                                const double x = ldexp(static_cast<double>(hi[c]) + static_cast<double>(lo[c]), ex);
                                args.W[orow + m] = args.accumulate ? args.W[orow + m] + x : x;
                            } else {
                                float x = ldexpf(hi[c], ex);
                                if (args.accumulate) x += args.C[orow + m];
                                else if (args.D) x += args.D[orow + m];
                                args.C[orow + m] = x;
                            }
                        }
                    }
                }
            }
            fence_before_sync();
            mbar_arrive(acc_empty);
            tphase ^= 1u;
        }
    }

    fence_before_sync();
    __syncthreads();
    if (warp == 1) {
        fence_after_sync();
        tmem_dealloc(tmem_base, kTmemCols);
    }
}

// Workspace: 11 digit planes in one block (the product's 4 + 7; the corrections reuse them: T over planes 0-1,
// its digits on planes 2-5, the digits of U~^T on planes 6-9, the residuals' digits on planes 4-7) and the row
// exponents of both sides.
struct OzWs {
    __half* planes;
    __half *up, *ap;
    int *eu, *ea;
    int64_t ldp, plane;  // elements per plane: rows x ldp
    size_t bytes;
};

OzWs carve_oz(void* base, int N, int batch) {
    OzWs w{};
    w.ldp = (static_cast<int64_t>(N) + 7) / 8 * 8;
    const size_t rows = static_cast<size_t>(N) * batch;
    w.plane = static_cast<int64_t>(rows) * w.ldp;
    size_t off = 0;
    auto take = [&](size_t nbytes) {
        void* p = base ? static_cast<char*>(base) + off : nullptr;
        off += (nbytes + 1023) / 1024 * 1024;
        return p;
    };
    w.planes = static_cast<__half*>(take(sizeof(__half) * (kUPlanes + kAPlanes) * rows * w.ldp));
    w.up = w.planes;
    w.ap = w.planes ? w.planes + kUPlanes * w.plane : nullptr;
    w.eu = static_cast<int*>(take(sizeof(int) * rows));
    w.ea = static_cast<int*>(take(sizeof(int) * rows));
    w.bytes = off;
    return w;
}

int sm_count_current() {
    int dev = 0, sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 0;
    return sm;
}

// FP32 rows (rows, pitch N) -> 4 digit planes at `planes` (plane stride w.plane) and row exponents; Ut (optional) the
// rounding the planes represent.
int digits_f32(const float* X, int64_t rows, int N, __half* planes, const OzWs& w, int* expo, float* Ut,
               cudaStream_t st) {
    k_digits_u<<<ceil_div(rows * 32, 256), 256, 0, st>>>(X, rows, N, planes, w.ldp, rows, expo, Ut);
    return check_launch("k_digits_u");
}

// The digit-plane product of configuration <PA, PB, LV, F64>: out[b][i][m] = sum over pairs of A-side planes (rows i)
// and B-side planes (rows m), scaled by the row exponents; FP64 into W or FP32 into C (+ D).  Reductions longer than
// kMaxChunk run as several launches that add into the output.
template <int PA, int PB, int LV, bool F64>
int launch_oz(const __half* aplanes, const int* ea_side, const __half* bplanes, const int* eb_side, int N, int batch,
              const OzWs& w, double* W, float* C, const float* D, cudaStream_t st) {
    using Cfg = OzCfg<PA, PB, LV, F64>;
    const int64_t rows = static_cast<int64_t>(N) * batch;
    if (rows * PB > 0x7fffffffLL || rows * PA > 0x7fffffffLL)
        return fail(FLMM_ERR_ARG, "refine product: too many rows for a TMA map");
    OzMaps maps;
    std::memset(&maps, 0, sizeof(maps));
    int rc;
    if ((rc = tc::make_map_f16(&maps.u, aplanes, static_cast<int>(PA * rows), N, w.ldp, kBK, kBM))) return rc;
    if ((rc = tc::make_map_f16(&maps.a, bplanes, static_cast<int>(PB * rows), N, w.ldp, kBK, kBN))) return rc;
    static std::once_flag attr_once;
    static cudaError_t attr_rc = cudaSuccess;
    std::call_once(attr_once, [] {
        attr_rc = cudaFuncSetAttribute(k_ozaki<PA, PB, LV, F64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       Cfg::kSmemBytes);
    });
    if (attr_rc != cudaSuccess) return fail(FLMM_ERR_CUDA, "k_ozaki: %s", cudaGetErrorString(attr_rc));
    int dev = 0;
    FLMM_CUDA(cudaGetDevice(&dev));
    int* err = device_err_flag(dev);
    if (!err) return fail(FLMM_ERR_CUDA, "refine product: cannot allocate the device error flag");
    const int sm = sm_count_current();
    const int64_t tiles = static_cast<int64_t>(batch) * ((N + kBM - 1) / kBM) * ((N + kBN - 1) / kBN);
    const int grid = static_cast<int>(tiles < sm ? tiles : sm);
    if (grid <= 0) return FLMM_OK;
    for (int k0 = 0; k0 < N; k0 += kMaxChunk) {
        OzArgs a;
        a.N = N;
        a.batch = batch;
        a.k0 = k0;
        a.klen = N - k0 < kMaxChunk ? N - k0 : kMaxChunk;
        a.eU = ea_side;
        a.eA = eb_side;
        a.W = W;
        a.C = C;
        a.D = D;
        a.accumulate = k0 > 0;
        a.err = err;
        k_ozaki<PA, PB, LV, F64><<<grid, kThreads, Cfg::kSmemBytes, st>>>(maps, a);
        if ((rc = check_launch("k_ozaki"))) return rc;
    }
    return FLMM_OK;
}

// batched (N, N) FP32 transpose, 32 x 32 tiles through shared memory
__global__ void k_transpose_f32(const float* __restrict__ X, int N, float* __restrict__ Y) {
    __shared__ float t[32][33];
    const int64_t nn = static_cast<int64_t>(N) * N;
    const float* x = X + blockIdx.z * nn;
    float* y = Y + blockIdx.z * nn;
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int i = by + r, j = bx + threadIdx.x;
        t[r][threadIdx.x] = (i < N && j < N) ? x[static_cast<int64_t>(i) * N + j] : 0.0f;
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int i = bx + r, j = by + threadIdx.x;
        if (i < N && j < N) y[static_cast<int64_t>(i) * N + j] = t[threadIdx.x][r];
    }
}

}  // namespace

namespace flmm {

size_t refine_product_tc_bytes(int N, int batch) { return carve_oz(nullptr, N, batch).bytes; }

// W (batch, N, N) FP64 = U~ A^T with U~ (written to Ut) the digit-plane rounding of U; work of
// refine_product_tc_bytes(N, batch) bytes (1,024-byte aligned).  The digit planes of U~ stay in the workspace for
// refine_m_tc.
int refine_product_tc(const float* U, const double* A, int N, int batch, float* Ut, double* W, void* work,
                      cudaStream_t st) {
    const OzWs w = carve_oz(work, N, batch);
    const int64_t rows = static_cast<int64_t>(N) * batch;
    int rc = digits_f32(U, rows, N, w.up, w, w.eu, Ut, st);
    if (rc) return rc;
    k_digits_a<<<ceil_div(rows * 32, 256), 256, 0, st>>>(A, rows, N, w.ap, w.ldp, rows, w.ea);
    if ((rc = check_launch("k_digits_a"))) return rc;
    return launch_oz<4, 7, 8, true>(w.up, w.eu, w.ap, w.ea, N, batch, w, W, nullptr, nullptr, st);
}

// M[b][i][j] = u~_i . r_j (FP32) from the digit planes of U~ that refine_product_tc left in `work` and the residual
// rows R (batch N, N) FP32.
int refine_m_tc(const float* R, int N, int batch, float* M, void* work, cudaStream_t st) {
    const OzWs w = carve_oz(work, N, batch);
    const int64_t rows = static_cast<int64_t>(N) * batch;
    __half* rp = w.planes + 4 * w.plane;
    int rc = digits_f32(R, rows, N, rp, w, w.ea, nullptr, st);
    if (rc) return rc;
    // levels 0..2 use planes 0..2 of either side only: the fourth planes are not loaded
    return launch_oz<3, 3, 3, false>(w.up, w.eu, rp, w.ea, N, batch, w, nullptr, M, nullptr, st);
}

// U_out = U~ + T U~ (FP32), T (batch, N, N) FP32 at the start of `work` (over planes 0-1), scratch an (batch, N, N)
// FP32 buffer for U~^T.
int refine_update_tc(const float* T, const float* Ut, float* scratch, int N, int batch, float* U_out, void* work,
                     cudaStream_t st) {
    const OzWs w = carve_oz(work, N, batch);
    const int64_t rows = static_cast<int64_t>(N) * batch;
    if (reinterpret_cast<const char*>(T) + sizeof(float) * rows * N > reinterpret_cast<const char*>(w.planes + 2 * w.plane))
        return fail(FLMM_ERR_ARG, "refine update: T overlaps its digit planes");
    const dim3 tg(ceil_div(N, 32), ceil_div(N, 32), batch);
    k_transpose_f32<<<tg, dim3(32, 8), 0, st>>>(Ut, N, scratch);
    int rc = check_launch("k_transpose_f32");
    if (rc) return rc;
    __half* tp = w.planes + 2 * w.plane;
    __half* up = w.planes + 6 * w.plane;
    if ((rc = digits_f32(T, rows, N, tp, w, w.eu, nullptr, st))) return rc;
    if ((rc = digits_f32(scratch, rows, N, up, w, w.ea, nullptr, st))) return rc;
    return launch_oz<4, 4, 5, false>(tp, w.eu, up, w.ea, N, batch, w, nullptr, U_out, Ut, st);
}

}  // namespace flmm
