// Split-precision tensor-core form of the scan.
//
// Operands are carried as FP16 pairs x = (hi + lo) * 2^-e with one power-of-two exponent e per row (chosen so
// the row's largest |x| 2^e lies in [2^14, 2^15)); |x - (hi + lo) 2^-e| <= 2^-22 |x| in the normal range.  A product
// of two split operands is summed as hi*hi + hi*lo + lo*hi (the dropped lo*lo term is below 2^-22 relative), each
// term a tcgen05.mma kind::f16 with FP32 accumulation in tensor memory, and the two row exponents are applied in
// the epilogue.  This gives ~21-bit operand precision at FP16 tensor rate.
//
// One persistent kernel template serves both uses:
//   NG = 1: C = A B^T for the eigenbasis rotations (UY = U_eff^T Y_r, US = U_eff^T S_r; fasterlmm/core.py:518, 629)
//           and the per-chromosome Gram (fasterlmm/io.py:264);
//   NG = 2: the Wald scan (fasterlmm/core.py:649-667): sWy = (w o UY) US^T and sWs = w (US o US)^T accumulated
//           side by side, with beta, var_beta, F, SE, SFVE and the per-column genome max computed in the epilogue.
// Warp roles: warp 0 issues TMA loads, warp 1 owns tensor memory and issues the MMAs, the rest run the epilogue
// (warp w reads TMEM lanes 32 (w % 4) .. +31): warps 2-9 with half of the tile's columns each in the single-CTA
// kernel, warps 2-17 with a quarter each in the pair kernel (four epilogue warps per scheduler, 96 registers a
// thread).  Shared memory holds 192 KB of operand stages.
//
// Accumulation in K chunks: the tensor core's FP32 accumulation does not round to nearest -- every MMA step loses
// about an ulp of the accumulator's magnitude towards zero, so a product over K accumulated in one place carries a
// relative bias that grows linearly with K (measured on GB300 with positive operands: -7e-6 at K = 1,000, -4e-5 at
// K = 5,000, -1.7e-4 at K = 20,000).  Each accumulator therefore covers only a chunk of a few k-blocks: tensor
// memory holds a ring of kSlots chunk accumulators, the MMA issuer starts every chunk afresh in the next free slot,
// and the epilogue warps drain each finished chunk into FP32 registers with round-to-nearest additions.  The bias is
// then that of a 128- or 256-long accumulation (~1e-6) whatever K is, and the ring lets the MMAs of the next chunks
// (and tiles) run while the epilogue drains or finishes a tile.
#include <cudaTypedefs.h>
#include <cuda_fp16.h>
#include <math.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "flmm_common.cuh"
#include "flmm_split.cuh"
#include "flmm_tc.cuh"

using namespace flmm;
using namespace flmm::tc;

namespace {

constexpr int kBM = 128;  // A rows per tile (TMEM lanes)
constexpr int kBN = 128;  // B rows per tile (accumulator columns)
constexpr int kThreads = 320;        // warp 0 TMA, warp 1 MMA, warps 2-9 epilogue
constexpr int kEpilogueThreads = 256;
// the pair kernel: warp 0 TMA, warp 1 MMA, warps 2-17 epilogue (four per TMEM lane quarter, 32 columns each)
constexpr int kPairEpiWarps = 16;
constexpr int kPairThreads = 64 + 32 * kPairEpiWarps;
constexpr int kPairCols = kBN / (kPairEpiWarps / 4);  // accumulator columns per epilogue thread
constexpr int kBK = 64;  // reduction depth of one pipeline stage: 64 gives 3 stages of 64 KB, 32 gives 6 of 32 KB
constexpr int kSlots = 4;  // tensor-memory chunk accumulators of kBN columns (all 512 columns)
// k-blocks of 64 per chunk accumulator (TcArgs::chunk_kb; FLMM_CHUNK_KB / FLMM_WALD_CHUNK_KB override): 2 for the
// GEMMs (Grams and the sWs node table are sums of positive terms); 8 for the Wald product sWy, whose partial sums are
// small next to sWs except for strong associations, and those are recomputed (flmm_wald_refine_f32).  Every drained
// chunk is handed back to the MMA warp with a cluster-scope release arrive, whose memory barrier is the epilogue's
// largest stall: 8-k-block chunks (three hand-backs per tile at K = 995) run the headline launch in 1.995 ms against
// 2.09 ms with 4, with every parity test unchanged.  The Wald kernel's second product (the interpolated sWs, K = R
// nodes) is always one chunk, read straight from its slot in the epilogue.
template <int NG>
constexpr int default_chunk_kb() { return NG == 2 ? 8 : 2; }

template <int NG, int BK>
struct Cfg {
    static constexpr int kTileBytes = 128 * BK * 2;
    static constexpr int kStageBytes = 4 * kTileBytes;  // A hi, A lo, B hi, B lo of one product
    static constexpr int kStages = (BK == 32) ? 6 : 3;   // 192 KB of operand stages either way
    static constexpr uint32_t kSwizzle = (BK == 64) ? 2u : 4u;  // 128-byte / 64-byte swizzle
    static constexpr uint32_t kSBO = 8u * BK * 2u;             // bytes between 8-row groups
    static constexpr int kTmemCols = kSlots * kBN;
    static constexpr int kBarBytes = 256;
    // per epilogue warp: the scales of its 64 variants (two products) and their output rows, staged once per tile
    static constexpr int kEpiWarpBytes = 64 * 4 * 2 + 64 * 8;
    static constexpr int kEpiBytes = 8 * kEpiWarpBytes;
    static constexpr int kSmemBytes = kStages * kStageBytes + kBarBytes + kEpiBytes + 1024;  // + alignment slack
    static_assert(kSmemBytes <= 227 * 1024, "shared memory budget");
};

struct TcMaps {
    CUtensorMap m[8];  // [g * 4 + {0: A hi, 1: A lo, 2: B hi, 3: B lo}]
};

struct TcArgs {
    int Mr, Nr, K;  // A rows, B rows, reduction length of product 0
    int K2;         // reduction length of product 1 (NG == 2)
    int* err;       // device error flag (bounded waits)
    // NG == 1 epilogue
    const float* sa;
    const float* sb;
    float* C;
    int64_t ldc;
    int accumulate;
    // NG == 2 (Wald) epilogue
    const float* sa2;
    const float* sb2;
    const float* rWr;
    const float* rWr0;  // rWr with the unscaled weights w = 1 / (s + delta), for the sWs = 0 clamp
    int n_real;
    float var_df;
    const int64_t* rows;
    double* f;
    double* beta;
    double* se;
    double* sfve;
    int64_t ldo;
    double* max_F;
    // FP64-accurate re-evaluation of strong real tests: a real test whose F exceeds f_refine is listed as
    // (variant index in the chromosome, column) in flags[*flag_count] (up to flag_cap entries) and left out of
    // max_F, which the re-evaluation (flmm_wald_refine_f32) then updates; flag_count == nullptr turns this off
    float f_refine;
    int* flag_count;
    int2* flags;
    int flag_cap;
    // tile order of the persistent schedule (see tile_coords); 0 or 1 = A-major
    int group;
    // k-blocks per chunk accumulator of product 0 (>= 1)
    int chunk_kb;
};

// Tile t of the persistent schedule -> (A block ta, B block tb).  Tiles are visited in groups of `group` A blocks;
// inside a group the B block is the major index, so the group's A blocks stay in L2 while every B block passes
// them once.  group = 1 is A-major order (one A block against every B block), group >= tiles_a B-major order.
// The map is a bijection of [0, tiles_a * tiles_b) for every group >= 1.
__device__ __forceinline__ void tile_coords(int t, int tiles_a, int tiles_b, int group, int& ta, int& tb) {
    const int g = group > 1 ? group : 1;
    const int per = g * tiles_b;
    const int k = t / per;
    const int tl = t - k * per;
    const int ga = min(g, tiles_a - k * g);
    tb = tl / ga;
    ta = k * g + tl % ga;
}

// hardware reciprocal (relative error ~2^-23); arguments here are clamped to normal numbers
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Wald statistics of one epilogue thread: accumulator row p (a column of the phenotype table) against tile columns
// [cbeg, cbeg + 64) (variants): the sums of product 0 in y[] (drained from its chunk accumulators), product 1 read
// from its TMEM slot at tl_s (this thread's lane, column cbeg), the warp's staged scales sc1 / sc2 and output rows.
template <int NC>
__device__ __forceinline__ void wald_rows(const TcArgs& args, const float (&y)[NC], uint32_t tl_s, int p,
                                          bool real_tile, int nvalid, int cbeg, int mbase, const float* sc1,
                                          const float* sc2, const int64_t* rws) {
    static_assert(NC == 32 || NC == 64, "columns per epilogue thread");
    // Wald statistics (fasterlmm/core.py:651-667) in FP32 on the unscaled sums, rearranged so that each test needs
    // two reciprocals: with q = sWy^2 / sWs and rss = rWr - q,
    //     F = beta^2 / var_beta = q df / rss,  beta = sWy / sWs,  var_beta = rss / (df sWs).
    const bool row_ok = p < args.Mr;
    const float sa1 = row_ok ? args.sa[p] : 0.0f;
    const float sa2 = row_ok ? args.sa2[p] : 0.0f;
    const float rwr = row_ok ? args.rWr[p] : 1.0f;
    const float df = args.var_df;
    const bool real = row_ok && p < args.n_real;
    float colmax = -INFINITY;
    bool col_nan = false;
    // one 16-column quarter per iteration; the loop is kept rolled (the statistics' code is long) and the quarter's
    // sums are picked from the register array by selects
#pragma unroll 1
    for (int qd = 0; qd < NC / 16; ++qd) {
        const int c0 = cbeg + 16 * qd;
        float vy[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            if constexpr (NC == 64)
                vy[j] = qd == 0 ? y[j] : (qd == 1 ? y[16 + j] : (qd == 2 ? y[32 + j] : y[48 + j]));
            else
                vy[j] = qd == 0 ? y[j] : y[16 + j];
        }
        float vs[16];
        tmem_ld16_wait(tl_s + static_cast<uint32_t>(16 * qd), vs);
        if (!row_ok) continue;
        const float* s1 = sc1 + 16 * qd;
        const float* s2 = sc2 + 16 * qd;
        if (!real_tile) {
            // permutation columns: F and the column maximum only
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float swy = vy[j] * sa1 * s1[j];
                const float sws = vs[j] * sa2 * s2[j];
                const float qv = swy * swy * rcp_approx(fmaxf(sws, 1e-30f));
                float F = qv * df * rcp_approx(fmaxf(rwr - qv, 1e-30f));
                F = (sws > 0.0f) ? F : 0.0f;  // no variance left: the reference's clamp gives F = 0
                F = (c0 + j < nvalid) ? F : -INFINITY;
                colmax = fmaxf(colmax, F);
                col_nan |= (F != F);
            }
            continue;
        }
        const float inv_df = 1.0f / df;
        const float inv_rwr = 1.0f / rwr;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            if (c0 + j >= nvalid) continue;
            const float swy = vy[j] * sa1 * s1[j];
            const float sws = vs[j] * sa2 * s2[j];
            const float inv_d = rcp_approx(fmaxf(sws, 1e-30f));
            const float qv = swy * swy * inv_d;
            const float rss = fmaxf(rwr - qv, 1e-30f);
            const bool var_ok = sws > 0.0f;
            const float F = var_ok ? qv * df * rcp_approx(rss) : 0.0f;
            bool listed = false;
            if (real && F > args.f_refine && args.flag_count != nullptr) {
                // FP32 cancellation in rss grows with F: the re-evaluation recomputes this test and its max
                const int slot = atomicAdd(args.flag_count, 1);
                if (slot < args.flag_cap) args.flags[slot] = make_int2(mbase + c0 + j, p);
                listed = true;  // also when the list is full: the re-evaluation then scans the chromosome
            }
            if (!listed) colmax = fmaxf(colmax, F);
            col_nan |= (F != F);
            if (!real) continue;
            const int64_t o = rws[16 * qd + j] * args.ldo + p;
            if (var_ok) {
                args.f[o] = F;
                args.beta[o] = swy * inv_d;
                args.se[o] = sqrtf(rss * inv_d * inv_df);
                args.sfve[o] = sqrtf(fmaxf(qv * inv_rwr, 0.0f));
            } else {
                // a variant with no variance left (e.g. monomorphic): the reference clamps sWs to 1e-300 in FP64,
                // which gives beta = F = SFVE = 0 and SE = sqrt(rWr / df / 1e-300)
                args.f[o] = 0.0;
                args.beta[o] = 0.0;
                args.se[o] = sqrt(fmax(static_cast<double>(args.rWr0[p]), 1e-300) / args.var_df / 1e-300);
                args.sfve[o] = 0.0;
            }
        }
    }
    if (row_ok && (colmax >= 0.0f || col_nan)) atomic_max_nonneg(args.max_F + p, col_nan ? NAN : (double)colmax);
}

// C = sa sb^T (acc) for one epilogue thread: accumulator row i against tile columns [cbeg, cbeg + 64) starting at
// column col0 of C, with the drained sums v[], staged column scales sc1.
template <int NC>
__device__ __forceinline__ void gemm_rows(const TcArgs& args, const float (&v)[NC], int i, int col0, int nvalid,
                                          int cbeg, const float* sc1) {
    const bool row_ok = i < args.Mr;
    if (!row_ok) return;
    const float sa = args.sa[i];
    float* crow = args.C + static_cast<int64_t>(i) * args.ldc + col0;
#pragma unroll
    for (int qd = 0; qd < NC / 16; ++qd) {
        const int c0 = cbeg + 16 * qd;
        const float* sc = sc1 + 16 * qd;
        const float* vv = v + 16 * qd;
        float* dst = crow + c0;
        if (c0 + 16 <= nvalid && (reinterpret_cast<uintptr_t>(dst) & 15u) == 0) {
            // a thread owns 16 consecutive outputs of its row: four 16-byte stores
            float4* d4 = reinterpret_cast<float4*>(dst);
#pragma unroll
            for (int q4 = 0; q4 < 4; ++q4) {
                float4 x = make_float4(vv[4 * q4] * sa * sc[4 * q4], vv[4 * q4 + 1] * sa * sc[4 * q4 + 1],
                                       vv[4 * q4 + 2] * sa * sc[4 * q4 + 2], vv[4 * q4 + 3] * sa * sc[4 * q4 + 3]);
                if (args.accumulate) {
                    const float4 o = d4[q4];
                    x.x += o.x;
                    x.y += o.y;
                    x.z += o.z;
                    x.w += o.w;
                }
                d4[q4] = x;
            }
            continue;
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            if (c0 + j < nvalid) {
                const float x = vv[j] * sa * sc[j];
                dst[j] = args.accumulate ? dst[j] + x : x;
            }
        }
    }
}

// Add the 64 accumulator columns at TMEM address tl (this thread's lane) into acc[] (FP32, round to nearest): four
// loads in flight, one wait.
__device__ __forceinline__ void drain64(uint32_t tl, float (&acc)[64]) {
    uint32_t v[64];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%64];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, "
        "[%65];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47}, "
        "[%66];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, "
        "[%67];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31]),
          "=r"(v[32]), "=r"(v[33]), "=r"(v[34]), "=r"(v[35]), "=r"(v[36]), "=r"(v[37]), "=r"(v[38]), "=r"(v[39]),
          "=r"(v[40]), "=r"(v[41]), "=r"(v[42]), "=r"(v[43]), "=r"(v[44]), "=r"(v[45]), "=r"(v[46]), "=r"(v[47]),
          "=r"(v[48]), "=r"(v[49]), "=r"(v[50]), "=r"(v[51]), "=r"(v[52]), "=r"(v[53]), "=r"(v[54]), "=r"(v[55]),
          "=r"(v[56]), "=r"(v[57]), "=r"(v[58]), "=r"(v[59]), "=r"(v[60]), "=r"(v[61]), "=r"(v[62]), "=r"(v[63])
        : "r"(tl), "r"(tl + 16u), "r"(tl + 32u), "r"(tl + 48u)
        : "memory");
#pragma unroll
    for (int j = 0; j < 64; ++j) acc[j] += __uint_as_float(v[j]);
}

// The same for 32 columns: two loads in flight, one wait.
__device__ __forceinline__ void drain32(uint32_t tl, float (&acc)[32]) {
    float a[16], b[16];
    tmem_ld16x2(tl, tl + 16u, a, b);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        acc[j] += a[j];
        acc[16 + j] += b[j];
    }
}

template <int NG, int BK>
__global__ void __launch_bounds__(kThreads, 1) k_tc(const __grid_constant__ TcMaps maps, const TcArgs args) {
    using C = Cfg<NG, BK>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023u)) & 1023u);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + C::kStages * C::kStageBytes);
    uint64_t* full = bars;                          // [kStages]
    uint64_t* empty = bars + C::kStages;            // [kStages]
    uint64_t* slot_full = bars + 2 * C::kStages;    // [kSlots] chunk accumulated (MMA -> epilogue)
    uint64_t* slot_empty = slot_full + kSlots;      // [kSlots] chunk drained (epilogue -> MMA)
    uint64_t* final_bar = slot_empty + kSlots;      // [1]
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(final_bar + 1);
    uint8_t* epi_smem = smem + C::kStages * C::kStageBytes + C::kBarBytes;  // [8][kEpiWarpBytes]

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tiles_b = (args.Nr + kBN - 1) / kBN;
    const int tiles_a = (args.Mr + kBM - 1) / kBM;
    const int n_tiles = tiles_a * tiles_b;
    // the NG products of a tile run one after the other, product g over its own K: k-blocks [0, n_kb0) belong to
    // product 0, [n_kb0, n_kb) to product 1; product 0 is accumulated in chunks of args.chunk_kb k-blocks, product
    // 1 in one chunk
    const int n_kb0 = (args.K + BK - 1) / BK;
    const int n_kb = n_kb0 + (NG == 2 ? (args.K2 + BK - 1) / BK : 0);
    constexpr uint32_t idesc = idesc_f16_f32(kBM, kBN);

    if (threadIdx.x == 0) {
        for (int s = 0; s < C::kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < kSlots; ++b) {
            mbar_init(&slot_full[b], 1);
            mbar_init(&slot_empty[b], kEpilogueThreads);
        }
        mbar_init(final_bar, 1);
        fence_barrier_init();
    }
    if (warp == 0 && lane == 0) {
        for (int i = 0; i < NG * 4; ++i) tma_prefetch_desc(&maps.m[i]);
    }
    if (warp == 1) {
        tmem_alloc(tmem_slot, C::kTmemCols);
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
            bool armed[C::kStages] = {};
            uint32_t armed_phase[C::kStages] = {};
            bool ok = true;
            for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x) {
                int ta, tb;
                tile_coords(t, tiles_a, tiles_b, args.group, ta, tb);
                for (int kb = 0; kb < n_kb; ++kb) {
                    if (!mbar_wait(&empty[stage], phase ^ 1u, args.err, 1)) { ok = false; break; }
                    mbar_arrive_expect_tx(&full[stage], C::kStageBytes);
                    armed[stage] = true;
                    armed_phase[stage] = phase;
                    uint8_t* base = smem + stage * C::kStageBytes;
                    const int g = kb < n_kb0 ? 0 : 1;
                    const int kx = (kb - g * n_kb0) * BK;
                    tma_load_2d(base + 0 * C::kTileBytes, &maps.m[g * 4 + 0], kx, ta * kBM, &full[stage]);
                    tma_load_2d(base + 1 * C::kTileBytes, &maps.m[g * 4 + 1], kx, ta * kBM, &full[stage]);
                    tma_load_2d(base + 2 * C::kTileBytes, &maps.m[g * 4 + 2], kx, tb * kBN, &full[stage]);
                    tma_load_2d(base + 3 * C::kTileBytes, &maps.m[g * 4 + 3], kx, tb * kBN, &full[stage]);
                    if (++stage == C::kStages) { stage = 0; phase ^= 1u; }
                }
            }
            // never leave the CTA with copies still landing in shared memory
            for (int s = 0; s < C::kStages; ++s)
                if (armed[s]) mbar_drain(&full[s], armed_phase[s]);
        }
    } else if (warp == 1) {
        // ---- MMA issuer: every chunk starts afresh in the next slot of the ring ----
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            int slot = 0;
            uint32_t sphase = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x) {
                for (int kc = 0, kc_end = 0; kc < n_kb && ok; kc = kc_end) {
                    kc_end = kc < n_kb0 ? min(kc + args.chunk_kb, n_kb0) : n_kb;
                    if (!mbar_wait(&slot_empty[slot], sphase ^ 1u, args.err, 2)) { ok = false; break; }
                    fence_after_sync();
                    const uint32_t d = tmem_base + static_cast<uint32_t>(slot * kBN);
                    for (int kb = kc; kb < kc_end; ++kb) {
                        if (!mbar_wait(&full[stage], phase, args.err, 3)) { ok = false; break; }
                        fence_after_sync();
                        const uint32_t sbase = smem_u32(smem + stage * C::kStageBytes);
#pragma unroll
                        for (int kk = 0; kk < BK / 16; ++kk) {
                            const uint64_t ah = smem_desc(sbase + 0 * C::kTileBytes, C::kSBO, C::kSwizzle) + 2u * kk;
                            const uint64_t al = smem_desc(sbase + 1 * C::kTileBytes, C::kSBO, C::kSwizzle) + 2u * kk;
                            const uint64_t bh = smem_desc(sbase + 2 * C::kTileBytes, C::kSBO, C::kSwizzle) + 2u * kk;
                            const uint64_t bl = smem_desc(sbase + 3 * C::kTileBytes, C::kSBO, C::kSwizzle) + 2u * kk;
                            mma_f16(d, ah, bh, idesc, (kb != kc || kk) ? 1u : 0u);
                            mma_f16(d, ah, bl, idesc, 1u);
                            mma_f16(d, al, bh, idesc, 1u);
                        }
                        mma_commit(&empty[stage]);
                        if (++stage == C::kStages) { stage = 0; phase ^= 1u; }
                    }
                    if (!ok) break;
                    mma_commit(&slot_full[slot]);
                    if (++slot == kSlots) { slot = 0; sphase ^= 1u; }
                }
            }
            // every MMA this thread issued has completed before tensor memory is released
            mma_commit(final_bar);
            mbar_drain(final_bar, 0);
        }
    } else {
        // ---- epilogue: warps 2..9.  Warp w reads TMEM lanes 32 (w % 4) .. +31 (thread = one accumulator row) and
        // half (w - 2) / 4 of the tile's columns, so two warps share each lane quarter.  Each warp stages the scales
        // (and output rows) of its 64 variants in its own shared-memory slot before draining the chunks, so those
        // loads overlap the MMAs instead of stalling the epilogue.
        const int q = warp & 3;
        const int cbeg = ((warp - 2) >> 2) * (kBN / 2);
        const int r = q * 32 + lane;
        float* sc1 = reinterpret_cast<float*>(epi_smem + (warp - 2) * C::kEpiWarpBytes);  // [64]
        float* sc2 = sc1 + 64;                                                           // [64]
        int64_t* rws = reinterpret_cast<int64_t*>(sc2 + 64);                             // [64]
        const uint32_t tl0 = tmem_base + (static_cast<uint32_t>(q * 32) << 16) + static_cast<uint32_t>(cbeg);
        int slot = 0;
        uint32_t sphase = 0;
        bool ok = true;
        for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x) {
            int ta, tb;
            tile_coords(t, tiles_a, tiles_b, args.group, ta, tb);
            const int nvalid = min(kBN, args.Nr - tb * kBN);  // columns of this tile inside B
            const bool real_tile = NG == 2 && ta * kBM < args.n_real;  // uniform over the CTA
            __syncwarp();  // every lane is done with the previous tile's slot
            for (int k = lane; k < kBN / 2; k += 32) {
                const int c = cbeg + k;
                const int m = tb * kBN + c;
                const bool okc = c < nvalid;
                sc1[k] = okc ? args.sb[m] : 0.0f;
                if constexpr (NG == 2) {
                    sc2[k] = okc ? args.sb2[m] : 0.0f;
                    if (real_tile) rws[k] = okc ? args.rows[m] : 0;
                }
            }
            __syncwarp();
            float acc0[64];
#pragma unroll
            for (int j = 0; j < 64; ++j) acc0[j] = 0.0f;
            // product 0: drain every chunk into acc0 and hand its slot back
            for (int kc = 0, kc_end = 0; kc < n_kb0; kc = kc_end) {
                kc_end = min(kc + args.chunk_kb, n_kb0);
                if (!mbar_wait(&slot_full[slot], sphase, args.err, 4)) { ok = false; break; }
                fence_after_sync();
                drain64(tl0 + static_cast<uint32_t>(slot * kBN), acc0);
                fence_before_sync();
                mbar_arrive(&slot_empty[slot]);
                if (++slot == kSlots) { slot = 0; sphase ^= 1u; }
            }
            if (!ok) break;
            const int i = ta * kBM + r;  // A row
            if constexpr (NG == 1) {
                gemm_rows(args, acc0, i, tb * kBN, nvalid, cbeg, sc1);
            } else {
                // product 1 (one chunk) is read from its slot by the statistics, then the slot is handed back
                if (!mbar_wait(&slot_full[slot], sphase, args.err, 4)) { ok = false; break; }
                fence_after_sync();
                wald_rows(args, acc0, tl0 + static_cast<uint32_t>(slot * kBN), i, real_tile, nvalid, cbeg, tb * kBN,
                          sc1, sc2, rws);
                fence_before_sync();
                mbar_arrive(&slot_empty[slot]);
                if (++slot == kSlots) { slot = 0; sphase ^= 1u; }
            }
        }
    }

    fence_before_sync();
    __syncthreads();
    if (warp == 1) {
        fence_after_sync();
        tmem_dealloc(tmem_base, C::kTmemCols);
    }
}

// ---- the tcgen05 kernels on CTA pairs -----------------------------------------------------------------------------
// k_pair<NG> is k_tc<NG, 64> run on CTA pairs (NG = 2: the Wald scan, NG = 1: the split GEMM).
// Each tile is 256 A rows (e.g. phenotype columns) x 128 B rows (e.g. variants), run by a cluster of two CTAs with
// tcgen05.mma.cta_group::2 (M = 256, N = 128): CTA r of the pair loads A rows 128 r .. +127 and B rows 64 r .. +63
// of the tile into its own shared memory, the even CTA issues the MMAs, and each CTA's tensor memory receives its
// 128 A rows against all 128 B rows, so the epilogue is the single-CTA one.  Per SM, one MMA step reads 128 + 64
// operand rows from shared memory instead of 128 + 128, and a pipeline stage is 48 KB instead of 64 KB: shared
// memory bandwidth is what bounds the single-CTA form.
//
// Synchronisation: both CTAs' TMA loads of a stage complete on the even CTA's full[stage] (its producer expects the
// pair's bytes); the MMA issuer's commits arrive on empty[stage], slot_full[] and the final barrier of both CTAs
// (multicast); the epilogue warps of both CTAs arrive on the even CTA's slot_empty[] (16 warps) once they have
// drained a chunk.  Every wait is bounded as in the single-CTA kernel.
template <int NG>
struct PairCfg {
    static constexpr int kBK = 64;
    static constexpr int kATileBytes = 128 * kBK * 2;                      // 16 KB: 128 A rows of one half
    static constexpr int kBTileBytes = 64 * kBK * 2;                       // 8 KB: 64 B rows of one half
    static constexpr int kStageBytes = 2 * kATileBytes + 2 * kBTileBytes;  // A hi, A lo, B hi, B lo
    static constexpr int kStages = 4;
    static constexpr uint32_t kSwizzle = 2u;   // 128-byte
    static constexpr uint32_t kSBO = 1024u;    // bytes between 8-row groups
    static constexpr int kTmemCols = kSlots * kBN;  // the ring of chunk accumulators
    static constexpr int kBarBytes = 256;
    static constexpr int kEpiWarpBytes = kPairCols * 4 * 2 + kPairCols * 8;
    static constexpr int kEpiBytes = kPairEpiWarps * kEpiWarpBytes;
    static constexpr int kSmemBytes = kStages * kStageBytes + kBarBytes + kEpiBytes + 1024;
    static_assert(kSmemBytes <= 227 * 1024, "shared memory budget");
};

constexpr int kPairRows = 256;  // A rows per pair tile


template <int NG>
__global__ void __launch_bounds__(kPairThreads, 1) k_pair(const __grid_constant__ TcMaps maps, const TcArgs args) {
    using C = PairCfg<NG>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023u)) & 1023u);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + C::kStages * C::kStageBytes);
    uint64_t* full = bars;                          // [kStages], used in the even CTA
    uint64_t* empty = bars + C::kStages;            // [kStages]
    uint64_t* slot_full = bars + 2 * C::kStages;    // [kSlots] chunk accumulated (MMA -> both CTAs' epilogues)
    uint64_t* slot_empty = slot_full + kSlots;      // [kSlots] chunk drained by both CTAs, used in the even CTA
    uint64_t* final_bar = slot_empty + kSlots;      // [1]
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(final_bar + 1);
    uint8_t* epi_smem = smem + C::kStages * C::kStageBytes + C::kBarBytes;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = cluster_ctarank();
    const bool leader = rank == 0;
    const int cl = static_cast<int>(cluster_id_x()), n_cl = static_cast<int>(cluster_count_x());
    const int tiles_b = (args.Nr + kBN - 1) / kBN;
    const int tiles_a = (args.Mr + kPairRows - 1) / kPairRows;
    const int n_tiles = tiles_a * tiles_b;
    const int n_kb0 = (args.K + C::kBK - 1) / C::kBK;
    const int n_kb = n_kb0 + (NG == 2 ? (args.K2 + C::kBK - 1) / C::kBK : 0);
    constexpr uint32_t idesc = idesc_f16_f32(kPairRows, kBN);

    if (threadIdx.x == 0) {
        for (int s = 0; s < C::kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < kSlots; ++b) {
            mbar_init(&slot_full[b], 1);
            mbar_init(&slot_empty[b], 2 * kPairEpiWarps);
        }
        mbar_init(final_bar, 1);
        fence_barrier_init();
    }
    if (warp == 0 && lane == 0) {
        for (int i = 0; i < NG * 4; ++i) tma_prefetch_desc(&maps.m[i]);
    }
    if (warp == 1) {
        tmem_alloc_pair(tmem_slot, C::kTmemCols);
        tmem_relinquish_pair();
    }
    fence_before_sync();
    __syncwarp();
    cluster_sync();  // barriers initialised and tensor memory allocated in both CTAs
    fence_after_sync();
    const uint32_t tmem_base = *tmem_slot;

    if (warp == 0) {
        // ---- TMA producer (both CTAs): this CTA's halves of the tile, counted on the even CTA's full[] ----
        if (lane == 0) {
            const uint32_t full0 = map_to_rank(smem_u32(full), 0);
            int stage = 0;
            uint32_t phase = 0;
            bool armed[C::kStages] = {};
            uint32_t armed_phase[C::kStages] = {};
            bool ok = true;
            for (int t = cl; t < n_tiles && ok; t += n_cl) {
                int ta, tb;
                tile_coords(t, tiles_a, tiles_b, args.group, ta, tb);
                const int arow = ta * kPairRows + static_cast<int>(rank) * 128;
                const int brow = tb * kBN + static_cast<int>(rank) * (kBN / 2);
                for (int kb = 0; kb < n_kb; ++kb) {
                    if (!mbar_wait(&empty[stage], phase ^ 1u, args.err, 1)) { ok = false; break; }
                    if (leader) {
                        mbar_arrive_expect_tx(&full[stage], 2 * C::kStageBytes);
                        armed[stage] = true;
                        armed_phase[stage] = phase;
                    }
                    uint8_t* base = smem + stage * C::kStageBytes;
                    const uint32_t bar = full0 + static_cast<uint32_t>(stage * 8);
                    const int g = kb < n_kb0 ? 0 : 1;
                    const int kx = (kb - g * n_kb0) * C::kBK;
                    tma_load_2d_pair(base, &maps.m[g * 4 + 0], kx, arow, bar);
                    tma_load_2d_pair(base + C::kATileBytes, &maps.m[g * 4 + 1], kx, arow, bar);
                    tma_load_2d_pair(base + 2 * C::kATileBytes, &maps.m[g * 4 + 2], kx, brow, bar);
                    tma_load_2d_pair(base + 2 * C::kATileBytes + C::kBTileBytes, &maps.m[g * 4 + 3], kx, brow, bar);
                    if (++stage == C::kStages) { stage = 0; phase ^= 1u; }
                }
            }
            if (leader) {
                // the pair's copies of every armed phase have landed before the CTAs leave
                for (int s = 0; s < C::kStages; ++s)
                    if (armed[s]) mbar_drain(&full[s], armed_phase[s]);
            } else if (*reinterpret_cast<volatile int*>(args.err) != 0) {
                // the even CTA may have stopped waiting on this CTA's last copies: give them time to land
                for (int i = 0; i < 100; ++i) __nanosleep(1000);
            }
        }
    } else if (warp == 1) {
        if (leader && lane == 0) {
            // ---- MMA issuer (even CTA): every chunk starts afresh in the next slot of the ring ----
            int stage = 0;
            uint32_t phase = 0;
            int slot = 0;
            uint32_t sphase = 0;
            bool ok = true;
            for (int t = cl; t < n_tiles && ok; t += n_cl) {
                for (int kc = 0, kc_end = 0; kc < n_kb && ok; kc = kc_end) {
                    kc_end = kc < n_kb0 ? min(kc + args.chunk_kb, n_kb0) : n_kb;
                    if (!mbar_wait_cluster(&slot_empty[slot], sphase ^ 1u, args.err, 2)) { ok = false; break; }
                    fence_after_sync();
                    const uint32_t d = tmem_base + static_cast<uint32_t>(slot * kBN);
                    for (int kb = kc; kb < kc_end; ++kb) {
                        if (!mbar_wait(&full[stage], phase, args.err, 3)) { ok = false; break; }
                        fence_after_sync();
                        const uint32_t sbase = smem_u32(smem + stage * C::kStageBytes);
#pragma unroll
                        for (int kk = 0; kk < C::kBK / 16; ++kk) {
                            const uint64_t ah = smem_desc(sbase, C::kSBO, C::kSwizzle) + 2u * kk;
                            const uint64_t al = smem_desc(sbase + C::kATileBytes, C::kSBO, C::kSwizzle) + 2u * kk;
                            const uint64_t bh = smem_desc(sbase + 2 * C::kATileBytes, C::kSBO, C::kSwizzle) + 2u * kk;
                            const uint64_t bl =
                                smem_desc(sbase + 2 * C::kATileBytes + C::kBTileBytes, C::kSBO, C::kSwizzle) + 2u * kk;
                            mma_f16_pair(d, ah, bh, idesc, (kb != kc || kk) ? 1u : 0u);
                            mma_f16_pair(d, ah, bl, idesc, 1u);
                            mma_f16_pair(d, al, bh, idesc, 1u);
                        }
                        mma_commit_pair(&empty[stage], 3);
                        if (++stage == C::kStages) { stage = 0; phase ^= 1u; }
                    }
                    if (!ok) break;
                    mma_commit_pair(&slot_full[slot], 3);
                    if (++slot == kSlots) { slot = 0; sphase ^= 1u; }
                }
            }
            mma_commit_pair(final_bar, 3);
            mbar_drain(final_bar, 0);
        } else if (lane == 0) {
            // odd CTA: its shared and tensor memory stay live until the even CTA's last MMA has completed
            mbar_drain(final_bar, 0);
        }
    } else {
        // ---- epilogue (both CTAs): warps 2..17, warp w reads TMEM lanes 32 (w % 4) .. +31 (thread = one accumulator
        // row of this CTA's half of the pair tile) and quarter (w - 2) / 4 of the tile's columns: four warps per lane
        // quarter, so that each scheduler has four epilogue warps to hide the epilogue's latencies with ----
        const int q = warp & 3;
        const int cbeg = ((warp - 2) >> 2) * kPairCols;
        const int r = q * 32 + lane;
        float* sc1 = reinterpret_cast<float*>(epi_smem + (warp - 2) * C::kEpiWarpBytes);
        float* sc2 = sc1 + kPairCols;
        int64_t* rws = reinterpret_cast<int64_t*>(sc2 + kPairCols);
        const uint32_t slot_empty0 = map_to_rank(smem_u32(slot_empty), 0);
        const uint32_t tl0 = tmem_base + (static_cast<uint32_t>(q * 32) << 16) + static_cast<uint32_t>(cbeg);
        int slot = 0;
        uint32_t sphase = 0;
        bool ok = true;
        for (int t = cl; t < n_tiles && ok; t += n_cl) {
            int ta, tb;
            tile_coords(t, tiles_a, tiles_b, args.group, ta, tb);
            const int nvalid = min(kBN, args.Nr - tb * kBN);
            const int row0 = ta * kPairRows + static_cast<int>(rank) * 128;
            const bool real_tile = NG == 2 && row0 < args.n_real;  // uniform over the CTA
            __syncwarp();
            for (int k = lane; k < kPairCols; k += 32) {
                const int c = cbeg + k;
                const int m = tb * kBN + c;
                const bool okc = c < nvalid;
                sc1[k] = okc ? args.sb[m] : 0.0f;
                if constexpr (NG == 2) {
                    sc2[k] = okc ? args.sb2[m] : 0.0f;
                    if (real_tile) rws[k] = okc ? args.rows[m] : 0;
                }
            }
            __syncwarp();
            float acc0[kPairCols];
#pragma unroll
            for (int j = 0; j < 64; ++j) acc0[j] = 0.0f;
            // product 0: drain every chunk into acc0 and hand its slot back
            for (int kc = 0, kc_end = 0; kc < n_kb0; kc = kc_end) {
                kc_end = min(kc + args.chunk_kb, n_kb0);
                const bool got = mbar_wait(&slot_full[slot], sphase, args.err, 4);
                if (!__all_sync(0xffffffffu, got)) { ok = false; break; }
                fence_after_sync();
                drain32(tl0 + static_cast<uint32_t>(slot * kBN), acc0);
                fence_before_sync();
                __syncwarp();
                if (lane == 0) mbar_arrive_cluster_relaxed(slot_empty0 + static_cast<uint32_t>(slot * 8));
                if (++slot == kSlots) { slot = 0; sphase ^= 1u; }
            }
            if (!ok) break;
            if constexpr (NG == 1) {
                gemm_rows(args, acc0, row0 + r, tb * kBN, nvalid, cbeg, sc1);
            } else {
                // product 1 (one chunk) is read from its slot by the statistics, then the slot is handed back
                const bool got = mbar_wait(&slot_full[slot], sphase, args.err, 4);
                if (!__all_sync(0xffffffffu, got)) { ok = false; break; }
                fence_after_sync();
                wald_rows(args, acc0, tl0 + static_cast<uint32_t>(slot * kBN), row0 + r, real_tile, nvalid, cbeg,
                          tb * kBN, sc1, sc2, rws);
                fence_before_sync();
                __syncwarp();
                if (lane == 0) mbar_arrive_cluster_relaxed(slot_empty0 + static_cast<uint32_t>(slot * 8));
                if (++slot == kSlots) { slot = 0; sphase ^= 1u; }
            }
        }
    }

    fence_before_sync();
    __syncwarp();
    cluster_sync();  // no CTA leaves while its peer may still signal its barriers or read its operands
    if (warp == 1) {
        fence_after_sync();
        tmem_dealloc_pair(tmem_base, C::kTmemCols);
    }
}

// ---- operand preparation ---------------------------------------------------------------------------------------

constexpr int kSplitCache = 32;  // per-lane register cache of k_split_rows: rows up to 1,024 entries

// One warp per row, eight rows per 256-thread block: the row's largest |x|, then the split.  FP64 inputs are rounded
// to FP32 first (2^-24 relative, below the split's 2^-22), which keeps the per-element work off the FP64 pipe (a
// small fraction of the FP32 rate on this GPU).
template <typename T>
__global__ void __launch_bounds__(256)
k_split_rows(const T* __restrict__ X, int64_t ldx, int rows, int K, __half* __restrict__ hi,
             __half* __restrict__ lo, int64_t ldo, float* __restrict__ scale) {
    const int lane = threadIdx.x & 31;
    const int64_t r = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    if (r >= rows) return;
    const T* x = X + r * ldx;
    // rows of up to 32 * kSplitCache entries are read and rounded once, into registers, for both passes
    float xv[kSplitCache];
    const bool cached = K <= 32 * kSplitCache;
    float amax = 0.0f;
    if (cached) {
#pragma unroll
        for (int i = 0; i < kSplitCache; ++i) {
            const int k = lane + 32 * i;
            xv[i] = k < K ? static_cast<float>(x[k]) : 0.0f;
        }
#pragma unroll
        for (int i = 0; i < kSplitCache; ++i) amax = fmaxf(amax, fabsf(xv[i]));
    } else {
#pragma unroll 4
        for (int k = lane; k < K; k += 32) amax = fmaxf(amax, fabsf(static_cast<float>(x[k])));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    int e;
    const float mul = row_scale_exp(amax, &e);
    if (cached) {
#pragma unroll
        for (int i = 0; i < kSplitCache; ++i) {
            const int k = lane + 32 * i;
            if (k < K) split_store(xv[i], mul, hi, lo, r * ldo + k);
        }
    } else {
#pragma unroll 4
        for (int k = lane; k < K; k += 32) split_store(static_cast<float>(x[k]), mul, hi, lo, r * ldo + k);
    }
    if (lane == 0) scale[r] = ldexpf(1.0f, -e);
}

// The same split with one 256-thread block per row, for long rows (the kinship markers' rows span every marker).
template <typename T>
__global__ void __launch_bounds__(256)
k_split_long_rows(const T* __restrict__ X, int64_t ldx, int rows, int K, __half* __restrict__ hi,
                  __half* __restrict__ lo, int64_t ldo, float* __restrict__ scale) {
    __shared__ float red[8];
    const int64_t r = blockIdx.x;
    if (r >= rows) return;
    const T* x = X + r * ldx;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    float amax = 0.0f;
#pragma unroll 4
    for (int k = threadIdx.x; k < K; k += 256) amax = fmaxf(amax, fabsf(static_cast<float>(x[k])));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    if (lane == 0) red[wid] = amax;
    __syncthreads();
    amax = red[0];
#pragma unroll
    for (int w = 1; w < 8; ++w) amax = fmaxf(amax, red[w]);
    int e;
    const float mul = row_scale_exp(amax, &e);
#pragma unroll 4
    for (int k = threadIdx.x; k < K; k += 256) split_store(static_cast<float>(x[k]), mul, hi, lo, r * ldo + k);
    if (threadIdx.x == 0) scale[r] = ldexpf(1.0f, -e);
}

// sWs by interpolation.  sWs(delta) = sum_n US_n^2 / (s_n + delta) depends on the column only through delta.  All
// Wald outputs are unchanged when a column's weights w = 1 / (s + delta) are multiplied by a constant, so the scan
// uses w~ = (shat + delta) / (s + delta) (shat = mean eigenvalue), whose sums vary by a bounded factor over the whole
// delta range even when some s are 0.  f~(x) = sum_n US_n^2 w~_n(e^x) is smooth in x = log delta (poles at distance
// pi from the real axis), so it is evaluated at R equispaced nodes x_r = x0 + r h (h = 1/4) and interpolated at each
// column's x by the 10-point Lagrange polynomial on the nodes around it (interpolation error < 1e-9 relative).  The
// second product of the Wald kernel then has K = R (~90) instead of K = Neff.
constexpr int kInterpPoints = 10;
constexpr int kPrepCache = 32;  // per-lane register cache of k_wald_prep_columns: columns up to 1,024 entries

// Wald column side (fasterlmm/core.py:639-643): w~ = (shat + delta_p) / (s + delta_p), A1 = w~ o UY split,
// rWr = sum w~ UY^2, and the column's Lagrange weights L (R entries, 10 non-zero) split.  A block of kPrepCols warps
// handles kPrepCols columns.  GB300's FP64 rate is ~1/60 of its FP32 rate, so FP64 is kept off the per-element
// path: the Lagrange weights (FP64 products, one division each) are formed by ten threads per column before the
// warps start, delta = exp(x) comes from a hi / lo split of x in FP32, and rWr is a compensated FP32 sum.  The
// weights use the hardware reciprocal (within 1 ulp, below the split's 2^-22; tests strong enough for rWr's
// rounding to matter are re-evaluated in FP64).
constexpr int kPrepCols = 8;

// 1 / prod_{m != k} (k - m) over m = 0 .. 9, i.e. (-1)^(9-k) / (k! (9-k)!)
__constant__ double kLagrangeInvDen[kInterpPoints] = {
    -1.0 / 362880.0, 1.0 / 40320.0, -1.0 / 10080.0, 1.0 / 4320.0, -1.0 / 2880.0,
    1.0 / 2880.0,    -1.0 / 4320.0, 1.0 / 10080.0,  -1.0 / 40320.0, 1.0 / 362880.0};

__global__ void __launch_bounds__(32 * kPrepCols, 2)
k_wald_prep_columns(const float* __restrict__ s32, int Neff, const float* __restrict__ UYt, int64_t ldu,
                    const double* __restrict__ ld, int P, const float* __restrict__ shat_p, double x0, double h,
                    double inv_h, int R, __half* __restrict__ A1h, __half* __restrict__ A1l, int64_t lda,
                    __half* __restrict__ Lh, __half* __restrict__ Ll, int64_t ldl, float* __restrict__ sa1,
                    float* __restrict__ sl, float* __restrict__ rWr, float* __restrict__ rWr0) {
    __shared__ float lw[kPrepCols][kInterpPoints];
    __shared__ int lbase[kPrepCols];
    const int lane = threadIdx.x & 31, j = threadIdx.x >> 5;
    const int64_t p = static_cast<int64_t>(blockIdx.x) * kPrepCols + j;
    if (p >= P) return;
    const double x = ld[p];
    // Lagrange weights of the column's warp on nodes base .. base + 9 around x, by its lanes 0..9:
    // w_k = prod_{m != k} (t - m) / prod_{m != k} (k - m), the denominators' reciprocals being constants (the FP64
    // pipe is GB300's narrowest, and a division is many of its instructions); only this warp reads them
    if (lane < kInterpPoints) {
        const int k = lane;
        int base = static_cast<int>(floor((x - x0) * inv_h)) - (kInterpPoints / 2 - 1);
        base = max(0, min(base, R - kInterpPoints));
        const double t = (x - (x0 + base * h)) * inv_h;
        double num = 1.0;
#pragma unroll
        for (int m = 0; m < kInterpPoints; ++m)
            if (m != k) num *= t - m;
        lw[j][k] = static_cast<float>(num * kLagrangeInvDen[k]);
        if (k == 0) lbase[j] = base;
    }
    __syncwarp();
    const float xh = static_cast<float>(x);
    const float xl = static_cast<float>(x - static_cast<double>(xh));
    const float delta = expf(xh) * (1.0f + xl);
    const float num = *shat_p + delta;
    const float* u = UYt + p * ldu;
    float m1 = 0.0f, acc = 0.0f, comp = 0.0f;
    // a column of up to 32 * kPrepCache entries is read once and its weighted values kept in registers for the split
    float av[kPrepCache];
    const bool cached = Neff <= 32 * kPrepCache;
    if (cached) {
        // every load of the column first, so they are in flight together (the division's branches would otherwise
        // hold each load back until the previous element is done)
        float uv[kPrepCache], sv[kPrepCache];
#pragma unroll
        for (int i = 0; i < kPrepCache; ++i) {
            const int n = lane + 32 * i;
            uv[i] = n < Neff ? u[n] : 0.0f;
            sv[i] = n < Neff ? s32[n] : 0.0f;
        }
#pragma unroll
        for (int i = 0; i < kPrepCache; ++i) {
            const int n = lane + 32 * i;
            av[i] = 0.0f;
            if (n < Neff) {
                const float un = uv[i];
                const float a = (num * rcp_approx(sv[i] + delta)) * un;
                av[i] = a;
                m1 = fmaxf(m1, fabsf(a));
                neumaier(acc, comp, a * un);
            }
        }
    } else {
        for (int n = lane; n < Neff; n += 32) {
            const float un = u[n];
            const float a = (num * rcp_approx(s32[n] + delta)) * un;
            m1 = fmaxf(m1, fabsf(a));
            neumaier(acc, comp, a * un);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, o));
    const float rwr = warp_sum_pair(acc, comp);
    int e1;
    const float mul1 = row_scale_exp(m1, &e1);
    if (cached) {
#pragma unroll
        for (int i = 0; i < kPrepCache; ++i) {
            const int n = lane + 32 * i;
            if (n < Neff) split_store(av[i], mul1, A1h, A1l, p * lda + n);
        }
    } else {
        for (int n = lane; n < Neff; n += 32)
            split_store((num * rcp_approx(s32[n] + delta)) * u[n], mul1, A1h, A1l, p * lda + n);
    }
    const int base = lbase[j];
    float lm = 0.0f;
#pragma unroll
    for (int k = 0; k < kInterpPoints; ++k) lm = fmaxf(lm, fabsf(lw[j][k]));
    int el;
    const float mull = row_scale_exp(lm, &el);
    for (int r = lane; r < R; r += 32) {
        const int k = r - base;
        const float v = (k >= 0 && k < kInterpPoints) ? lw[j][k] : 0.0f;
        split_store(v, mull, Lh, Ll, p * ldl + r);
    }
    if (lane == 0) {
        sa1[p] = ldexpf(1.0f, -e1);
        sl[p] = ldexpf(1.0f, -el);
        rWr[p] = fmaxf(rwr, 0.0f);
        rWr0[p] = fmaxf(rwr, 0.0f) / num;  // 0 for an all-zero column: the epilogue applies the reference's floor
    }
}

// normalised weights at the interpolation nodes: W~[r, n] = (shat + e^{x_r}) / (s_n + e^{x_r}), FP64
__global__ void k_interp_nodes(const double* __restrict__ s, int Neff, const float* __restrict__ shat_p, double x0,
                               double h, int R, double* __restrict__ W) {
    const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t >= static_cast<int64_t>(R) * Neff) return;
    const int r = static_cast<int>(t / Neff), n = static_cast<int>(t % Neff);
    const double delta = exp(x0 + r * h);
    W[t] = (static_cast<double>(*shat_p) + delta) / (s[n] + delta);
}

__global__ void k_mean(const double* __restrict__ x, int n, float* __restrict__ out) {
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += 32) acc += x[i];
    acc = warp_sum(acc);
    if (threadIdx.x == 0) *out = static_cast<float>(acc / n);
}

// Wald variant side: B1 = US, B2 = US o US, each row split.  One warp per variant m.
__global__ void k_wald_prep_variants(const float* __restrict__ USt, int64_t ldus, int Mc, int Neff,
                                     __half* __restrict__ B1h, __half* __restrict__ B1l, __half* __restrict__ B2h,
                                     __half* __restrict__ B2l, int64_t ldb, float* __restrict__ sb1,
                                     float* __restrict__ sb2) {
    const int lane = threadIdx.x & 31;
    const int64_t m = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    if (m >= Mc) return;
    const float* u = USt + m * ldus;
    float m1 = 0.0f;
#pragma unroll 4
    for (int n = lane; n < Neff; n += 32) m1 = fmaxf(m1, fabsf(u[n]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, o));
    int e1, e2;
    const float mul1 = row_scale_exp(m1, &e1), mul2 = row_scale_exp(m1 * m1, &e2);
#pragma unroll 4
    for (int n = lane; n < Neff; n += 32) {
        const float x = u[n];
        split_store(x, mul1, B1h, B1l, m * ldb + n);
        split_store(x * x, mul2, B2h, B2l, m * ldb + n);
    }
    if (lane == 0) {
        sb1[m] = ldexpf(1.0f, -e1);
        sb2[m] = ldexpf(1.0f, -e2);
    }
}

// ---- host side: TMA descriptors and launches ---------------------------------------------------------------

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

int encode_fn(PFN_cuTensorMapEncodeTiled_v12000* out) {
    std::call_once(g_encode_once, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    });
    if (!g_encode) return fail(FLMM_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    *out = g_encode;
    return FLMM_OK;
}

// FP16 matrix (rows, K) with row pitch ld elements -> tiled map with box {BK, box_rows} and the matching swizzle.
int make_map(CUtensorMap* map, const void* base, int rows, int K, int64_t ld, int BK, int box_rows = 128) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = nullptr;
    int rc = encode_fn(&enc);
    if (rc) return rc;
    if ((reinterpret_cast<uintptr_t>(base) & 15u) != 0 || (ld * 2) % 16 != 0)
        return fail(FLMM_ERR_ARG, "split operand must be 16-byte aligned with a row pitch that is a multiple of 8");
    cuuint64_t gdim[2] = {static_cast<cuuint64_t>(K), static_cast<cuuint64_t>(rows)};
    cuuint64_t gstride[1] = {static_cast<cuuint64_t>(ld * 2)};
    cuuint32_t box[2] = {static_cast<cuuint32_t>(BK), static_cast<cuuint32_t>(box_rows)};
    cuuint32_t estride[2] = {1u, 1u};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(base), gdim, gstride, box, estride,
                     CU_TENSOR_MAP_INTERLEAVE_NONE,
                     BK == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(FLMM_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", static_cast<int>(r));
    return FLMM_OK;
}

template <int NG, int BK>
int launch_tc(const TcMaps& maps, const TcArgs& args, int sm_count, cudaStream_t st) {
    using C = Cfg<NG, BK>;
    FLMM_CUDA(cudaFuncSetAttribute(k_tc<NG, BK>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::kSmemBytes));
    const int tiles = ((args.Mr + kBM - 1) / kBM) * ((args.Nr + kBN - 1) / kBN);
    if (tiles == 0 || args.K <= 0) return FLMM_OK;
    const int grid = tiles < sm_count ? tiles : sm_count;
    k_tc<NG, BK><<<grid, kThreads, C::kSmemBytes, st>>>(maps, args);
    return check_launch(NG == 1 ? "k_tc<gemm>" : "k_tc<wald>");
}

// Clusters of the pair kernel k_pair<NG> that fit on the device at once (0 if it cannot run as pairs), per device.
template <int NG>
int pair_clusters(int device) {
    static std::mutex mu;
    static int cache[64];
    static bool done[64];
    std::lock_guard<std::mutex> lock(mu);
    if (device < 0 || device >= 64) return 0;
    if (!done[device]) {
        done[device] = true;
        cache[device] = 0;
        if (cudaFuncSetAttribute(k_pair<NG>, cudaFuncAttributeMaxDynamicSharedMemorySize, PairCfg<NG>::kSmemBytes) !=
            cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        int sm = 0;
        cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, device);
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = 2;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(static_cast<unsigned>(sm & ~1), 1, 1);
        cfg.blockDim = dim3(kPairThreads, 1, 1);
        cfg.dynamicSmemBytes = PairCfg<NG>::kSmemBytes;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, k_pair<NG>, &cfg) != cudaSuccess) {
            cudaGetLastError();
            n = 0;
        }
        cache[device] = n;
    }
    return cache[device];
}

template <int NG>
int launch_pair(const TcMaps& maps, const TcArgs& args, int n_clusters_max, cudaStream_t st) {
    const int tiles = ((args.Mr + kPairRows - 1) / kPairRows) * ((args.Nr + kBN - 1) / kBN);
    if (tiles == 0 || args.K <= 0) return FLMM_OK;
    const int n_cl = tiles < n_clusters_max ? tiles : n_clusters_max;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(static_cast<unsigned>(2 * n_cl), 1, 1);
    cfg.blockDim = dim3(kPairThreads, 1, 1);
    cfg.dynamicSmemBytes = PairCfg<NG>::kSmemBytes;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    FLMM_CUDA(cudaLaunchKernelEx(&cfg, k_pair<NG>, maps, args));
    return check_launch(NG == 1 ? "k_pair<gemm>" : "k_pair<wald>");
}

// k-blocks per chunk accumulator: the default, or FLMM_CHUNK_KB (GEMMs) / FLMM_WALD_CHUNK_KB (Wald) from the environment
template <int NG>
int chunk_kb_for() {
    static const int v = [] {
        const char* e = std::getenv(NG == 2 ? "FLMM_WALD_CHUNK_KB" : "FLMM_CHUNK_KB");
        const int x = e ? std::atoi(e) : 0;
        return x >= 1 ? x : default_chunk_kb<NG>();
    }();
    return v;
}

// tcgen05 kernel form: CTA pairs unless FLMM_TC_PAIR=0 asks for the single-CTA kernels (kept for cross-checks)
bool use_pair_kernel() {
    static const bool on = [] {
        const char* e = std::getenv("FLMM_TC_PAIR");
        return !(e && e[0] == '0');
    }();
    return on;
}

// ---- kernel form and tile order: fixed, forced or autotuned ------------------------------------------------------
//
// Every split product (GEMM, NG = 1) and fused Wald launch (NG = 2) picks a kernel form (CTA pair or single CTA) and
// a tile order (raster group, tile_coords).  Mode 0 uses the default (pair when the device can run pairs, A-major
// order); mode 2 forces one choice; mode 1 (the default mode) autotunes: the first launch of each product shape
// (NG, rows, columns, both reduction lengths) times every candidate on the caller's own operands with CUDA events on
// the caller's stream and keeps the fastest for the rest of the process.  Every candidate computes each output with
// the same products in the same K order, so all give bit-identical results and re-running one is harmless (the Wald
// kernel overwrites its detail rows and takes a maximum into max_F).  A GEMM that accumulates into C is not re-run:
// it takes the default.  Tuning synchronises the calling host thread on its events once per shape, and is skipped
// while the stream is being captured into a graph.

struct TcChoice {
    bool pair;
    int group;
};

struct TuneRecord {
    int ng, mr, nr, k, k2;
    TcChoice choice;
    float ms, default_ms;
};

std::mutex g_tune_mu;
int g_tune_mode = -1;  // -1: not read yet (FLMM_AUTOTUNE=0 in the environment starts in mode 0)
TcChoice g_forced = {true, 1};
TuneRecord g_tuned[256];
int g_n_tuned = 0;

constexpr int kGroups[] = {1, 2, 4, 8};

int tune_mode_locked() {
    if (g_tune_mode < 0) {
        const char* e = std::getenv("FLMM_AUTOTUNE");
        g_tune_mode = (e && e[0] == '0') ? 0 : 1;
    }
    return g_tune_mode;
}

template <int NG>
int launch_choice(const TcMaps& maps_tc, const TcMaps& maps_pair, TcArgs a, TcChoice c, int n_cl, int sm_count,
                  cudaStream_t st) {
    a.group = c.group;
    a.chunk_kb = chunk_kb_for<NG>();
    // every launch starts a fresh list of strong real tests (autotuning may run the Wald kernel several times)
    if (NG == 2 && a.flag_count != nullptr) FLMM_CUDA(cudaMemsetAsync(a.flag_count, 0, sizeof(int), st));
    if (c.pair && n_cl > 0) return launch_pair<NG>(maps_pair, a, n_cl, st);
    return launch_tc<NG, kBK>(maps_tc, a, sm_count, st);
}

template <int NG>
int time_choice(const TcMaps& maps_tc, const TcMaps& maps_pair, const TcArgs& a, TcChoice c, int n_cl, int sm_count,
                cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1, float* ms) {
    int rc = launch_choice<NG>(maps_tc, maps_pair, a, c, n_cl, sm_count, st);  // warm
    if (rc) return rc;
    FLMM_CUDA(cudaEventRecord(e0, st));
    for (int r = 0; r < 2 && !rc; ++r) rc = launch_choice<NG>(maps_tc, maps_pair, a, c, n_cl, sm_count, st);
    if (rc) return rc;
    FLMM_CUDA(cudaEventRecord(e1, st));
    FLMM_CUDA(cudaEventSynchronize(e1));
    float t = 0.0f;
    FLMM_CUDA(cudaEventElapsedTime(&t, e0, e1));
    *ms = 0.5f * t;
    return FLMM_OK;
}

// Launch one split product with the configured choice (see above).  maps_pair holds the pair kernel's half-height B
// maps; n_cl = 0 when the device cannot run the pair kernel.
template <int NG>
int launch_product(const TcMaps& maps_tc, const TcMaps& maps_pair, const TcArgs& a, int n_cl, int sm_count,
                   bool rerunnable, cudaStream_t st) {
    if (!use_pair_kernel()) n_cl = 0;  // FLMM_TC_PAIR=0: single-CTA kernels only
    const TcChoice def = {n_cl > 0, 1};
    TcChoice choice = def;
    std::unique_lock<std::mutex> lock(g_tune_mu);
    const int mode = tune_mode_locked();
    if (mode == 2) {
        choice = g_forced;
    } else if (mode == 1 && rerunnable) {
        bool found = false;
        for (int i = 0; i < g_n_tuned; ++i) {
            const TuneRecord& t = g_tuned[i];
            if (t.ng == NG && t.mr == a.Mr && t.nr == a.Nr && t.k == a.K && t.k2 == a.K2) {
                choice = t.choice;
                found = true;
                break;
            }
        }
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        FLMM_CUDA(cudaStreamIsCapturing(st, &cap));
        if (!found && cap == cudaStreamCaptureStatusNone && g_n_tuned < 256) {
            // time the candidates without the lock, so other host threads keep launching products meanwhile
            lock.unlock();
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            FLMM_CUDA(cudaEventCreate(&e0));
            if (cudaEventCreate(&e1) != cudaSuccess) {
                cudaEventDestroy(e0);
                return fail(FLMM_ERR_CUDA, "autotune: cannot create events");
            }
            float best = 0.0f, def_ms = 0.0f;
            bool have = false;
            int rc = FLMM_OK;
            for (int pi = 0; pi < 2 && !rc; ++pi) {
                const bool pair = pi == 0;
                if (pair && !(n_cl > 0)) continue;
                for (int g : kGroups) {
                    const TcChoice c = {pair, g};
                    float ms = 0.0f;
                    if ((rc = time_choice<NG>(maps_tc, maps_pair, a, c, n_cl, sm_count, st, e0, e1, &ms))) break;
                    if (c.pair == def.pair && c.group == def.group) def_ms = ms;
                    if (!have || ms < best) {
                        best = ms;
                        choice = c;
                        have = true;
                    }
                }
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            if (rc) return rc;
            lock.lock();
            // another thread may have tuned the same shape meanwhile: the first record stands (every candidate
            // gives the same bits, so either choice is correct; one choice per shape keeps the report consistent)
            bool again = false;
            for (int i = 0; i < g_n_tuned; ++i) {
                const TuneRecord& t = g_tuned[i];
                if (t.ng == NG && t.mr == a.Mr && t.nr == a.Nr && t.k == a.K && t.k2 == a.K2) {
                    choice = t.choice;
                    again = true;
                    break;
                }
            }
            if (!again && g_n_tuned < 256) g_tuned[g_n_tuned++] = {NG, a.Mr, a.Nr, a.K, a.K2, choice, best, def_ms};
        }
    }
    if (lock.owns_lock()) lock.unlock();
    return launch_choice<NG>(maps_tc, maps_pair, a, choice, n_cl, sm_count, st);
}

}  // namespace

// FP16 operand maps for the other tcgen05 kernels of the library (flmm_ozaki.cu).
int flmm::tc::make_map_f16(CUtensorMap* map, const void* base, int rows, int K, int64_t ld, int BK, int box_rows) {
    return make_map(map, base, rows, K, ld, BK, box_rows);
}

extern "C" int flmm_tc_config(int mode, int pair, int group) {
    FLMM_REQUIRE(mode >= 0 && mode <= 2 && (mode != 2 || group >= 1),
                 "flmm_tc_config: mode 0 (default), 1 (autotune) or 2 (forced pair / group >= 1)");
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_mode = mode;
    g_forced = {pair != 0, group};
    return FLMM_OK;
}

extern "C" int flmm_autotune_report(char* buf, size_t len, int* n_records) {
    FLMM_REQUIRE(buf && len > 0 && n_records, "flmm_autotune_report: bad arguments");
    std::lock_guard<std::mutex> lock(g_tune_mu);
    size_t off = 0;
    buf[0] = 0;
    for (int i = 0; i < g_n_tuned && off < len; ++i) {
        const TuneRecord& t = g_tuned[i];
        const int w = std::snprintf(buf + off, len - off, "%d %d %d %d %d %d %d %.6f %.6f\n", t.ng, t.mr, t.nr, t.k,
                                    t.k2, t.choice.pair ? 1 : 0, t.choice.group, t.ms, t.default_ms);
        if (w < 0) break;
        off += static_cast<size_t>(w);
    }
    *n_records = g_n_tuned;
    return FLMM_OK;
}

// ---- C ABI -----------------------------------------------------------------------------------------------------

int flmm_ctx_sm_count(flmm_context* ctx);
int* flmm_ctx_err_flag(flmm_context* ctx);

extern "C" int flmm_split_rows_f16(const void* X, int x_is_f64, int64_t ldx, int rows, int K, void* hi, void* lo,
                                   int64_t ldo, float* scale, void* stream) {
    FLMM_REQUIRE(X && hi && lo && scale && rows >= 0 && K > 0 && ldx >= K && ldo >= K,
                 "flmm_split_rows_f16: bad arguments");
    if (rows == 0) return FLMM_OK;
    cudaStream_t st = as_stream(stream);
    __half* h = static_cast<__half*>(hi);
    __half* l = static_cast<__half*>(lo);
    if (K > 4096) {  // long rows: a block per row
        if (x_is_f64)
            k_split_long_rows<double><<<rows, 256, 0, st>>>(static_cast<const double*>(X), ldx, rows, K, h, l, ldo, scale);
        else
            k_split_long_rows<float><<<rows, 256, 0, st>>>(static_cast<const float*>(X), ldx, rows, K, h, l, ldo, scale);
        return check_launch("k_split_long_rows");
    }
    const unsigned grid = ceil_div(static_cast<int64_t>(rows) * 32, 256);  // one warp per row
    if (x_is_f64)
        k_split_rows<double><<<grid, 256, 0, st>>>(static_cast<const double*>(X), ldx, rows, K, h, l, ldo, scale);
    else
        k_split_rows<float><<<grid, 256, 0, st>>>(static_cast<const float*>(X), ldx, rows, K, h, l, ldo, scale);
    return check_launch("k_split_rows");
}

extern "C" int flmm_gemm_split_f16(flmm_context* ctx, const void* Ah, const void* Al, const float* sa, int64_t lda,
                                   int Mr, const void* Bh, const void* Bl, const float* sb, int64_t ldb, int Nr, int K,
                                   float* Cout, int64_t ldc, int accumulate, void* stream) {
    FLMM_REQUIRE(ctx && Ah && Al && sa && Bh && Bl && sb && Cout && Mr >= 0 && Nr >= 0 && K > 0 && lda >= K &&
                     ldb >= K && ldc >= Nr,
                 "flmm_gemm_split_f16: bad arguments");
    if (Mr == 0 || Nr == 0) return FLMM_OK;
    TcMaps maps;
    std::memset(&maps, 0, sizeof(maps));
    int rc;
    if ((rc = make_map(&maps.m[0], Ah, Mr, K, lda, kBK))) return rc;
    if ((rc = make_map(&maps.m[1], Al, Mr, K, lda, kBK))) return rc;
    if ((rc = make_map(&maps.m[2], Bh, Nr, K, ldb, kBK))) return rc;
    if ((rc = make_map(&maps.m[3], Bl, Nr, K, ldb, kBK))) return rc;
    TcArgs a;
    std::memset(&a, 0, sizeof(a));
    a.Mr = Mr;
    a.Nr = Nr;
    a.K = K;
    a.err = flmm_ctx_err_flag(ctx);
    a.sa = sa;
    a.sb = sb;
    a.C = Cout;
    a.ldc = ldc;
    a.accumulate = accumulate;
    int dev = 0;
    FLMM_CUDA(cudaGetDevice(&dev));
    const int n_cl = pair_clusters<1>(dev);
    TcMaps maps_pair = maps;  // the pair kernel loads 64 B rows per CTA: half-height B boxes
    if (n_cl > 0) {
        if ((rc = make_map(&maps_pair.m[2], Bh, Nr, K, ldb, kBK, kBN / 2))) return rc;
        if ((rc = make_map(&maps_pair.m[3], Bl, Nr, K, ldb, kBK, kBN / 2))) return rc;
    }
    return launch_product<1>(maps, maps_pair, a, n_cl, flmm_ctx_sm_count(ctx), accumulate == 0, as_stream(stream));
}

extern "C" int flmm_mean_f32(const double* x, int n, float* out, void* stream) {
    FLMM_REQUIRE(x && out && n > 0, "flmm_mean_f32: bad arguments");
    k_mean<<<1, 32, 0, as_stream(stream)>>>(x, n, out);
    return check_launch("k_mean");
}

extern "C" int flmm_wald_interp_nodes(const double* s, int Neff, const float* shat, double x0, double h, int R,
                                      double* W, void* stream) {
    FLMM_REQUIRE(s && shat && W && Neff > 0 && R >= kInterpPoints && h > 0, "flmm_wald_interp_nodes: bad arguments");
    k_interp_nodes<<<ceil_div(static_cast<int64_t>(R) * Neff, 256), 256, 0, as_stream(stream)>>>(s, Neff, shat, x0, h,
                                                                                               R, W);
    return check_launch("k_interp_nodes");
}

extern "C" int flmm_wald_split_prep_columns(const float* s32, int Neff, const float* UYt, int64_t ldu,
                                            const double* log_delta, int P, const float* shat, double x0, double h,
                                            int R, void* A1h, void* A1l, int64_t lda, void* Lh, void* Ll, int64_t ldl,
                                            float* sa1, float* sl, float* rWr, float* rWr0, void* stream) {
    FLMM_REQUIRE(s32 && UYt && log_delta && shat && A1h && A1l && Lh && Ll && sa1 && sl && rWr && rWr0 && Neff > 0 &&
                     ldu >= Neff && lda >= Neff && ldl >= R && R >= kInterpPoints && h > 0 && P >= 0,
                 "flmm_wald_split_prep_columns: bad arguments");
    if (P == 0) return FLMM_OK;
    k_wald_prep_columns<<<ceil_div(P, kPrepCols), 32 * kPrepCols, 0, as_stream(stream)>>>(
        s32, Neff, UYt, ldu, log_delta, P, shat, x0, h, 1.0 / h, R, static_cast<__half*>(A1h), static_cast<__half*>(A1l), lda,
        static_cast<__half*>(Lh), static_cast<__half*>(Ll), ldl, sa1, sl, rWr, rWr0);
    return check_launch("k_wald_prep_columns");
}

extern "C" int flmm_wald_split_prep_variants(const float* USt, int64_t ldus, int Mc, int Neff, void* B1h, void* B1l,
                                             void* B2h, void* B2l, int64_t ldb, float* sb1, float* sb2,
                                             void* stream) {
    FLMM_REQUIRE(USt && B1h && B1l && B2h && B2l && sb1 && sb2 && Neff > 0 && ldus >= Neff && ldb >= Neff && Mc >= 0,
                 "flmm_wald_split_prep_variants: bad arguments");
    if (Mc == 0) return FLMM_OK;
    k_wald_prep_variants<<<ceil_div(static_cast<int64_t>(Mc) * 32, 256), 256, 0, as_stream(stream)>>>(
        USt, ldus, Mc, Neff, static_cast<__half*>(B1h), static_cast<__half*>(B1l), static_cast<__half*>(B2h),
        static_cast<__half*>(B2l), ldb, sb1, sb2);
    return check_launch("k_wald_prep_variants");
}

extern "C" int flmm_wald_split_f16(flmm_context* ctx, const void* A1h, const void* A1l, int64_t lda, const float* sa1,
                                   const void* Lh, const void* Ll, int64_t ldl, const float* sl, const float* rWr,
                                   const float* rWr0, int P, int n_real, const void* B1h, const void* B1l, int64_t ldb, const float* sb1,
                                   const void* Fh, const void* Fl, int64_t ldf, const float* sf, int Mc, int Neff,
                                   int R, const int64_t* rows, double* f, double* beta, double* se, double* sfve,
                                   int64_t ldo, double* max_F, float f_refine, int32_t* flag_count,
                                   int32_t* flags, int flag_cap, void* stream) {
    return flmm_wald_split_f16_df(ctx, A1h, A1l, lda, sa1, Lh, Ll, ldl, sl, rWr, rWr0, P, n_real, B1h, B1l, ldb, sb1,
                                  Fh, Fl, ldf, sf, Mc, Neff, R, rows, f, beta, se, sfve, ldo, max_F, f_refine,
                                  flag_count, flags, flag_cap, Neff - 1, stream);
}

extern "C" int flmm_wald_split_f16_df(flmm_context* ctx, const void* A1h, const void* A1l, int64_t lda,
                                      const float* sa1, const void* Lh, const void* Ll, int64_t ldl, const float* sl,
                                      const float* rWr, const float* rWr0, int P, int n_real, const void* B1h,
                                      const void* B1l, int64_t ldb, const float* sb1, const void* Fh, const void* Fl,
                                      int64_t ldf, const float* sf, int Mc, int Neff, int R, const int64_t* rows,
                                      double* f, double* beta, double* se, double* sfve, int64_t ldo, double* max_F,
                                      float f_refine, int32_t* flag_count, int32_t* flags, int flag_cap, int var_df,
                                      void* stream) {
    FLMM_REQUIRE(var_df > 0, "flmm_wald_split_f16_df: var_df must be positive");
    FLMM_REQUIRE(ctx && A1h && A1l && sa1 && Lh && Ll && sl && rWr && rWr0 && B1h && B1l && sb1 && Fh && Fl && sf && max_F &&
                     Neff > 1 && R > 0 && P >= 0 && Mc >= 0 && n_real >= 0 && n_real <= P && lda >= Neff &&
                     ldb >= Neff && ldl >= R && ldf >= R,
                 "flmm_wald_split_f16: bad arguments");
    FLMM_REQUIRE(n_real == 0 || Mc == 0 || (rows && f && beta && se && sfve && ldo >= n_real),
                 "flmm_wald_split_f16: real-column outputs missing");
    FLMM_REQUIRE(flag_count == nullptr || (flag_cap >= 0 && (flags != nullptr || flag_cap == 0)),
                 "flmm_wald_split_f16: strong-test list without storage");
    if (flag_count != nullptr) FLMM_CUDA(cudaMemsetAsync(flag_count, 0, sizeof(int32_t), as_stream(stream)));
    if (P == 0 || Mc == 0) return FLMM_OK;
    TcMaps maps;
    std::memset(&maps, 0, sizeof(maps));
    int rc;
    // product 0: sWy = (w~ o UY) US^T over K = Neff; product 1: sWs~ = L F^T over K = R
    if ((rc = make_map(&maps.m[0], A1h, P, Neff, lda, kBK))) return rc;
    if ((rc = make_map(&maps.m[1], A1l, P, Neff, lda, kBK))) return rc;
    if ((rc = make_map(&maps.m[2], B1h, Mc, Neff, ldb, kBK))) return rc;
    if ((rc = make_map(&maps.m[3], B1l, Mc, Neff, ldb, kBK))) return rc;
    if ((rc = make_map(&maps.m[4], Lh, P, R, ldl, kBK))) return rc;
    if ((rc = make_map(&maps.m[5], Ll, P, R, ldl, kBK))) return rc;
    if ((rc = make_map(&maps.m[6], Fh, Mc, R, ldf, kBK))) return rc;
    if ((rc = make_map(&maps.m[7], Fl, Mc, R, ldf, kBK))) return rc;
    TcArgs a;
    std::memset(&a, 0, sizeof(a));
    a.Mr = P;
    a.Nr = Mc;
    a.K = Neff;
    a.K2 = R;
    a.err = flmm_ctx_err_flag(ctx);
    a.sa = sa1;
    a.sb = sb1;
    a.sa2 = sl;
    a.sb2 = sf;
    a.rWr = rWr;
    a.rWr0 = rWr0;
    a.n_real = n_real;
    a.var_df = static_cast<float>(var_df);
    a.rows = rows;
    a.f = f;
    a.beta = beta;
    a.se = se;
    a.sfve = sfve;
    a.ldo = ldo;
    a.max_F = max_F;
    a.f_refine = f_refine;
    a.flag_count = flag_count;
    a.flags = reinterpret_cast<int2*>(flags);
    a.flag_cap = flag_cap;
    int dev = 0;
    FLMM_CUDA(cudaGetDevice(&dev));
    const int n_cl = pair_clusters<2>(dev);
    TcMaps maps_pair = maps;  // the pair kernel loads 64 B rows per CTA: variant-side maps with half-height boxes
    if (n_cl > 0) {
        if ((rc = make_map(&maps_pair.m[2], B1h, Mc, Neff, ldb, kBK, kBN / 2))) return rc;
        if ((rc = make_map(&maps_pair.m[3], B1l, Mc, Neff, ldb, kBK, kBN / 2))) return rc;
        if ((rc = make_map(&maps_pair.m[6], Fh, Mc, R, ldf, kBK, kBN / 2))) return rc;
        if ((rc = make_map(&maps_pair.m[7], Fl, Mc, R, ldf, kBK, kBN / 2))) return rc;
    }
    return launch_product<2>(maps, maps_pair, a, n_cl, flmm_ctx_sm_count(ctx), true, as_stream(stream));
}
