// Permutation row orders on the device, bit-identical to the reference's host draw (fasterlmm/perms.py:51-55):
//     orders[b, j, :] = argsort(numpy.random.default_rng([seed, col_b]).random((n_perm, N))[j])
//
// The generator is numpy's default: SeedSequence entropy mixing of the uint32 words of [seed, col] (pool of four
// words, hashmix / mix with the published constants), generate_state(4, uint64) seeding PCG64 (128-bit LCG with
// multiplier 0x2360ED051FC65DA4_4385DF649FCCF645, XSL-RR output, one step before each output), and
// random() = (next64 >> 11) * 2^-53.  Row j of column b is positions [j N, (j + 1) N) of that column's stream; each
// thread jumps straight to its positions with the O(log n) LCG advance (Brown 1994), generates one key per stride
// and the block sorts (key, position) pairs with a bitonic network in shared memory.  Keys are the 53-bit integers
// (next64 >> 11), which order exactly like the doubles; equal keys (probability ~N^2 2^-54 per row) are ordered by
// position.
#include <stdint.h>

#include "flmm_common.cuh"

using namespace flmm;

namespace {

typedef unsigned __int128 u128;

constexpr uint32_t kInitA = 0x43b0d7e5u, kMultA = 0x931e8875u, kInitB = 0x8b51f9ddu, kMultB = 0x58f38dedu;
constexpr uint32_t kMixL = 0xca01f9ddu, kMixR = 0x4973f715u;

__device__ __forceinline__ u128 pcg_mult() {
    return (static_cast<u128>(0x2360ED051FC65DA4ull) << 64) | static_cast<u128>(0x4385DF649FCCF645ull);
}

struct Pcg {
    u128 state, inc;
};

// SeedSequence([seed, col]).generate_state(4, uint64) -> PCG64 state (numpy's seeding path)
__device__ Pcg seed_pcg(uint64_t seed, uint64_t col) {
    uint32_t words[4];
    int nw = 0;
    words[nw++] = static_cast<uint32_t>(seed);
    if (seed >> 32) words[nw++] = static_cast<uint32_t>(seed >> 32);
    words[nw++] = static_cast<uint32_t>(col);
    if (col >> 32) words[nw++] = static_cast<uint32_t>(col >> 32);
    uint32_t h = kInitA;
    auto hashmix = [&](uint32_t v) {
        v ^= h;
        h *= kMultA;
        v *= h;
        return v ^ (v >> 16);
    };
    auto mix = [](uint32_t x, uint32_t y) {
        uint32_t r = kMixL * x - kMixR * y;
        return r ^ (r >> 16);
    };
    uint32_t pool[4];
    for (int i = 0; i < 4; ++i) pool[i] = hashmix(i < nw ? words[i] : 0u);
    for (int s = 0; s < 4; ++s)
        for (int d = 0; d < 4; ++d)
            if (s != d) pool[d] = mix(pool[d], hashmix(pool[s]));
    for (int s = 4; s < nw; ++s)
        for (int d = 0; d < 4; ++d) pool[d] = mix(pool[d], hashmix(words[s]));
    uint32_t hb = kInitB;
    uint32_t st[8];
    for (int i = 0; i < 8; ++i) {
        uint32_t v = pool[i & 3];
        v ^= hb;
        hb *= kMultB;
        v *= hb;
        st[i] = v ^ (v >> 16);
    }
    uint64_t v64[4];
    for (int i = 0; i < 4; ++i) v64[i] = static_cast<uint64_t>(st[2 * i]) | (static_cast<uint64_t>(st[2 * i + 1]) << 32);
    const u128 initstate = (static_cast<u128>(v64[0]) << 64) | v64[1];
    const u128 initseq = (static_cast<u128>(v64[2]) << 64) | v64[3];
    Pcg g;
    g.inc = (initseq << 1) | 1u;
    g.state = 0;
    g.state = g.state * pcg_mult() + g.inc;
    g.state += initstate;
    g.state = g.state * pcg_mult() + g.inc;
    return g;
}

// affine map of `delta` LCG steps: state -> mult * state + plus
__device__ void lcg_jump(u128 inc, uint64_t delta, u128* mult, u128* plus) {
    u128 acc_m = 1, acc_p = 0, cur_m = pcg_mult(), cur_p = inc;
    while (delta) {
        if (delta & 1u) {
            acc_m *= cur_m;
            acc_p = acc_p * cur_m + cur_p;
        }
        cur_p = (cur_m + 1) * cur_p;
        cur_m *= cur_m;
        delta >>= 1;
    }
    *mult = acc_m;
    *plus = acc_p;
}

__device__ __forceinline__ uint64_t xsl_rr(u128 s) {
    const uint64_t x = static_cast<uint64_t>(s >> 64) ^ static_cast<uint64_t>(s);
    const unsigned r = static_cast<unsigned>(s >> 122);
    return (x >> r) | (x << ((64u - r) & 63u));
}

constexpr int kThreads = 256;

// one block per (column b, permutation j); shared memory: npow2 keys (uint64) + npow2 positions (int32)
__global__ void __launch_bounds__(kThreads)
k_perm_orders(const int64_t* __restrict__ cols, uint64_t seed, int n_perm, int N, int npow2,
              int32_t* __restrict__ orders) {
    extern __shared__ uint64_t sm[];
    uint64_t* key = sm;
    int32_t* pos = reinterpret_cast<int32_t*>(sm + npow2);
    const int b = blockIdx.x / n_perm, j = blockIdx.x % n_perm;
    const Pcg g = seed_pcg(seed, static_cast<uint64_t>(cols[b]));
    // thread t draws stream positions j N + t + k * blockDim; one output per LCG step, taken after the step
    u128 m0, p0, ms, ps;
    lcg_jump(g.inc, static_cast<uint64_t>(j) * N + threadIdx.x, &m0, &p0);
    lcg_jump(g.inc, blockDim.x, &ms, &ps);
    u128 s = m0 * g.state + p0;  // state before the first step of this thread
    for (int i = threadIdx.x; i < npow2; i += blockDim.x) {
        if (i < N) {
            const u128 s1 = s * pcg_mult() + g.inc;
            key[i] = xsl_rr(s1) >> 11;
            s = ms * s + ps;
        } else {
            key[i] = ~0ull;  // padding sorts last
        }
        pos[i] = i;
    }
    __syncthreads();
    // bitonic sort of (key, pos) ascending
    for (int size = 2; size <= npow2; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = threadIdx.x; i < npow2 / 2; i += blockDim.x) {
                const int lo = 2 * i - (i & (stride - 1));
                const int hi = lo + stride;
                const bool up = (lo & size) == 0;
                const uint64_t ka = key[lo], kb = key[hi];
                const int32_t pa = pos[lo], pb = pos[hi];
                const bool gt = (ka > kb) || (ka == kb && pa > pb);
                if (gt == up) {
                    key[lo] = kb;
                    key[hi] = ka;
                    pos[lo] = pb;
                    pos[hi] = pa;
                }
            }
            __syncthreads();
        }
    }
    int32_t* out = orders + (static_cast<int64_t>(b) * n_perm + j) * N;
    for (int i = threadIdx.x; i < N; i += blockDim.x) out[i] = pos[i];
}

// Same orders for N <= 2048: the 53-bit key and the 11-bit position packed into one word (key << 11 | position),
// so the bitonic sort moves and compares single 64-bit values; ascending packed order is the (key, position) order.
constexpr int kPackBits = 11;

__global__ void __launch_bounds__(kThreads)
k_perm_orders_packed(const int64_t* __restrict__ cols, uint64_t seed, int n_perm, int N, int npow2,
                     int32_t* __restrict__ orders) {
    extern __shared__ uint64_t kp[];
    const int b = blockIdx.x / n_perm, j = blockIdx.x % n_perm;
    const Pcg g = seed_pcg(seed, static_cast<uint64_t>(cols[b]));
    u128 m0, p0, ms, ps;
    lcg_jump(g.inc, static_cast<uint64_t>(j) * N + threadIdx.x, &m0, &p0);
    lcg_jump(g.inc, blockDim.x, &ms, &ps);
    u128 s = m0 * g.state + p0;
    for (int i = threadIdx.x; i < npow2; i += blockDim.x) {
        if (i < N) {
            const u128 s1 = s * pcg_mult() + g.inc;
            kp[i] = ((xsl_rr(s1) >> 11) << kPackBits) | static_cast<uint64_t>(i);
            s = ms * s + ps;
        } else {
            kp[i] = ~0ull;  // padding sorts last
        }
    }
    __syncthreads();
    for (int size = 2; size <= npow2; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = threadIdx.x; i < npow2 / 2; i += blockDim.x) {
                const int lo = 2 * i - (i & (stride - 1));
                const int hi = lo + stride;
                const bool up = (lo & size) == 0;
                const uint64_t a = kp[lo], c = kp[hi];
                if ((a > c) == up) {
                    kp[lo] = c;
                    kp[hi] = a;
                }
            }
            __syncthreads();
        }
    }
    int32_t* out = orders + (static_cast<int64_t>(b) * n_perm + j) * N;
    for (int i = threadIdx.x; i < N; i += blockDim.x) out[i] = static_cast<int32_t>(kp[i] & ((1u << kPackBits) - 1));
}

}  // namespace

extern "C" int flmm_perm_orders(const int64_t* seed_cols, int B, uint64_t seed, int n_perm, int N, int32_t* orders,
                                void* stream) {
    FLMM_REQUIRE(B >= 0 && n_perm >= 0 && N > 0, "flmm_perm_orders: bad sizes");
    if (B == 0 || n_perm == 0) return FLMM_OK;
    FLMM_REQUIRE(seed_cols && orders, "flmm_perm_orders: NULL argument");
    FLMM_REQUIRE(N <= 16384, "flmm_perm_orders: N must be <= 16384 (shared-memory sort), got %d", N);
    FLMM_REQUIRE(static_cast<int64_t>(B) * n_perm <= 0x7fffffff, "flmm_perm_orders: too many rows");
    int npow2 = 1;
    while (npow2 < N) npow2 <<= 1;
    if (npow2 <= (1 << kPackBits)) {
        const size_t smem_p = static_cast<size_t>(npow2) * sizeof(uint64_t);
        k_perm_orders_packed<<<B * n_perm, kThreads, smem_p, as_stream(stream)>>>(seed_cols, seed, n_perm, N, npow2,
                                                                                orders);
        return check_launch("k_perm_orders_packed");
    }
    const size_t smem = static_cast<size_t>(npow2) * (sizeof(uint64_t) + sizeof(int32_t));
    if (smem > 48 * 1024)
        FLMM_CUDA(cudaFuncSetAttribute(k_perm_orders, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    k_perm_orders<<<B * n_perm, kThreads, smem, as_stream(stream)>>>(seed_cols, seed, n_perm, N, npow2, orders);
    return check_launch("k_perm_orders");
}
