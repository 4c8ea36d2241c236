// Batched FP32 symmetric eigendecomposition of the projected LOCO kinships (N below 2,500), the fast form's
// replacement for the library's batched eigensolver.  The reference decomposes each kinship in FP64
// (fasterlmm/core.py:54-77, torch.linalg.eigh); the fast form takes an FP32 decomposition and refines it
// (flmm_eigh_refine_f32), so only FP32-quality eigenpairs are needed here.
//
// Five stages, all matrices of the batch side by side:
//
// 1. k_sytrd_cluster: Householder tridiagonalisation A = Q T Q^T, one thread-block cluster of 2 to 8 CTAs per
//    matrix (one CTA per SM).  The FP32 matrix stays in global memory (L2-resident for the batch sizes used), rows
//    dealt round-robin to the cluster's CTAs.  Column k's reflector is formed redundantly by every CTA, each CTA
//    computes p = tau W v for its rows and stores it, with its partial p^T v, into every CTA's shared memory
//    (distributed shared memory), so after the barrier each CTA reads only its own.  The symmetric rank-2 update
//    W -= v w^T + w v^T is applied lazily, in the same pass that forms the next column's W v, so the trailing
//    matrix is read and written once per column; the next pivot row gets its last update in registers in every
//    CTA, which forms the next reflector from it.  Both products of an update term are rounded before the add, so
//    W stays exactly symmetric.  One cluster barrier per column.
// 2. k_tridiag_bisect: each eigenvalue of T by multisection on FP32 Sturm counts (ascending, by index; three points
//    per step, so 24 steps narrow the bracket as 48 halvings would).
// 3. k_tridiag_invit: each eigenvector of T by inverse iteration in FP64 (LDL^T of T - lambda I with a pivot floor,
//    three solves from a fixed pseudo-random start, the first fused with the factorisation), one thread each.
// 4. k_cluster_orth: eigenvalues closer than kClusterTol * ||T|| form a cluster; one warp orthonormalises its
//    vectors (modified Gram-Schmidt in FP64).  Each vector of a cluster has converged into the cluster's invariant
//    subspace from its own start, so the result is an orthonormal basis of that subspace.
// 5. k_wy_factors + k_backtransform: the reflectors in blocks of kWy as I - V T V^T (forward, columnwise), applied to
//    column tiles of the eigenvector matrix of T held in shared memory, last block first; the result is written as
//    one eigenvector per row.
//
// Every loop is bounded by N and fixed iteration counts; the only waits are cluster barriers that every CTA of the
// cluster reaches on the same trip count.
#include <math.h>

#include <algorithm>
#include <stdint.h>

#include "flmm_common.cuh"

using namespace flmm;

namespace {

constexpr int kMaxClusterCtas = 8;
constexpr int kSytrdThreads = 512;
constexpr int kRowsPerWarp = 4;    // rows a warp of the tridiagonalisation works on at once
constexpr int kLoadsPerRow = 8;    // loads of each of them a lane has in flight
constexpr int kWy = 16;            // reflectors per WY block
constexpr int kTile = 16;          // eigenvectors per back-transform CTA
constexpr int kBtThreads = 256;
constexpr int kChunk = 128;        // rows of a V block staged at a time in the back-transform
// the FP32 shift is within ~1e-7 ||T|| of its eigenvalue: at the cluster cut (a gap of 1e-5 ||T||) each solve shrinks
// the neighbour by ~1e-2, so three solves leave ~1e-6 of it (two left pairs near the cut ~1e-4 from orthogonal)
constexpr int kInvitSolves = 3;
constexpr int kInvitBlock = 16;     // elements whose loads a recurrence pass issues ahead
constexpr double kClusterTol = 1e-5;
constexpr int kSectPts = 3;        // points per multisection step of the eigenvalue brackets (its quarters)
constexpr int kBisectSteps = 24;   // 4^-24 = 2^-48 of the Gershgorin interval
constexpr int kBisectThreads = 128;

__device__ __forceinline__ uint32_t cta_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

__device__ __forceinline__ uint32_t cluster_index() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
    return r;
}

__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// FP32 store into the shared memory of the cluster's CTA `rank` at the address of `p` in this CTA (made visible to it
// by the next cluster barrier)
__device__ __forceinline__ void st_remote(float* p, uint32_t rank, float v) {
    uint32_t a;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(a) : "r"(smem_addr(p)), "r"(rank));
    asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
}

// block-wide FP32 sum (all threads get it); red holds >= 32 floats
__device__ float block_sum(float v, float* red) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    float t = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0f;
    if (wid == 0) t = warp_sum(t);
    if (threadIdx.x == 0) red[0] = t;
    __syncthreads();
    return red[0];
}

// W (batch, N, N) FP32 symmetric, full storage, overwritten: row k holds the reflector v_k on columns k+1..N-1
// (v_k[k+1] = 1).  d (batch, N), e (batch, N), tau (batch, N): T's diagonal, off-diagonal (e[k] = T[k][k+1]) and the
// reflector scalars (tau[N-2] = tau[N-1] = 0).  The cluster size C is the launch's (%cluster_nctarank); CTA r owns
// the rows i with i % C == r.
//
// Step k: (B) each CTA brings its rows i > k up to date with column k-1's update and forms p_i = tau_k W[i, k+1:] v_k;
// one cluster barrier; (C) every CTA gathers p and p^T v from the cluster, forms w_k, reads row k+1 (stored by its
// owner in (B), so it already carries every update but column k's), applies column k's update to it in registers and
// forms the next reflector v_{k+1} -- redundantly in every CTA, so no second barrier is needed.
__device__ __forceinline__ uint32_t cluster_size() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}

struct Reflector {
    float d, beta, tau;
};

// From x = row entries x[k .. N-1] in xs[] (xs[j] for j >= k + 1; d passed in): the reflector of column k into v[]
// (v[k+1] = 1, v[j] = x_j / (alpha - beta) for j >= k + 2), as LAPACK's larfg.  Every thread of the CTA calls it.
__device__ Reflector make_reflector(float d, float alpha, float ss_partial, float* v, int k, int N, float* red) {
    const float sigma = block_sum(ss_partial, red);
    Reflector R{d, alpha, 0.0f};
    float scal = 0.0f;
    if (sigma > 0.0f) {
        R.beta = -copysignf(sqrtf(fmaf(alpha, alpha, sigma)), alpha);
        R.tau = (R.beta - alpha) / R.beta;
        scal = 1.0f / (alpha - R.beta);
    }
    for (int j = k + 2 + threadIdx.x; j < N; j += blockDim.x) v[j] *= scal;
    if (threadIdx.x == 0) v[k + 1] = 1.0f;
    __syncthreads();
    return R;
}

__global__ void __launch_bounds__(kSytrdThreads, 1)
k_sytrd_cluster(float* __restrict__ W, int N, float* __restrict__ d_out, float* __restrict__ e_out,
                float* __restrict__ tau_out) {
    extern __shared__ float sm[];
    const int Np = (N + 3) & ~3;
    float* vbuf[2] = {sm, sm + Np};
    float* wbuf[2] = {sm + 2 * Np, sm + 3 * Np};
    float* pbuf[2] = {sm + 4 * Np, sm + 5 * Np};
    float* red = sm + 6 * Np;        // 32 floats
    float* part = red + 32;          // partial p^T v of every CTA of the cluster, [parity][rank]
    float* scal2 = part + 2 * kMaxClusterCtas;  // d and alpha of the next reflector
    const int C = static_cast<int>(cluster_size());
    const int b = static_cast<int>(cluster_index());
    const int r = static_cast<int>(cta_rank());
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = kSytrdThreads >> 5;
    float* Wb = W + static_cast<int64_t>(b) * N * N;
    float* db = d_out + static_cast<int64_t>(b) * N;
    float* eb = e_out + static_cast<int64_t>(b) * N;
    float* tb = tau_out + static_cast<int64_t>(b) * N;
    Reflector R{0.0f, 0.0f, 0.0f};
    if (N >= 3) {  // reflector of column 0 from the untouched row 0
        float ss = 0.0f;
        for (int j = 2 + threadIdx.x; j < N; j += kSytrdThreads) {
            const float x = Wb[j];
            vbuf[0][j] = x;
            ss = fmaf(x, x, ss);
        }
        R = make_reflector(Wb[0], Wb[1], ss, vbuf[0], 0, N, red);
    }
    for (int k = 0; k + 2 < N; ++k) {
        const int cur = k & 1;
        float* vc = vbuf[cur];
        float* wc = wbuf[cur];
        float* vn = vbuf[cur ^ 1];        // v_{k-1} until (B) is done, then v_{k+1}
        const float* wp = wbuf[cur ^ 1];  // w_{k-1}
        float* pb = pbuf[cur];
        const float tau = R.tau;
        // (B) rows i > k of this CTA: column k-1's update (lazy), then p_i = tau W[i, k+1:] . v.  A warp takes
        // kRowsPerWarp rows at a time and a lane issues kLoadsPerRow loads of each before using any, so the pass
        // keeps enough L2 reads in flight to run at bandwidth rather than at L2 latency.
        float dot = 0.0f;
        const int first = k + 1 + ((r - (k + 1)) % C + C) % C;
        const int n_own = first < N ? (N - 1 - first) / C + 1 : 0;
        const bool lazy = k > 0;
        for (int t0 = wid * kRowsPerWarp; t0 < n_own; t0 += nw * kRowsPerWarp) {
            float* rows[kRowsPerWarp];
            float vi[kRowsPerWarp], wi[kRowsPerWarp], acc[kRowsPerWarp];
#pragma unroll
            for (int q = 0; q < kRowsPerWarp; ++q) {
                const int t = t0 + q;
                const int i = first + t * C;
                rows[q] = t < n_own ? Wb + static_cast<int64_t>(i) * N : nullptr;
                vi[q] = (t < n_own && lazy) ? vn[i] : 0.0f;
                wi[q] = (t < n_own && lazy) ? wp[i] : 0.0f;
                acc[q] = 0.0f;
            }
            for (int j0 = k + 1; j0 < N; j0 += 32 * kLoadsPerRow) {
                float x[kRowsPerWarp][kLoadsPerRow];
#pragma unroll
                for (int q = 0; q < kRowsPerWarp; ++q)
#pragma unroll
                    for (int u = 0; u < kLoadsPerRow; ++u) {
                        const int j = j0 + lane + 32 * u;
                        x[q][u] = (rows[q] != nullptr && j < N) ? rows[q][j] : 0.0f;
                    }
#pragma unroll
                for (int u = 0; u < kLoadsPerRow; ++u) {
                    const int j = j0 + lane + 32 * u;
                    if (j < N) {
                        const float vj = vc[j];
                        const float vpj = lazy ? vn[j] : 0.0f, wpj = lazy ? wp[j] : 0.0f;
#pragma unroll
                        for (int q = 0; q < kRowsPerWarp; ++q) {
                            if (rows[q] == nullptr) continue;
                            float xv = x[q][u];
                            if (lazy) {
                                xv -= __fmul_rn(vi[q], wpj) + __fmul_rn(wi[q], vpj);
                                rows[q][j] = xv;
                            }
                            acc[q] = fmaf(xv, vj, acc[q]);
                        }
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < kRowsPerWarp; ++q) {
                const float a = warp_sum(acc[q]);
                if (rows[q] != nullptr) {
                    const int i = first + (t0 + q) * C;
                    const float pi = tau * a;
                    // p_i into every CTA's copy of p (lane l to CTA l): after the barrier all of p is local
                    if (lane < C) st_remote(&pb[i], static_cast<uint32_t>(lane), pi);
                    dot = fmaf(pi, vc[i], dot);
                }
            }
        }
        // lanes of a warp hold the same dot; sum one lane per warp
        const float dsum = block_sum(lane == 0 ? dot : 0.0f, red);
        if (threadIdx.x < static_cast<unsigned>(C))
            st_remote(&part[cur * kMaxClusterCtas + r], threadIdx.x, dsum);
        cluster_barrier();  // every CTA's p, p^T v and updated rows are visible
        // (C) w = p - (tau / 2) (p^T v) v over the whole trailing range (p^T v summed in rank order)
        float s = 0.0f;
        for (int q = 0; q < C; ++q) s += part[cur * kMaxClusterCtas + q];
        const float c = -0.5f * tau * s;
        for (int j = k + 1 + threadIdx.x; j < N; j += kSytrdThreads) wc[j] = fmaf(c, vc[j], pb[j]);
        __syncthreads();
        if (r == 0) {  // row k is read by nobody any more: it keeps the reflector
            float* rowv = Wb + static_cast<int64_t>(k) * N;
            for (int j = k + 1 + threadIdx.x; j < N; j += kSytrdThreads) rowv[j] = vc[j];
            if (threadIdx.x == 0) {
                db[k] = R.d;
                eb[k] = R.beta;
                tb[k] = tau;
            }
        }
        // row k + 1 with column k's update, in registers: the next reflector (or, after the last one, T's trailing
        // 2 x 2 block)
        const float* rown = Wb + static_cast<int64_t>(k + 1) * N;
        const float vk1 = vc[k + 1], wk1 = wc[k + 1];
        if (k + 3 < N) {
            float ss = 0.0f;
            for (int j = k + 1 + threadIdx.x; j < N; j += kSytrdThreads) {
                const float x = __ldcg(rown + j) - (__fmul_rn(vk1, wc[j]) + __fmul_rn(wk1, vc[j]));
                if (j == k + 1) scal2[0] = x;
                else if (j == k + 2) scal2[1] = x;
                else {
                    vn[j] = x;
                    ss = fmaf(x, x, ss);
                }
            }
            // the reduction synchronises the CTA before scal2 is read
            const float sig = block_sum(ss, red);
            const float dn = scal2[0], alpha = scal2[1];
            Reflector Rn{dn, alpha, 0.0f};
            float scl = 0.0f;
            if (sig > 0.0f) {
                Rn.beta = -copysignf(sqrtf(fmaf(alpha, alpha, sig)), alpha);
                Rn.tau = (Rn.beta - alpha) / Rn.beta;
                scl = 1.0f / (alpha - Rn.beta);
            }
            for (int j = k + 3 + threadIdx.x; j < N; j += kSytrdThreads) vn[j] *= scl;
            if (threadIdx.x == 0) vn[k + 2] = 1.0f;
            __syncthreads();
            R = Rn;
        } else if (r == 0 && threadIdx.x == 0) {  // k = N - 3: rows N - 2 and N - 1 get column k's update
            const float* rowl = Wb + static_cast<int64_t>(N - 1) * N;
            const float vl = vc[N - 1], wl = wc[N - 1];
            db[N - 2] = __ldcg(rown + N - 2) - (__fmul_rn(vk1, wc[N - 2]) + __fmul_rn(wk1, vc[N - 2]));
            eb[N - 2] = __ldcg(rown + N - 1) - (__fmul_rn(vk1, wc[N - 1]) + __fmul_rn(wk1, vc[N - 1]));
            db[N - 1] = __ldcg(rowl + N - 1) - (__fmul_rn(vl, wc[N - 1]) + __fmul_rn(wl, vc[N - 1]));
        }
    }
    if (r == 0 && threadIdx.x == 0) {
        if (N == 2) {
            db[0] = Wb[0];
            eb[0] = Wb[1];
            db[1] = Wb[N + 1];
        } else if (N == 1) {
            db[0] = Wb[0];
        }
        eb[N - 1] = 0.0f;
        tb[N - 1] = 0.0f;
        if (N >= 2) tb[N - 2] = 0.0f;
    }
    cluster_barrier();  // no CTA leaves while another may still read its shared memory
}

// ---- eigenvalues of T: multisection on Sturm counts ------------------------------------------------------------

// 1 / x by the hardware reciprocal (within 1 ulp; |x| >= pivmin >= 1e-30 is normal here)
__device__ __forceinline__ float rcp_hw(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Numbers of eigenvalues of T below each of K points (FP32, pivots floored at pivmin in magnitude).  The quotient
// e^2 / q takes the hardware reciprocal: the division's full-precision sequence made the search bound by its
// instruction count, and a count from quotients within 1 ulp is the exact count of a T whose e^2 differ by that
// much.  The K recurrences are independent, so their latencies overlap.
template <int K>
__device__ __forceinline__ void sturm_counts(const float* d, const float* e2, int N, const float (&x)[K], float pivmin,
                                             int (&cnt)[K]) {
    float q[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        q[k] = d[0] - x[k];
        if (fabsf(q[k]) < pivmin) q[k] = -pivmin;
        cnt[k] = q[k] < 0.0f;
    }
    for (int i = 1; i < N; ++i) {
        const float di = d[i], ei = e2[i - 1];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            q[k] = (di - x[k]) - ei * rcp_hw(q[k]);
            if (fabsf(q[k]) < pivmin) q[k] = -pivmin;
            cnt[k] += q[k] < 0.0f;
        }
    }
}

// grid (ceil(N / kBisectThreads), batch): eigenvalue j of matrix b into evals[b][j], ascending.  Each step splits
// the bracket at kSectPts equispaced points (multisection: kBisectSteps steps narrow it by 2^-48, as 48 halvings
// would); a thread's recurrences run interleaved, and the small blocks spread the eigenvalues over every SM.
__global__ void __launch_bounds__(kBisectThreads)
k_tridiag_bisect(const float* __restrict__ d_all, const float* __restrict__ e_all, int N, float* __restrict__ evals,
                 float* __restrict__ tnorm_out) {
    extern __shared__ float sm[];
    float* d = sm;
    float* e2 = sm + N;
    __shared__ float red[34];
    const int b = blockIdx.y;
    const float* db = d_all + static_cast<int64_t>(b) * N;
    const float* eb = e_all + static_cast<int64_t>(b) * N;
    float lo = INFINITY, hi = -INFINITY;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const float di = db[i];
        const float el = i > 0 ? fabsf(eb[i - 1]) : 0.0f;
        const float er = i + 1 < N ? fabsf(eb[i]) : 0.0f;
        d[i] = di;
        if (i + 1 < N) e2[i] = eb[i] * eb[i];
        lo = fminf(lo, di - el - er);
        hi = fmaxf(hi, di + el + er);
    }
    // block min / max through warp shuffles
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
        red[threadIdx.x >> 5] = lo;
        red[16 + (threadIdx.x >> 5)] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float l = red[0], h = red[16];
        for (int w = 1; w < (blockDim.x >> 5); ++w) {
            l = fminf(l, red[w]);
            h = fmaxf(h, red[16 + w]);
        }
        red[32] = l;
        red[33] = h;
    }
    __syncthreads();
    const float gl = red[32], gu = red[33];
    const float tnorm = fmaxf(fabsf(gl), fabsf(gu));
    if (blockIdx.x == 0 && threadIdx.x == 0) tnorm_out[b] = tnorm;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    const float pivmin = fmaxf(1e-30f, 1.2e-7f * 1e-6f * tnorm);
    float a = gl - 1e-6f * tnorm - 1e-30f, z = gu + 1e-6f * tnorm + 1e-30f;
    // the interval [a, z) holds the (j+1)-th smallest eigenvalue: count(a) <= j < count(z)
    for (int it = 0; it < kBisectSteps; ++it) {
        const float w = z - a;
        float m[kSectPts];
        bool inside = false;
#pragma unroll
        for (int k = 0; k < kSectPts; ++k) {
            m[k] = a + w * (static_cast<float>(k + 1) / static_cast<float>(kSectPts + 1));
            inside |= m[k] > a && m[k] < z;
        }
        if (!inside) break;  // the bracket is down to adjacent floats
        int cnt[kSectPts];
        sturm_counts<kSectPts>(d, e2, N, m, pivmin, cnt);
        // the points rise with k (a + w t is monotone in t), and so do their counts: the lowest point above index j
        // closes the bracket, the highest one at or below it opens it
        float na = a, nz = z;
#pragma unroll
        for (int k = kSectPts - 1; k >= 0; --k)
            if (cnt[k] > j) nz = m[k];
#pragma unroll
        for (int k = 0; k < kSectPts; ++k)
            if (cnt[k] <= j) na = m[k];
        a = na;
        z = nz;
    }
    evals[static_cast<int64_t>(b) * N + j] = 0.5f * (a + z);
}

// ---- eigenvectors of T: inverse iteration in FP64 -------------------------------------------------------------

__device__ __forceinline__ double start_value(int i, int j) {
    uint32_t h = static_cast<uint32_t>(i) * 0x9E3779B1u ^ (static_cast<uint32_t>(j) + 0x7F4A7C15u) * 0x85EBCA77u;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    return 0.5 + static_cast<double>(h & 0xFFFFFF) * (1.0 / 16777216.0);  // in [0.5, 1.5)
}

// grid (ceil(N / 128), batch), one thread per eigenvalue index j.  Scratch S (batch, 3, N, N) FP64: S[0] the
// reciprocal LDL^T pivots 1 / D, S[1] the multipliers L, S[2] the iterate x, element i of thread j at [i * N + j]
// (coalesced over a warp's consecutive j).  Z (batch, N, N) FP32: eigenvector j of T in column j.
//
// Each pass over a vector is a recurrence (one FP64 FMA per element on the previous element's result), so the loads
// it needs are issued kInvitBlock elements ahead into registers: the recurrence then waits only on FMA latency, not
// on a memory round trip per element.  The iterate is normalised lazily: the next solve scales it on the fly.
// Members of a cluster of close eigenvalues get slightly separated shifts (their cluster is orthonormalised after).
__global__ void __launch_bounds__(128)
k_tridiag_invit(const float* __restrict__ d_all, const float* __restrict__ e_all, const float* __restrict__ evals,
                const float* __restrict__ tnorm_all, int N, double* __restrict__ S, float* __restrict__ Z) {
    const int b = blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    const float* db = d_all + static_cast<int64_t>(b) * N;
    const float* eb = e_all + static_cast<int64_t>(b) * N;
    const float* lam = evals + static_cast<int64_t>(b) * N;
    const double tnorm = static_cast<double>(tnorm_all[b]);
    const double tol = kClusterTol * tnorm;
    int j0 = j;  // first index of j's cluster
    while (j0 > 0 && static_cast<double>(lam[j0]) - static_cast<double>(lam[j0 - 1]) < tol) --j0;
    const double lm = static_cast<double>(lam[j]) + (j - j0) * 1e-3 * tol;
    const int64_t NN = static_cast<int64_t>(N) * N;
    double* __restrict__ D = S + (static_cast<int64_t>(b) * 3 + 0) * NN + j;
    double* __restrict__ L = S + (static_cast<int64_t>(b) * 3 + 1) * NN + j;
    double* __restrict__ X = S + (static_cast<int64_t>(b) * 3 + 2) * NN + j;
    float* Zb = Z + static_cast<int64_t>(b) * NN;
    const double pivmin = 1e-14 * tnorm + 1e-300;
    constexpr int B = kInvitBlock;
    // LDL^T of T - lm I as the multipliers L and the reciprocal pivots 1 / D, with the first solve's forward pass
    // z_i = x_i - L_{i-1} z_{i-1} on the pseudo-random start x
    double dcur = static_cast<double>(db[0]) - lm;
    if (fabs(dcur) < pivmin) dcur = -pivmin;
    double inv = 1.0 / dcur;
    double z = start_value(0, j);
    D[0] = inv;
    X[0] = z;
    for (int i = 1; i < N; ++i) {
        const double ei = static_cast<double>(eb[i - 1]);
        const double l = ei * inv;
        dcur = (static_cast<double>(db[i]) - lm) - l * ei;
        if (fabs(dcur) < pivmin) dcur = -pivmin;
        inv = 1.0 / dcur;
        z = fma(-l, z, start_value(i, j));
        L[static_cast<int64_t>(i - 1) * N] = l;
        D[static_cast<int64_t>(i) * N] = inv;
        X[static_cast<int64_t>(i) * N] = z;
    }
    double sc = 1.0;  // pending scale of X
    for (int it = 0; it < kInvitSolves; ++it) {
        if (it > 0) {  // forward: z_i = sc x_i - L_{i-1} z_{i-1}
            z = sc * X[0];
            X[0] = z;
            for (int i0 = 1; i0 < N; i0 += B) {
                double xb[B], lb[B];
#pragma unroll
                for (int u = 0; u < B; ++u) {
                    const int i = i0 + u;
                    xb[u] = i < N ? X[static_cast<int64_t>(i) * N] : 0.0;
                    lb[u] = i < N ? L[static_cast<int64_t>(i - 1) * N] : 0.0;
                }
#pragma unroll
                for (int u = 0; u < B; ++u) {
                    const int i = i0 + u;
                    if (i < N) {
                        z = fma(-lb[u], z, sc * xb[u]);
                        X[static_cast<int64_t>(i) * N] = z;
                    }
                }
            }
        }
        // backward: y_i = z_i / D_i - L_i y_{i+1}
        double y = X[static_cast<int64_t>(N - 1) * N] * D[static_cast<int64_t>(N - 1) * N];
        X[static_cast<int64_t>(N - 1) * N] = y;
        double nrm = y * y;
        for (int i0 = N - 2; i0 >= 0; i0 -= B) {
            double xb[B], db2[B], lb[B];
#pragma unroll
            for (int u = 0; u < B; ++u) {
                const int i = i0 - u;
                xb[u] = i >= 0 ? X[static_cast<int64_t>(i) * N] : 0.0;
                db2[u] = i >= 0 ? D[static_cast<int64_t>(i) * N] : 0.0;
                lb[u] = i >= 0 ? L[static_cast<int64_t>(i) * N] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < B; ++u) {
                const int i = i0 - u;
                if (i >= 0) {
                    y = fma(xb[u], db2[u], -lb[u] * y);
                    X[static_cast<int64_t>(i) * N] = y;
                    nrm = fma(y, y, nrm);
                }
            }
        }
        sc = nrm > 0.0 ? 1.0 / sqrt(nrm) : 0.0;
    }
    for (int i = 0; i < N; ++i) Zb[static_cast<int64_t>(i) * N + j] = static_cast<float>(sc * X[static_cast<int64_t>(i) * N]);
}

// grid (ceil(N / 4), batch), 128 threads: a warp per eigenvalue index j; the warp of each cluster's first eigenvalue
// orthonormalises the cluster's columns of Z (modified Gram-Schmidt, lanes over the rows, FP64 sums)
__global__ void __launch_bounds__(128)
k_cluster_orth(const float* __restrict__ evals, const float* __restrict__ tnorm_all, int N, float* __restrict__ Z) {
    const int b = blockIdx.y;
    const int j = blockIdx.x * 4 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (j >= N) return;
    const float* lam = evals + static_cast<int64_t>(b) * N;
    const double tol = kClusterTol * static_cast<double>(tnorm_all[b]);
    if (j > 0 && static_cast<double>(lam[j]) - static_cast<double>(lam[j - 1]) < tol) return;
    int jend = j + 1;
    while (jend < N && static_cast<double>(lam[jend]) - static_cast<double>(lam[jend - 1]) < tol) ++jend;
    if (jend - j < 2) return;
    float* Zb = Z + static_cast<int64_t>(b) * N * N;
    for (int m = j; m < jend; ++m) {
        for (int q = j; q < m; ++q) {
            double pr = 0.0;
            for (int i = lane; i < N; i += 32)
                pr = fma(static_cast<double>(Zb[static_cast<int64_t>(i) * N + q]),
                         static_cast<double>(Zb[static_cast<int64_t>(i) * N + m]), pr);
            pr = warp_sum(pr);
            for (int i = lane; i < N; i += 32) {
                float* zm = Zb + static_cast<int64_t>(i) * N + m;
                *zm = static_cast<float>(static_cast<double>(*zm) - pr * static_cast<double>(Zb[static_cast<int64_t>(i) * N + q]));
            }
            __syncwarp();
        }
        double nrm = 0.0;
        for (int i = lane; i < N; i += 32) {
            const double v = static_cast<double>(Zb[static_cast<int64_t>(i) * N + m]);
            nrm = fma(v, v, nrm);
        }
        nrm = warp_sum(nrm);
        const double sc = nrm > 0.0 ? 1.0 / sqrt(nrm) : 0.0;
        for (int i = lane; i < N; i += 32) {
            float* zm = Zb + static_cast<int64_t>(i) * N + m;
            *zm = static_cast<float>(sc * static_cast<double>(*zm));
        }
        __syncwarp();
    }
}

// ---- back-transformation: U = Q Z with Q = H_0 ... H_{N-3} in WY blocks ---------------------------------------

// grid (nblocks, batch), kWy * kWy threads: T_q of block q (upper triangular, I - V T V^T = H_{k0} ... H_{k0+15}),
// from G = V^T V and tau (LAPACK larft, forward / columnwise)
__global__ void __launch_bounds__(kWy * kWy)
k_wy_factors(const float* __restrict__ W, const float* __restrict__ tau_all, int N, int n_refl,
             float* __restrict__ Tq) {
    __shared__ float G[kWy][kWy + 1];
    __shared__ float T[kWy][kWy + 1];
    const int b = blockIdx.y, q = blockIdx.x;
    const int k0 = q * kWy;
    const int a = threadIdx.x / kWy, c = threadIdx.x % kWy;
    const float* Wb = W + static_cast<int64_t>(b) * N * N;
    const float* tau = tau_all + static_cast<int64_t>(b) * N;
    const int ka = k0 + a, kc = k0 + c;
    float g = 0.0f;
    if (a < c && kc < n_refl) {  // v_a . v_c over rows > kc (v_c is zero above row kc + 1, where it is 1)
        const float* va = Wb + static_cast<int64_t>(ka) * N;
        const float* vc = Wb + static_cast<int64_t>(kc) * N;
        g = va[kc + 1];
        for (int i = kc + 2; i < N; ++i) g = fmaf(va[i], vc[i], g);
    }
    G[a][c] = g;
    T[a][c] = 0.0f;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 0; i < kWy; ++i) {
            const float ti = (k0 + i < n_refl) ? tau[k0 + i] : 0.0f;
            // T[0:i, i] = -ti * T[0:i, 0:i] G[0:i, i]
            for (int rr = 0; rr < i; ++rr) {
                float s = 0.0f;
                for (int m = rr; m < i; ++m) s = fmaf(T[rr][m], G[m][i], s);
                T[rr][i] = -ti * s;
            }
            T[i][i] = ti;
        }
    }
    __syncthreads();
    Tq[((static_cast<int64_t>(b) * gridDim.x + q) * kWy + a) * kWy + c] = T[a][c];
}

// grid (ceil(N / kTile), batch): columns c0 .. c0+15 of Z (eigenvectors of T) to eigenvector rows of A in U
__global__ void __launch_bounds__(kBtThreads)
k_backtransform(const float* __restrict__ W, const float* __restrict__ Tq_all, const float* __restrict__ Z, int N,
                int n_refl, int nblocks, float* __restrict__ U) {
    extern __shared__ float sm[];
    float* Zt = sm;                          // N x kTile
    float* Vc = Zt + N * kTile;              // kWy x kChunk: Vc[a * kChunk + ii] = v_{k0+a}[i0 + ii]
    __shared__ float Sm[kWy][kTile + 1];
    __shared__ float Sp[kWy][kTile + 1];
    __shared__ float Tm[kWy][kWy + 1];
    const int b = blockIdx.y;
    const int c0 = blockIdx.x * kTile;
    const int64_t NN = static_cast<int64_t>(N) * N;
    const float* Wb = W + b * NN;
    const float* Zb = Z + b * NN;
    const int ncols = min(kTile, N - c0);
    for (int t = threadIdx.x; t < N * kTile; t += kBtThreads) {
        const int i = t / kTile, c = t % kTile;
        Zt[t] = c < ncols ? Zb[static_cast<int64_t>(i) * N + c0 + c] : 0.0f;
    }
    const int a = threadIdx.x / kTile, cc = threadIdx.x % kTile;  // one (reflector, column) pair per thread
    // V is staged kChunk rows at a time; each thread loads its kPre entries of the next stage into registers while
    // the current one is used, so the stage's global loads overlap the block's arithmetic instead of preceding it
    constexpr int kPre = kChunk * kWy / kBtThreads;
    static_assert(kChunk * kWy % kBtThreads == 0, "stage entries per thread");
    float pre[kPre];
    int pk0 = 0;
    auto load_stage = [&](int i0) {
#pragma unroll
        for (int u = 0; u < kPre; ++u) {
            const int t = threadIdx.x + u * kBtThreads;
            const int aa = t / kChunk, ii = t % kChunk, i = i0 + ii, k = pk0 + aa;
            pre[u] = (i < N && k < n_refl && i > k) ? Wb[static_cast<int64_t>(k) * N + i] : 0.0f;
        }
    };
    auto store_stage = [&]() {
#pragma unroll
        for (int u = 0; u < kPre; ++u) Vc[threadIdx.x + u * kBtThreads] = pre[u];
    };
    for (int q = nblocks - 1; q >= 0; --q) {
        const int k0 = q * kWy;
        const int r0 = k0 + 1;  // first row any reflector of the block touches
        if (threadIdx.x < kWy * kWy)
            Tm[threadIdx.x / kWy][threadIdx.x % kWy] = Tq_all[(static_cast<int64_t>(b) * nblocks + q) * kWy * kWy + threadIdx.x];
        float s = 0.0f;
        pk0 = k0;
        // S = V^T Z over the block's rows, V staged kChunk rows at a time (V[i][a] = v_{k0+a}[i]; consecutive
        // threads read one row of W)
        load_stage(r0);
        for (int i0 = r0; i0 < N; i0 += kChunk) {
            __syncthreads();
            store_stage();
            __syncthreads();
            if (i0 + kChunk < N) load_stage(i0 + kChunk);
            const int iend = min(kChunk, N - i0);
            for (int ii = 0; ii < iend; ++ii) s = fmaf(Vc[a * kChunk + ii], Zt[(i0 + ii) * kTile + cc], s);
        }
        Sm[a][cc] = s;
        __syncthreads();
        // S' = T S
        float sp = 0.0f;
        for (int m = a; m < kWy; ++m) sp = fmaf(Tm[a][m], Sm[m][cc], sp);
        Sp[a][cc] = sp;
        __syncthreads();
        // Z -= V S'
        load_stage(r0);
        for (int i0 = r0; i0 < N; i0 += kChunk) {
            __syncthreads();
            store_stage();
            __syncthreads();
            if (i0 + kChunk < N) load_stage(i0 + kChunk);
            const int iend = min(kChunk, N - i0);
            for (int t = threadIdx.x; t < iend * kTile; t += kBtThreads) {
                const int ii = t / kTile, c = t % kTile;
                float acc = Zt[(i0 + ii) * kTile + c];
#pragma unroll
                for (int m = 0; m < kWy; ++m) acc = fmaf(-Vc[m * kChunk + ii], Sp[m][c], acc);
                Zt[(i0 + ii) * kTile + c] = acc;
            }
        }
        __syncthreads();
    }
    // eigenvector c0 + c is column c of the tile: one row of U each
    for (int c = 0; c < ncols; ++c)
        for (int i = threadIdx.x; i < N; i += kBtThreads)
            U[b * NN + static_cast<int64_t>(c0 + c) * N + i] = Zt[i * kTile + c];
}

struct OwnLayout {
    size_t W, Z, S, d, e, tau, ev, tn, T, total;
    int nblocks;
};

size_t up256(size_t x) { return (x + 255) / 256 * 256; }

OwnLayout own_layout(int N, int batch) {
    OwnLayout L;
    const size_t NN = static_cast<size_t>(N) * N * batch;
    const int n_refl = N > 2 ? N - 2 : 0;
    L.nblocks = n_refl > 0 ? (n_refl + kWy - 1) / kWy : 0;
    size_t o = 0;
    L.W = o; o += up256(4 * NN);
    L.Z = o; o += up256(4 * NN);
    L.S = o; o += up256(8 * 3 * NN);
    L.d = o; o += up256(4 * static_cast<size_t>(N) * batch);
    L.e = o; o += up256(4 * static_cast<size_t>(N) * batch);
    L.tau = o; o += up256(4 * static_cast<size_t>(N) * batch);
    L.ev = o; o += up256(4 * static_cast<size_t>(N) * batch);
    L.tn = o; o += up256(4 * static_cast<size_t>(batch));
    L.T = o; o += up256(4 * static_cast<size_t>(L.nblocks > 0 ? L.nblocks : 1) * kWy * kWy * batch);
    L.total = o;
    return L;
}

}  // namespace

namespace flmm {

size_t eigh_own_workspace_bytes(int N, int batch) { return own_layout(N, batch).total; }

// A (batch, N, N) FP32 symmetric in, eigenvector rows out (ascending eigenvalues into evals (batch, N) FP32)
int eigh_own_f32(float* A, int N, int batch, float* evals, void* work, cudaStream_t st) {
    const OwnLayout L = own_layout(N, batch);
    char* base = static_cast<char*>(work);
    float* W = reinterpret_cast<float*>(base + L.W);
    float* Z = reinterpret_cast<float*>(base + L.Z);
    double* S = reinterpret_cast<double*>(base + L.S);
    float* d = reinterpret_cast<float*>(base + L.d);
    float* e = reinterpret_cast<float*>(base + L.e);
    float* tau = reinterpret_cast<float*>(base + L.tau);
    float* tn = reinterpret_cast<float*>(base + L.tn);
    float* Tq = reinterpret_cast<float*>(base + L.T);
    const size_t NN = static_cast<size_t>(N) * N;
    FLMM_CUDA(cudaMemcpyAsync(W, A, 4 * NN * batch, cudaMemcpyDeviceToDevice, st));
    // 1. tridiagonalisation, one cluster per matrix
    const int Np = (N + 3) & ~3;
    const size_t smem1 = sizeof(float) * (6 * static_cast<size_t>(Np) + 32 + 2 * kMaxClusterCtas + 2);
    // cluster size: as many CTAs per matrix as fill the SMs once (one CTA per SM), 2 to 8
    int dev = 0, sms = 0;
    FLMM_CUDA(cudaGetDevice(&dev));
    FLMM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int C = std::max(2, std::min(kMaxClusterCtas, sms / std::max(batch, 1)));
    // (per device, so set on every call; the call is cheap)
    FLMM_CUDA(cudaFuncSetAttribute(k_sytrd_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
    FLMM_CUDA(cudaFuncSetAttribute(k_backtransform, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = static_cast<unsigned>(C);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(static_cast<unsigned>(C * batch), 1, 1);
    cfg.blockDim = dim3(kSytrdThreads, 1, 1);
    cfg.dynamicSmemBytes = smem1;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    FLMM_CUDA(cudaLaunchKernelEx(&cfg, k_sytrd_cluster, W, N, d, e, tau));
    int rc = check_launch("k_sytrd_cluster");
    if (rc) return rc;
    // 2. eigenvalues
    k_tridiag_bisect<<<dim3(ceil_div(N, kBisectThreads), batch), kBisectThreads,
                       sizeof(float) * 2 * static_cast<size_t>(N), st>>>(
        d, e, N, evals, tn);
    if ((rc = check_launch("k_tridiag_bisect"))) return rc;
    // 3. eigenvectors of T
    k_tridiag_invit<<<dim3(ceil_div(N, 128), batch), 128, 0, st>>>(d, e, evals, tn, N, S, Z);
    if ((rc = check_launch("k_tridiag_invit"))) return rc;
    k_cluster_orth<<<dim3(ceil_div(N, 4), batch), 128, 0, st>>>(evals, tn, N, Z);
    if ((rc = check_launch("k_cluster_orth"))) return rc;
    // 4. back-transformation into A
    const int n_refl = N > 2 ? N - 2 : 0;
    if (L.nblocks > 0) {
        k_wy_factors<<<dim3(L.nblocks, batch), kWy * kWy, 0, st>>>(W, tau, N, n_refl, Tq);
        if ((rc = check_launch("k_wy_factors"))) return rc;
    }
    const size_t smem4 = sizeof(float) * (static_cast<size_t>(N) * kTile + kChunk * kWy);
    k_backtransform<<<dim3(ceil_div(N, kTile), batch), kBtThreads, smem4, st>>>(W, Tq, Z, N, n_refl, L.nblocks, A);
    return check_launch("k_backtransform");
}

}  // namespace flmm
