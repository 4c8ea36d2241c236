// Exact evaluation of the fast delta fit's derivative and the safeguarded Newton refinement, shared by the grid
// path (flmm_delta_fast.cu) and the learned-proposal path (flmm_delta_learned.cu).
#pragma once

#include <math.h>

#include "flmm_common.cuh"

namespace flmm {
namespace dfit {

// FP32 throughout: the sums behind g are FP32, and the FP64 pipe of this part runs at a small fraction of the FP32
// rate, so only the abscissa x = log delta itself is kept in FP64.
struct NewtonEval {
    float g;      // T1 - Neff S2 / S1 (sign of d loss / d log delta)
    float gp;     // dg / dx
    float loss;   // Neff log S1 + sum log (s + delta), up to constants
};

// Sums over the aligned group of W lanes (W = 16 or 32) holding this thread; every lane of the group gets the sum.
// Groups of 16 let one warp work on two columns, which then share the per-evaluation scalar work (reductions,
// divisions, the Newton and bracketing logic) that dominates a column's instruction count.
template <int W>
__device__ __forceinline__ unsigned group_mask() {
    return W == 32 ? 0xffffffffu : (((1u << W) - 1u) << (threadIdx.x & 31u & ~static_cast<unsigned>(W - 1)));
}

template <int W>
__device__ __forceinline__ float group_sum(float v) {
    const unsigned m = group_mask<W>();
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) v += __shfl_xor_sync(m, v, o);
    return v;
}

// group sum of a compensated pair (hi + lo), TwoSum at every level of the butterfly
template <int W>
__device__ __forceinline__ float group_sum_pair(float hi, float lo) {
    const unsigned m = group_mask<W>();
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(m, hi, o);
        const float ol = __shfl_xor_sync(m, lo, o);
        float sum, err;
        two_sum(hi, oh, sum, err);
        hi = sum;
        lo = lo + ol + err;
    }
    return hi + lo;
}

// One evaluation by a group of W lanes at x = log delta (x is uniform over the group), all in FP32.
//
// g is formed around the centre c = 1 / (sbar + delta), sbar the mean eigenvalue: with d_n = r_n - c =
// (sbar - s_n) r_n c,
//     g = sum d - Neff (c E1 + E2) / (c U + E1),   U = sum u^2, E1 = sum u^2 d, E2 = sum u^2 d^2,
// which is T1 - Neff S2 / S1 rearranged so that no O(r) terms cancel: when delta >> s the r_n are nearly equal and
// the information in g is in their O(s / delta) spread, which the centred terms carry at full FP32 precision
// (compensated sums for the first-order terms).  delta = exp(x) is formed from a hi / lo split of x so that it is
// exact to FP32 rounding at any x.
struct EvalPoint {
    float delta, c;
};

__device__ __forceinline__ EvalPoint eval_point(double x, float sbar) {
    const float xh = static_cast<float>(x);
    const float xl = static_cast<float>(x - static_cast<double>(xh));
    const float delta = expf(xh) * (1.0f + xl);
    return {delta, 1.0f / (sbar + delta)};
}

// 1 / x for normal x > 0 by the hardware reciprocal (within 1 ulp; one instruction where the correctly rounded
// reciprocal takes several): each term of the sums below then carries ~2^-23 instead of 2^-24 relative error, which
// averages out over Neff like the rest of the terms' rounding.
__device__ __forceinline__ float rcp_approx_pos(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// per-lane partial sums of one evaluation
struct EvalSums {
    float d1 = 0.f, cd1 = 0.f, e1 = 0.f, ce1 = 0.f, e2 = 0.f, e3 = 0.f, f2 = 0.f, sl = 0.f;

    __device__ __forceinline__ void add(float sn, float dsn, float uu, const EvalPoint& pt, bool want_loss) {
        const float sd = sn + pt.delta;
        const float r = rcp_approx_pos(sd);
        const float d = dsn * r * pt.c;
        neumaier(d1, cd1, d);
        neumaier(e1, ce1, uu * d);
        const float ud = uu * d * d;
        e2 += ud;
        e3 += ud * d;
        f2 += d * d;
        if (want_loss) sl += __logf(sd);
    }
};

template <int W>
__device__ inline NewtonEval finish_eval(const EvalSums& t, float U, int Neff, const EvalPoint& pt, bool want_loss) {
    const float D1 = group_sum_pair<W>(t.d1, t.cd1);
    const float E1 = group_sum_pair<W>(t.e1, t.ce1);
    const float E2 = group_sum<W>(t.e2);
    const float E3 = group_sum<W>(t.e3);
    const float F2 = group_sum<W>(t.f2);
    const float c = pt.c;
    NewtonEval e;
    const float neff = static_cast<float>(Neff);
    if (U > 0.0f) {
        e.g = D1 - neff * (c * E1 + E2) / (c * U + E1);
        // dg/dx = delta (-T2 + Neff (2 S3 / S1 - (S2 / S1)^2)) in the same centred sums: with F2 = sum d^2,
        // E3 = sum u^2 d^3, a = E1 / (c U), b = E2 / (c^2 U), t3 = E3 / (c^3 U) one has T2 = Neff c^2 + 2 c D1 + F2,
        // S1 = c U (1 + a), S2 = c^2 U (1 + 2a + b), S3 = c^3 U (1 + 3a + 3b + t3), and the O(1) terms cancel exactly
        const float a = E1 / (c * U), b = E2 / (c * c * U), t3 = E3 / (c * c * c * U);
        const float br = -2.0f * D1 / (c * neff) - F2 / (c * c * neff) + (2.0f * a + 4.0f * b + 2.0f * t3) / (1.0f + a) -
                         (a + b) * (a + b) / ((1.0f + a) * (1.0f + a));
        e.gp = pt.delta * neff * c * c * br;
    } else {  // all-zero rotated column: the loss only grows with delta
        e.g = 1.0f;
        e.gp = 1.0f;
    }
    e.loss = 0.0f;
    if (want_loss) e.loss = neff * logf(fmaxf(c * U + E1, 1e-30f)) + group_sum<W>(t.sl);
    return e;
}

// One evaluation by a group of W lanes over a column read from global (L1 / L2) memory; dsb[n] = sbar - s[n] and the
// column's sum of squares U are precomputed.  Not inlined: the refinement calls the evaluator from a dozen places,
// and one shared copy of the loop keeps the instruction cache warm (inlined copies made instruction fetch the main
// stall).
template <int W>
static __device__ __noinline__ NewtonEval eval_global_column(const float* __restrict__ s32,
                                                             const float* __restrict__ dsb,
                                                             const float* __restrict__ u, int Neff, float sbar,
                                                             float U, double x, bool want_loss) {
    const int lane = threadIdx.x & (W - 1);
    const EvalPoint pt = eval_point(x, sbar);
    EvalSums t;
    // four iterations per trip: their loads issue together instead of each waiting out its own L1 / L2 latency
    // (each lane still adds its terms in the same order, so the sums are unchanged)
#pragma unroll 4
    for (int n = lane; n < Neff; n += W) t.add(s32[n], dsb[n], u[n] * u[n], pt, want_loss);
    return finish_eval<W>(t, U, Neff, pt, want_loss);
}

// Evaluator over a column in global memory, W lanes per column.  (Keeping the squares in registers instead cost
// occupancy and ran slower.)
template <int W>
struct GlobalColumn {
    const float* s32;
    const float* dsb;
    const float* u;
    int Neff;
    float sbar, U;

    __device__ NewtonEval operator()(double x, bool want_loss) const {
        return eval_global_column<W>(s32, dsb, u, Neff, sbar, U, x, want_loss);
    }
};

// Safeguarded Newton on g in a bracket with g(lo) < 0 < g(hi), starting at x0 (the bracket's midpoint if x0 is not
// inside).  The FP32 sums put a noise floor of ~1e-7 on x: near the root the Newton steps stop shrinking and jump
// around the root by that much, so the iteration ends once a step or the bracket is below 1e-7.  It also ends right
// after a Newton step shorter than kNewtonDone: Newton's error after a step of length h is ~|g'' / 2g'| h^2, below
// the noise floor for h < 3e-5 on these losses, so the evaluation that would only confirm convergence is skipped.
constexpr double kNewtonDone = 3e-5;

template <class Ev>
__device__ double newton_in_bracket(const Ev& ev, double lo, double hi, double x0, const NewtonEval* first = nullptr) {
    const bool inside = x0 > lo && x0 < hi;
    double x = inside ? x0 : 0.5 * (lo + hi);
    for (int it = 0; it < 60; ++it) {
        const NewtonEval e = (it == 0 && inside && first) ? *first : ev(x, false);
        if (e.g == 0.0f) break;
        if (e.g < 0.0f) lo = x; else hi = x;
        double xn = x - static_cast<double>(e.g / e.gp);
        const bool newton = xn > lo && xn < hi;
        if (!newton) xn = 0.5 * (lo + hi);
        const double stepx = fabs(xn - x);
        x = xn;
        if (stepx < 1e-7 || hi - lo < 1e-7 || (newton && stepx < kNewtonDone)) break;
    }
    return x;
}

// Root of the cubic Hermite interpolant of g on [xl, xr] through (xl, gl, dl) and (xr, gr, dr), dl and dr the
// derivatives dg/dx, for gl < 0 < gr: safeguarded Newton on t = (x - xl) / (xr - xl) in FP32 from the secant point.
// With the grid spacing h the interpolant is within ~h^4 max|g^(4)| / 384 of g, so the root lands ~1e-5 or closer
// to the stationary point, where one Newton step of the exact evaluator finishes.
__device__ inline double hermite_root(double xl, double xr, float gl, float dl, float gr, float dr) {
    const float h = static_cast<float>(xr - xl);
    const float hl = h * dl, hr = h * dr;
    float lo = 0.0f, hi = 1.0f, t = gl / (gl - gr);
    for (int it = 0; it < 12; ++it) {
        const float t2 = t * t, t3 = t2 * t;
        const float p = (2.0f * t3 - 3.0f * t2 + 1.0f) * gl + (t3 - 2.0f * t2 + t) * hl + (3.0f * t2 - 2.0f * t3) * gr +
                        (t3 - t2) * hr;
        if (p == 0.0f) break;
        if (p < 0.0f) lo = t; else hi = t;
        const float dp = (6.0f * t2 - 6.0f * t) * gl + (3.0f * t2 - 4.0f * t + 1.0f) * hl + (6.0f * t - 6.0f * t2) * gr +
                         (3.0f * t2 - 2.0f * t) * hr;
        float tn = t - p / dp;
        if (!(tn > lo && tn < hi)) tn = 0.5f * (lo + hi);
        const bool done = fabsf(tn - t) < 1e-7f;
        t = tn;
        if (done) break;
    }
    return xl + static_cast<double>(t) * (xr - xl);
}

// Evaluations a first pass over the column may have done already: at grid[i] (`at`) and, when the argmin is inside
// the grid, at its neighbours grid[i - 1] and grid[i + 1] (`lo`, `hi`).
struct FirstEvals {
    NewtonEval at, lo, hi;
    bool have_at = false, have_nb = false;
};

// log delta of one column from its grid argmin i (uniform over the column's lanes).  `first`, if given, holds
// evaluations already done.
template <class Ev>
__device__ double refine_column(const Ev& ev, const double* __restrict__ grid, int G, int i, int refine,
                                const FirstEvals* first = nullptr) {
    double out = grid[i];
    const NewtonEval* at = (first && first->have_at) ? &first->at : nullptr;
    if (refine && i > 0 && i < G - 1) {
        // the usual case: d loss / d log delta changes sign between the argmin's neighbours
        const double a = grid[i - 1], b = grid[i + 1];
        const bool nb = first && first->have_nb;
        const float ga = nb ? first->lo.g : ev(a, false).g;
        if (ga < 0.0f && (nb ? first->hi.g : ev(b, false).g) > 0.0f) {
            if (nb && at) {
                // g and dg/dx at all three nodes: start from the Hermite root on the half that changes sign
                const float gi = at->g;
                if (gi == 0.0f) return grid[i];
                const bool left = gi > 0.0f;
                const double xl = left ? a : grid[i], xr = left ? grid[i] : b;
                const NewtonEval& el = left ? first->lo : *at;
                const NewtonEval& er = left ? *at : first->hi;
                return newton_in_bracket(ev, xl, xr, hermite_root(xl, xr, el.g, el.gp, er.g, er.gp));
            }
            return newton_in_bracket(ev, a, b, grid[i], at);
        }
    }
    if (refine && G > 1) {
        // The FP32 grid argmin is only as good as the FP32 loss (~1e-4 absolute); on flat losses it can sit several
        // nodes from the minimum.  The exact derivative sign at that node says which side the minimum is on, and a
        // binary search over the grid nodes on that side finds where d loss / d log delta changes sign, so the
        // bracket [grid[i-1], grid[i+1]] always contains the minimum (for losses with one minimum on that side).
        const float gi = at ? at->g : ev(grid[i], false).g;
        if (gi < 0.0f) {
            if (ev(grid[G - 1], false).g < 0.0f) {
                i = G - 1;  // still falling at the top of the grid
            } else {
                int lo = i, hi = G - 1;  // g(lo) < 0 <= g(hi)
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (ev(grid[mid], false).g < 0.0f) lo = mid; else hi = mid;
                }
                i = hi;
            }
        } else if (gi > 0.0f) {
            if (ev(grid[0], false).g > 0.0f) {
                i = 0;  // already rising at the bottom of the grid
            } else {
                int lo = 0, hi = i;  // g(lo) <= 0 < g(hi)
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (ev(grid[mid], false).g > 0.0f) hi = mid; else lo = mid;
                }
                i = lo;
            }
        }
        const double a = grid[max(i - 1, 0)], b = grid[min(i + 1, G - 1)];
        const NewtonEval ea = ev(a, false);
        const NewtonEval eb = ev(b, false);
        if (ea.g >= 0.0f && eb.g <= 0.0f) {
            // loss rises from a and falls towards b: the minimum is an edge
            out = (ev(a, true).loss <= ev(b, true).loss) ? a : b;
        } else if (ea.g >= 0.0f) {
            out = a;
        } else if (eb.g <= 0.0f) {
            out = b;
        } else {
            out = newton_in_bracket(ev, a, b, grid[i]);
        }
    }
    return out;
}


// Spectrum in shared memory as FP32 (s32) and sbar - s (dsb), sbar the mean eigenvalue; all threads call it.
__device__ inline float load_spectrum(const double* __restrict__ s, int Neff, float* s32, float* dsb, float* sbar_s) {
    for (int n = threadIdx.x; n < Neff; n += blockDim.x) s32[n] = static_cast<float>(s[n]);
    if (threadIdx.x < 32) {
        double acc = 0.0;
        for (int n = threadIdx.x; n < Neff; n += 32) acc += s[n];
        acc = warp_sum(acc);
        if (threadIdx.x == 0) *sbar_s = static_cast<float>(acc / Neff);
    }
    __syncthreads();
    const float sbar = *sbar_s;
    for (int n = threadIdx.x; n < Neff; n += blockDim.x) dsb[n] = sbar - s32[n];
    __syncthreads();
    return sbar;
}

// ---- pieces of the fast fit shared with the learned-proposal path (defined in flmm_delta_fast.cu) -------------

// workspace of the fast fit: grid (G doubles) | Wg (G x Neff) | sum_log (G) | s32 (Neff) | dsb (Neff) | sbar
struct FastWs {
    double* grid;
    float *Wg, *sum_log, *s32, *dsb, *sbar;
};
size_t fast_ws(int Neff, int G);
FastWs carve_fast(void* base, int Neff, int G);
// grid nodes, Wg[g, n] = 1 / (s_n + delta_g) and sum_log[g] = sum_n log(s_n + delta_g)
int launch_grid_tables(const double* s, int Neff, double lo, double hi, int G, const FastWs& w, cudaStream_t st);
// first FP32 grid argmin of the columns cols[0 .. *count) (device list and count), written to idx[col]
int launch_grid_argmin_list(const FastWs& w, const float* UYt, int64_t ldu, int Neff, int P, int G,
                            const int32_t* cols, const int32_t* count, int32_t* idx, cudaStream_t st);
// exact refinement of every column from its grid index idx[p] (the fast fit's second half)
int launch_refine(const double* s, int Neff, const float* UYt, int64_t ldu, int P, int G, const int32_t* idx,
                  int refine, const FastWs& w, double* log_delta, cudaStream_t st);

}  // namespace dfit
}  // namespace flmm
