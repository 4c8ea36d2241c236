// -log10 of the F(1, df2) upper tail, the CLI's p-value (fasterlmm/cli.py:405-406, scipy.stats.f.sf(F, 1, df2)),
// computed in log space so that very large F gives a finite value instead of underflowing to p = 0.
//
// P(F(1, n) > F) = I_x(n / 2, 1 / 2) with x = n / (n + F), the regularized incomplete beta function.  It is
// evaluated from the continued fraction for I_x(a, b) (Abramowitz & Stegun 26.5.8) with the modified Lentz
// algorithm (Lentz 1976; Thompson & Barnett 1986), on the side of the symmetry I_x(a, b) = 1 - I_{1-x}(b, a)
// where the fraction converges fast (x < (a + 1) / (a + b + 2)).  The prefactor x^a (1-x)^b / B(a, b) is kept as a
// logarithm; log B(a, b) is passed in (it depends only on df2).
#pragma once

#ifdef __CUDACC__
#define FLMM_HD __host__ __device__ __forceinline__
#else
#define FLMM_HD inline
#endif

#include <math.h>

namespace flmm {

// Continued fraction of I_x(a, b): returns h with I_x(a, b) = x^a (1 - x)^b / (a B(a, b)) * h.
template <typename T>
FLMM_HD T betacf_lentz(T a, T b, T x, int max_iter) {
    const T tiny = sizeof(T) == 8 ? T(1e-300) : T(1e-30);
    const T eps = sizeof(T) == 8 ? T(1e-15) : T(1e-7);
    const T qab = a + b, qap = a + T(1), qam = a - T(1);
    T c = T(1);
    T d = T(1) - qab * x / qap;
    if (fabs(d) < tiny) d = tiny;
    d = T(1) / d;
    T h = d;
    for (int m = 1; m <= max_iter; ++m) {
        const T mm = T(m), m2 = T(2 * m);
        // even step: d_{2m} = m (b - m) x / ((a + 2m - 1)(a + 2m))
        T aa = mm * (b - mm) * x / ((qam + m2) * (a + m2));
        d = T(1) + aa * d;
        if (fabs(d) < tiny) d = tiny;
        c = T(1) + aa / c;
        if (fabs(c) < tiny) c = tiny;
        d = T(1) / d;
        h *= d * c;
        // odd step: d_{2m+1} = -(a + m)(a + b + m) x / ((a + 2m)(a + 2m + 1))
        aa = -(a + mm) * (qab + mm) * x / ((a + m2) * (qap + m2));
        d = T(1) + aa * d;
        if (fabs(d) < tiny) d = tiny;
        c = T(1) + aa / c;
        if (fabs(c) < tiny) c = tiny;
        d = T(1) / d;
        const T del = d * c;
        h *= del;
        if (fabs(del - T(1)) < eps) break;
    }
    return h;
}

// P(F(1, df2) > F) for F > 0 and finite, lbeta = log B(df2 / 2, 1 / 2), returned as one of two terms: true with v =
// log p (the fraction for I_x(a, b) itself, x < (a + 1) / (a + b + 2)), or false with v = I_{1-x}(b, a) = 1 - p.
template <typename T>
FLMM_HD bool fsf_terms(T F, T df2, T lbeta, T& v) {
    const T a = df2 * T(0.5), b = T(0.5);
    // log x = -log1p(F / n), log(1 - x) = log(F / (n + F))
    const T logx = -log1p(F / df2);
    const T y = F / (df2 + F);  // 1 - x without cancellation
    const T log1mx = log(y);
    const T lpre = a * logx + b * log1mx - lbeta;
    const T x = df2 / (df2 + F);
    if (x < (a + T(1)) / (a + b + T(2))) {
        const T h = betacf_lentz<T>(a, b, x, 4000);
        v = lpre + log(h) - log(a);
        return true;
    }
    const T h = betacf_lentz<T>(b, a, y, 4000);
    v = exp(lpre) * h / b;
    return false;
}

// -log10 P(F(1, df2) > F); lbeta = log B(df2 / 2, 1 / 2).  F <= 0 gives 0 (p = 1); NaN propagates.
template <typename T>
FLMM_HD T neglog10_fsf(T F, T df2, T lbeta) {
    if (!(F > T(0))) return (F == F) ? T(0) : F;
    if (isinf(F)) return T(INFINITY);
    const T ln10 = T(2.302585092994045684);
    T v;
    const T logp = fsf_terms<T>(F, df2, lbeta, v) ? v : log1p(-v);
    return -logp / ln10;
}

// P(F(1, df2) > F) itself (scipy.stats.f.sf(F, 1, df2)): F <= 0 gives 1, +inf gives 0, NaN propagates.
template <typename T>
FLMM_HD T fsf(T F, T df2, T lbeta) {
    if (!(F > T(0))) return (F == F) ? T(1) : F;
    if (isinf(F)) return T(0);
    T v;
    return fsf_terms<T>(F, df2, lbeta, v) ? exp(v) : T(1) - v;
}

}  // namespace flmm
