// special.cuh -- FP64 spherical Bessel function j_l(x), usable on host and device.
//
// Stands in for gsl_sf_bessel_jl, which the reference calls for its interpolation
// tables (SBesselInterpolator.cpp:16), its exact branch (sfb_raw.cpp:51) and its
// zero finder (SphericalBesselZeros.cpp:54-55).  Published algorithms:
//   x^2 < 2l+3 : ascending series, DLMF 10.53.1
//   x >= l     : upward three-term recurrence from j_0, j_1, DLMF 10.51.1
//   otherwise  : Miller's backward recurrence normalised by j_0 or j_1, DLMF 10.74(iii)
// Accuracy ~1e-14 relative to the envelope min(1, 1/x) for l <= 512, x <= 1e4.
#pragma once
#include <math.h>

#if defined(__CUDACC__)
#define CG_HD __host__ __device__ __forceinline__
#else
#define CG_HD inline
#endif

namespace catana_gpu {

constexpr double kPi = 3.14159265358979323846264338327950288;

CG_HD double jl_series(int l, double x) {
    double pre = 1.0;
    for (int i = 1; i <= l; ++i) pre *= x / (2.0 * i + 1.0);
    double hx2 = 0.5 * x * x;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k < 200; ++k) {
        term *= -hx2 / ((double)k * (2.0 * l + 2.0 * k + 1.0));
        sum += term;
        if (fabs(term) < 1e-17 * fabs(sum)) break;
    }
    return pre * sum;
}

CG_HD double jl_upward(int l, double x) {
    double s = sin(x), c = cos(x);
    double j0 = s / x;
    if (l == 0) return j0;
    double j1 = (j0 - c) / x;
    for (int k = 1; k < l; ++k) {
        double j2 = (2.0 * k + 1.0) / x * j1 - j0;
        j0 = j1;
        j1 = j2;
    }
    return j1;
}

CG_HD double jl_miller(int l, double x) {
    double big = (double)l > x ? (double)l : x;
    int nstart = (int)(big + 20.0 + 16.0 * cbrt(big + 1.0));
    double jp1 = 0.0, jk = 1e-200, jl = 0.0;
    if (nstart == l) jl = jk;
    for (int k = nstart; k > 0; --k) {
        double jm1 = (2.0 * k + 1.0) / x * jk - jp1;
        jp1 = jk;
        jk = jm1;
        if (k - 1 == l) jl = jk;
        if (fabs(jk) > 1e200) {
            jk *= 1e-200;
            jp1 *= 1e-200;
            jl *= 1e-200;
        }
    }
    double s = sin(x), c = cos(x);
    double t0 = s / x;
    double t1 = (t0 - c) / x;
    if (fabs(t0) >= fabs(t1)) return jl * (t0 / jk);
    return jl * (t1 / jp1);
}

CG_HD double sbessel_jl(int l, double x) {
    if (x == 0.0) return l == 0 ? 1.0 : 0.0;
    double sgn = 1.0;
    if (x < 0.0) {
        x = -x;
        sgn = (l & 1) ? -1.0 : 1.0;
    }
    if (x * x < 2.0 * l + 3.0) return sgn * jl_series(l, x);
    if (x >= (double)l) return sgn * jl_upward(l, x);
    return sgn * jl_miller(l, x);
}

// j_l(x) for all l in [0, lcount) at one x (FP64): upward recurrence below
// min(x, lcount), Miller's backward recurrence above it.  out[l] for l < lcount.
// Used for the piecewise-cubic tables of the split form, whose nodes are shared
// by every multipole.
CG_HD void sbessel_jl_all(int lcount, double x, double *out) {
    if (x == 0.0) {
        for (int l = 0; l < lcount; ++l) out[l] = l == 0 ? 1.0 : 0.0;
        return;
    }
    double s = sin(x), c = cos(x);
    double t0 = s / x, t1 = (t0 - c) / x;
    // upward part, stable for l <= x
    int lup = (int)x;
    if (lup > lcount - 1) lup = lcount - 1;
    if (x * x < 3.0) lup = -1;  // tiny x: series/Miller for everything but j_0 handled below
    double j0 = t0, j1 = t1;
    if (lup >= 0) out[0] = t0;
    if (lup >= 1) out[1] = t1;
    for (int k = 1; k < lup; ++k) {
        double j2 = (2.0 * k + 1.0) / x * j1 - j0;
        j0 = j1;
        j1 = j2;
        out[k + 1] = j2;
    }
    int lfirst = lup + 1;  // first l still to fill
    if (lfirst >= lcount) return;
    // Miller from above: normalise against the closed form of j_0 or j_1
    double big = (double)(lcount - 1) > x ? (double)(lcount - 1) : x;
    int nstart = (int)(big + 20.0 + 16.0 * cbrt(big + 1.0));
    double jp1 = 0.0, jk = 1e-200;
    for (int k = nstart; k > 0; --k) {
        double jm1 = (2.0 * k + 1.0) / x * jk - jp1;
        jp1 = jk;
        jk = jm1;
        int lk = k - 1;
        if (lk >= lfirst && lk < lcount) out[lk] = jk;
        if (fabs(jk) > 1e200) {
            jk *= 1e-200;
            jp1 *= 1e-200;
            for (int q = (lk > lfirst ? lk : lfirst); q < lcount; ++q) out[q] *= 1e-200;
        }
    }
    double f = (fabs(t0) >= fabs(t1)) ? t0 / jk : t1 / jp1;
    for (int q = lfirst; q < lcount; ++q) out[q] *= f;
}

}  // namespace catana_gpu
