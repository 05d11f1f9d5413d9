/*
 * catana_oracle.c -- CPU restatement of CatAna's spherical Fourier-Bessel (SFB)
 * decomposition hot path.
 *
 * THIS FILE IS TEST INFRASTRUCTURE (the oracle). Only the test-suite, the smoke
 * check and the CPU-baseline leg of bench.py load it, and only as the checker or
 * as the timed CPU reference. The product library (catana_gb300) never links,
 * imports or calls anything here.
 *
 * Parity pinning: the reference (CatAna) cannot be built in this environment
 * (GSL, FFTW3, Eigen, HEALPix C++ and CFITSIO are absent and its submodules are
 * empty).  This restatement follows the reference's algorithm step by step (file
 * and line cited at every function) and is pinned by
 *   - the reference's golden vectors test/test_data/gaussian_catalog.{python,
 *     pythonrev}.{c_ln,k_ln} (rtol 1e-2 on C_ln, allclose on k_ln, exactly the
 *     tolerance of test/python/decomposition_test.py:15-73);
 *   - the reference's known answers (Bessel zeros, interpolator accuracy, point
 *     conversion, HEALPix count maps);
 *   - a bit-for-bit comparison of the zero finder and the interpolation table
 *     against the reference's own SphericalBesselZeros.cpp / FunctionInterpolator.cpp
 *     / SBesselInterpolator.cpp compiled from the reference tree against a GSL
 *     shim whose j_l is the function below (oracle/Makefile, target `ref`);
 *   - scipy/mpmath for the special functions (spherical_jn, sph_legendre_p).
 * GSL's gsl_sf_bessel_jl and gsl_sf_legendre_sphPlm are replaced by published
 * algorithms (DLMF 10.51, 10.53, 10.74 for j_l; DLMF 14.10 for the normalised
 * associated Legendre recurrence) accurate to ~1e-15 relative.
 *
 * All entry points are plain C with an OpenMP parallel loop over points, in the
 * same loop order as the reference: per multipole l, every point evaluates
 * j_l(k_ln r) for all n, then P_lm for every m <= l from scratch (O(l-m) each,
 * like gsl_sf_legendre_sphPlm), then accumulates k*j*Y*.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define CO_PI 3.14159265358979323846264338327950288

/* ------------------------------------------------------------------------- */
/* Spherical Bessel function j_l(x), FP64.                                   */
/* Replaces gsl_sf_bessel_jl (called at sfb_raw.cpp:51,                      */
/* SphericalBesselZeros.cpp:54-55, SBesselInterpolator.cpp:16).              */
/* ------------------------------------------------------------------------- */

/* Ascending series, DLMF 10.53.1: j_l(x) = x^l/(2l+1)!! * sum_k (-x^2/2)^k /
 * (k! (2l+3)(2l+5)...(2l+2k+1)). */
static double co_jl_series(int l, double x)
{
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

/* Upward recurrence, DLMF 10.51.1, stable while l <= x. */
static double co_jl_upward(int l, double x)
{
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

/* Miller's backward recurrence (DLMF 3.6(vi), 10.74(iii)), normalised with the
 * closed forms of j_0 or j_1, whichever is larger in magnitude. */
static double co_jl_miller(int l, double x)
{
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
    /* jk = j_0 (unnormalised), jp1 = j_1 (unnormalised) */
    double s = sin(x), c = cos(x);
    double t0 = s / x;
    double t1 = (t0 - c) / x;
    if (fabs(t0) >= fabs(t1))
        return jl * (t0 / jk);
    return jl * (t1 / jp1);
}

double co_sbessel_jl(int l, double x)
{
    if (x == 0.0) return l == 0 ? 1.0 : 0.0;
    if (x < 0.0) { /* j_l(-x) = (-1)^l j_l(x) */
        double v = co_sbessel_jl(l, -x);
        return (l & 1) ? -v : v;
    }
    if (x * x < 2.0 * l + 3.0) return co_jl_series(l, x);
    if (x >= (double)l) return co_jl_upward(l, x);
    return co_jl_miller(l, x);
}

/* ------------------------------------------------------------------------- */
/* Normalised associated Legendre function with Condon-Shortley phase,       */
/* sqrt((2l+1)/(4pi) (l-m)!/(l+m)!) P_l^m(x): the quantity                   */
/* gsl_sf_legendre_sphPlm returns (sfb_raw.cpp:73, sfb_reverse_fft.cpp:119). */
/* Recurrence in l at fixed m, DLMF 14.10.3 in normalised form.              */
/* ------------------------------------------------------------------------- */
double co_sph_plm(int l, int m, double x)
{
    double somx2 = sqrt((1.0 - x) * (1.0 + x));
    double pmm = 1.0 / sqrt(4.0 * CO_PI);
    for (int i = 1; i <= m; ++i)
        pmm *= -sqrt((2.0 * i + 1.0) / (2.0 * i)) * somx2;
    if (l == m) return pmm;
    double p1 = x * sqrt(2.0 * m + 3.0) * pmm;
    if (l == m + 1) return p1;
    double p2 = pmm;
    double mm = (double)m * (double)m;
    for (int ll = m + 2; ll <= l; ++ll) {
        double dl = (double)ll, dl1 = (double)(ll - 1);
        double a = sqrt((4.0 * dl * dl - 1.0) / (dl * dl - mm));
        double b = sqrt((dl1 * dl1 - mm) / (4.0 * dl1 * dl1 - 1.0));
        double p = a * (x * p1 - b * p2);
        p2 = p1;
        p1 = p;
    }
    return p1;
}

/* ------------------------------------------------------------------------- */
/* Zeros of j_l: SphericalBesselZeros.cpp:11-68.                             */
/* First two zeros from the asymptotic guesses (:17-47), Newton with the     */
/* reference's stopping rule `while (delta/z > 1e-15)` (:49-62), which ends  */
/* the loop after any negative step; further zeros start from the linear     */
/* extrapolation 2 z_{n-1} - z_{n-2} (:64-68).                               */
/* ------------------------------------------------------------------------- */
static double co_newton(unsigned int l, double z)
{
    double delta, jl;
    do {
        jl = co_sbessel_jl((int)l, z);
        delta = jl / ((double)l / z * jl - co_sbessel_jl((int)l + 1, z));
        z -= delta;
    } while (delta / z > 1e-15);
    return z;
}

/* out[0..count) = zeros 0..count-1 of j_l, in the reference's order. */
void co_sbessel_zeros(unsigned int l, int count, double *out)
{
    double z0, z1;
    if (l == 0) {
        z0 = 3.141592653589793238463;
        z1 = 6.283185307179586476925;
    } else {
        double lh = l + 0.5;
        z0 = l + 0.5 + 1.8557571 * pow(lh, 1. / 3.) + 1.033150 * pow(lh, -1. / 3.) - 0.00397 * pow(lh, -1.) -
             0.0908 * pow(lh, -5. / 3.) + 0.043 * pow(lh, -7. / 3.);
        z1 = l + 0.5 + 3.2446076 * pow(lh, 1. / 3.) + 3.158244 * pow(lh, -1. / 3.) - 0.08331 * pow(lh, -1.) -
             0.8437 * pow(lh, -5. / 3.) + 0.864 * pow(lh, -7. / 3.);
    }
    double zs[2];
    zs[0] = co_newton(l, z0);
    zs[1] = co_newton(l, z1);
    for (int n = 0; n < count && n < 2; ++n) out[n] = zs[n];
    double a = zs[0], b = zs[1];
    for (int n = 2; n < count; ++n) {
        double z = co_newton(l, 2 * b - a);
        out[n] = z;
        a = b;
        b = z;
    }
}

/* k_ln table: return_types.cpp:10-20, k_ln(l,n) = SBZ(l)[n] / rmax.
 * Output row-major [l][n] (lmax x nmax). */
void co_compute_kln(int lmax, int nmax, double rmax, double *k_ln)
{
    double *z = (double *)malloc(sizeof(double) * (nmax > 2 ? nmax : 2));
    for (int l = 0; l < lmax; ++l) {
        co_sbessel_zeros((unsigned)l, nmax, z);
        for (int n = 0; n < nmax; ++n) k_ln[(size_t)l * nmax + n] = z[n] / rmax;
    }
    free(z);
}

/* ------------------------------------------------------------------------- */
/* Linear interpolation table of j_l: SBesselInterpolator.cpp:10-26 and      */
/* FunctionInterpolator.cpp:6-19. npts nodes x_i = 0 + i*dx on [0, zmax],     */
/* dx = zmax/(npts-1), dx_inv = 1/dx, y_i = j_l(x_i).                         */
/* ------------------------------------------------------------------------- */
void co_lerp_table(int l, double zmax, int npts, double *y, double *dx_inv_out)
{
    double dx = (zmax - 0.0) / (npts - 1);
    *dx_inv_out = 1. / dx;
    /* the reference fills its table in an OpenMP loop (FunctionInterpolator.cpp:15) */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < npts; ++i) y[i] = co_sbessel_jl(l, 0.0 + (size_t)i * dx);
}

/* Evaluation: SBesselInterpolator.cpp:20-26.  Returns 0 and sets *err=1 when
 * z >= zmax (the reference throws std::domain_error there). */
static inline double co_lerp_eval(const double *y, int npts, double dx_inv, double zmax, double z, int *err)
{
    if (z >= zmax) {
        *err = 1;
        return 0.0;
    }
    double i_approx = z * dx_inv;
    int i = (int)i_approx;
    if (i > npts - 2) i = npts - 2; /* the reference would read y[npts] here */
    return y[i] + (y[i + 1] - y[i]) * (i_approx - i);
}

double co_lerp_eval_pub(const double *y, int npts, double dx_inv, double zmax, double z, int *err)
{
    return co_lerp_eval(y, npts, dx_inv, zmax, z, err);
}

/* ------------------------------------------------------------------------- */
/* Raw SFB decomposition: sfb_raw.cpp:13-108 (+ the interpolation rule of    */
/* sfb_decomposition.cpp:15-19 is chosen by the caller).                      */
/*                                                                           */
/* pts: N x 3 row-major (r, theta, phi) -- the PointContainer buffer layout   */
/* (py_basictypes.cpp:126-135).  w: optional per-point weights (extension;    */
/* with weights the normalisation uses V/sum(w) instead of V/N).              */
/* Outputs: k_ln, c_ln row-major [l][n]; f_re/f_im (optional) packed by l,    */
/* each l block (l+1) x nmax row-major [m][n].                                */
/* Returns 0, or 2 when an argument left the interpolation range (the         */
/* reference throws std::domain_error).                                       */
/* ------------------------------------------------------------------------- */
int co_sfb_raw(const double *pts, const double *w, int64_t npoints, int lmax, int nmax, double rmax,
               int interpolated, int nthreads, double *k_ln, double *c_ln, double *f_re, double *f_im)
{
    if (nthreads <= 0) {
#ifdef _OPENMP
        nthreads = omp_get_max_threads();
#else
        nthreads = 1;
#endif
    }
    double wsum = (double)npoints;
    if (w) {
        wsum = 0.0;
        for (int64_t i = 0; i < npoints; ++i) wsum += w[i];
    }
    /* sfb_raw.cpp:29-30 */
    double norm_factor = sqrt(2. / CO_PI) * (4. / 3.) * CO_PI;
    norm_factor *= rmax * rmax * rmax / wsum;

    co_compute_kln(lmax, nmax, rmax, k_ln);
    memset(c_ln, 0, sizeof(double) * (size_t)lmax * nmax);

    int npts_tab = 1000 * nmax; /* BESSELINTERPOLATIONPOINTS_PER_ZERO * nmax */
    double *table = interpolated ? (double *)malloc(sizeof(double) * npts_tab) : NULL;
    double *zl = (double *)malloc(sizeof(double) * (nmax + 1 > 2 ? nmax + 1 : 2));
    int err_any = 0;

    size_t fsize_max = (size_t)lmax * nmax;
    double *acc = (double *)calloc((size_t)nthreads * 2 * fsize_max, sizeof(double));
    double *fl = (double *)malloc(sizeof(double) * 2 * fsize_max);
    size_t foff = 0;

    for (int l = 0; l < lmax; ++l) {
        double dx_inv = 0.0, zmax = 0.0;
        if (interpolated) {
            /* SBesselInterpolator_uptozero(l, nmax, 1000*nmax): zmax = SBZ(l)[nmax] */
            co_sbessel_zeros((unsigned)l, nmax + 1, zl);
            zmax = zl[nmax];
            co_lerp_table(l, zmax, npts_tab, table, &dx_inv);
        }
        size_t fs = (size_t)(l + 1) * nmax;
        memset(acc, 0, sizeof(double) * (size_t)nthreads * 2 * fs);
#pragma omp parallel num_threads(nthreads) reduction(| : err_any)
        {
            int tid = 0;
#ifdef _OPENMP
            tid = omp_get_thread_num();
#endif
            double *are = acc + (size_t)tid * 2 * fs;
            double *aim = are + fs;
            double *jn = (double *)malloc(sizeof(double) * nmax);
            int err = 0;
            /* contiguous static chunks: thread-private sums combined in thread order */
#pragma omp for schedule(static)
            for (int64_t i = 0; i < npoints; ++i) {
                double r = pts[3 * i + 0], theta = pts[3 * i + 1], phi = pts[3 * i + 2];
                double wi = w ? w[i] : 1.0;
                for (int n = 0; n < nmax; ++n) {
                    double z = k_ln[(size_t)l * nmax + n] * r;
                    jn[n] = interpolated ? co_lerp_eval(table, npts_tab, dx_inv, zmax, z, &err)
                                         : co_sbessel_jl(l, z);
                }
                double ct = cos(theta);
                for (int m = 0; m <= l; ++m) {
                    double plm = co_sph_plm(l, m, ct);
                    double yre = plm * cos(-m * phi);
                    double yim = plm * sin(-m * phi);
                    for (int n = 0; n < nmax; ++n) {
                        double kj = k_ln[(size_t)l * nmax + n] * jn[n] * wi;
                        are[(size_t)m * nmax + n] += kj * yre;
                        aim[(size_t)m * nmax + n] += kj * yim;
                    }
                }
            }
            free(jn);
            err_any |= err;
        }
        /* reduction over threads (the reference's omp critical, sfb_raw.cpp:81-84) */
        for (size_t q = 0; q < fs; ++q) {
            double sre = 0.0, sim = 0.0;
            for (int t = 0; t < nthreads; ++t) {
                sre += acc[(size_t)t * 2 * fs + q];
                sim += acc[(size_t)t * 2 * fs + fs + q];
            }
            fl[q] = sre * norm_factor;
            fl[fs + q] = sim * norm_factor;
        }
        /* C_ln: sfb_raw.cpp:91-96 */
        for (int n = 0; n < nmax; ++n) {
            double c = 0.0;
            for (int m = -l; m <= l; ++m) {
                int am = m < 0 ? -m : m;
                double re = fl[(size_t)am * nmax + n], im = fl[fs + (size_t)am * nmax + n];
                c += re * re + im * im;
            }
            c_ln[(size_t)l * nmax + n] = c / (2 * l + 1);
        }
        if (f_re && f_im) {
            memcpy(f_re + foff, fl, sizeof(double) * fs);
            memcpy(f_im + foff, fl + fs, sizeof(double) * fs);
        }
        foff += fs;
    }
    free(acc);
    free(fl);
    free(zl);
    free(table);
    return err_any ? 2 : 0;
}

/* ------------------------------------------------------------------------- */
/* HEALPix RING scheme (nside a power of two), restated from Gorski et al.    */
/* 2005, ApJ 622:759, section 4 and the HEALPix primer.  The reference calls  */
/* Healpix_Base::ang2pix / pix2ang / get_ring_info_small                      */
/* (PixelizedPointContainer.cpp:16-30, sfb_reverse_fft.cpp:78).  The branch   */
/* structure and operation order (sin(theta) near the poles, the za < 0.99    */
/* polar test, kshift and (t1 >> 1) & (nl4 - 1)) follow HEALPix C++'s         */
/* Healpix_Base::loc2pix / pix2loc (Healpix_cxx/healpix_base.cc, GPL-2), which */
/* bit-exact pixels need; the paper does not give them.                       */
/* ------------------------------------------------------------------------- */
static double co_fmodulo(double v1, double v2)
{
    if (v1 >= 0) return (v1 < v2) ? v1 : fmod(v1, v2);
    double tmp = fmod(v1, v2) + v2;
    return (tmp == v2) ? 0. : tmp;
}

static int64_t co_isqrt(int64_t v)
{
    int64_t r = (int64_t)sqrt((double)v + 0.5);
    while (r * r > v) --r;
    while ((r + 1) * (r + 1) <= v) ++r;
    return r;
}

/* theta in [0, pi]; returns -1 for theta outside that range (HEALPix asserts). */
int64_t co_ang2pix_ring(int64_t nside, double theta, double phi)
{
    if (!(theta >= 0.0 && theta <= CO_PI)) return -1;
    int64_t npix = 12 * nside * nside, ncap = 2 * nside * (nside - 1);
    int have_sth = (theta < 0.01) || (theta > 3.14159 - 0.01);
    double z = cos(theta), sth = have_sth ? sin(theta) : 0.0;
    double za = fabs(z);
    double tt = co_fmodulo(phi * 0.63661977236758134308, 4.0); /* phi / (pi/2) in [0,4) */
    if (za <= 2. / 3.) {
        int64_t nl4 = 4 * nside;
        double temp1 = nside * (0.5 + tt);
        double temp2 = nside * z * 0.75;
        int64_t jp = (int64_t)(temp1 - temp2);
        int64_t jm = (int64_t)(temp1 + temp2);
        int64_t ir = nside + 1 + jp - jm;
        int64_t kshift = 1 - (ir & 1);
        int64_t t1 = jp + jm - nside + kshift + 1 + nl4 + nl4;
        int64_t ip = (t1 >> 1) & (nl4 - 1);
        return ncap + (ir - 1) * nl4 + ip;
    } else {
        double tp = tt - (int64_t)tt;
        double tmp = ((za < 0.99) || !have_sth) ? nside * sqrt(3 * (1 - za)) : nside * sth / sqrt((1. + za) / 3.);
        int64_t jp = (int64_t)(tp * tmp);
        int64_t jm = (int64_t)((1.0 - tp) * tmp);
        int64_t ir = jp + jm + 1;
        int64_t ip = (int64_t)(tt * ir);
        if (ip >= 4 * ir) ip -= 4 * ir;
        return (z > 0) ? 2 * ir * (ir - 1) + ip : npix - 2 * ir * (ir + 1) + ip;
    }
}

void co_pix2ang_ring(int64_t nside, int64_t pix, double *theta, double *phi)
{
    int64_t npix = 12 * nside * nside, ncap = 2 * nside * (nside - 1);
    double fact2 = 4. / npix, fact1 = (nside << 1) * fact2;
    double z, ph, sth = 0.0;
    int have_sth = 0;
    if (pix < ncap) {
        int64_t iring = (1 + co_isqrt(1 + 2 * pix)) >> 1;
        int64_t iphi = (pix + 1) - 2 * iring * (iring - 1);
        double tmp = (iring * iring) * fact2;
        z = 1.0 - tmp;
        if (z > 0.99) {
            sth = sqrt(tmp * (2.0 - tmp));
            have_sth = 1;
        }
        ph = (iphi - 0.5) * (0.5 * CO_PI) / iring;
    } else if (pix < (npix - ncap)) {
        int64_t nl4 = 4 * nside, ip = pix - ncap;
        int64_t tmp = ip / nl4;
        int64_t iring = tmp + nside, iphi = ip - nl4 * tmp + 1;
        double fodd = ((iring + nside) & 1) ? 1 : 0.5;
        z = (2 * nside - iring) * fact1;
        ph = (iphi - fodd) * CO_PI * 0.75 * fact1;
    } else {
        int64_t ip = npix - pix;
        int64_t iring = (1 + co_isqrt(2 * ip - 1)) >> 1;
        int64_t iphi = 4 * iring + 1 - (ip - 2 * iring * (iring - 1));
        double tmp = (iring * iring) * fact2;
        z = tmp - 1.0;
        if (z < -0.99) {
            sth = sqrt(tmp * (2.0 - tmp));
            have_sth = 1;
        }
        ph = (iphi - 0.5) * (0.5 * CO_PI) / iring;
    }
    *theta = have_sth ? atan2(sth, z) : acos(z);
    *phi = ph;
}

/* ring in [1, 4 nside - 1] */
void co_ring_info(int64_t nside, int64_t ring, int64_t *startpix, int64_t *ringpix)
{
    int64_t npix = 12 * nside * nside, ncap = 2 * nside * (nside - 1);
    if (ring < nside) {
        *ringpix = 4 * ring;
        *startpix = 2 * ring * (ring - 1);
    } else if (ring < 3 * nside) {
        *ringpix = 4 * nside;
        *startpix = ncap + (ring - nside) * 4 * nside;
    } else {
        int64_t nr = 4 * nside - ring;
        *ringpix = 4 * nr;
        *startpix = npix - 2 * nr * (nr + 1);
    }
}

/* Bin points into RING pixels (PixelizedPointContainer.cpp:11-30): the output
 * is CSR -- offsets[npix+1] and r values in point order within each pixel.
 * Returns -1 on a theta outside [0, pi]. */
int co_bin_points(int64_t nside, const double *pts, int64_t npoints, int64_t *offsets, double *r_sorted)
{
    int64_t npix = 12 * nside * nside;
    int64_t *pix = (int64_t *)malloc(sizeof(int64_t) * (npoints > 0 ? npoints : 1));
    for (int64_t p = 0; p <= npix; ++p) offsets[p] = 0;
    for (int64_t i = 0; i < npoints; ++i) {
        pix[i] = co_ang2pix_ring(nside, pts[3 * i + 1], pts[3 * i + 2]);
        if (pix[i] < 0) {
            free(pix);
            return -1;
        }
        offsets[pix[i] + 1]++;
    }
    for (int64_t p = 0; p < npix; ++p) offsets[p + 1] += offsets[p];
    int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * npix);
    memcpy(fill, offsets, sizeof(int64_t) * npix);
    for (int64_t i = 0; i < npoints; ++i) r_sorted[fill[pix[i]]++] = pts[3 * i];
    free(fill);
    free(pix);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* HEALPix SFB: sfb_reverse_fft.cpp:43-209.  Per (l, n): per ring, the map of  */
/* summed j_l(k r) per pixel, its real DFT (FFTW r2c convention, F[s] =       */
/* sum_j map_j exp(-2 pi i j s / rpix), s <= rpix/2), then the m-extraction   */
/* with the reference's index mapping m_ = rpix/2 - |rpix/2 - (m % rpix)| and */
/* sign = (m > 0): the imaginary part is never negated, so m > rpix/2 takes   */
/* F[rpix - m%rpix] instead of its conjugate (sfb_reverse_fft.cpp:192-207).  */
/* The DFT is evaluated directly for the frequencies the extraction reads.    */
/* ------------------------------------------------------------------------- */
/* One multipole's pixel maps for the FFT form of the HEALPix SFB (oracle.sfb_healpix_fft):
 * map[pix * nmax + n] = sum over the pixel's points, in order, of j_l(k_ln r) -- the same
 * sums as the map loop of co_sfb_healpix (sfb_reverse_fft.cpp:91-113), with the same j_l
 * rule (the lerp table of SBesselInterpolator.cpp:10-26 or the direct j_l).  Returns 2 when
 * an argument lies outside the table. */
int co_healpix_maps(int64_t npix, const int64_t *offsets, const double *r_sorted, int l, int nmax,
                    const double *k_row, double rmax, int interpolated, int nthreads, double *map)
{
    (void)rmax;
    if (nthreads <= 0) {
#ifdef _OPENMP
        nthreads = omp_get_max_threads();
#else
        nthreads = 1;
#endif
    }
    int npts_tab = 1000 * nmax;
    double *table = NULL, dx_inv = 0.0, zmax = 0.0;
    if (interpolated) {
        double *zl = (double *)malloc(sizeof(double) * (nmax + 1 > 2 ? nmax + 1 : 2));
        co_sbessel_zeros((unsigned)l, nmax + 1, zl);
        zmax = zl[nmax];
        free(zl);
        table = (double *)malloc(sizeof(double) * npts_tab);
        co_lerp_table(l, zmax, npts_tab, table, &dx_inv);
    }
    int err_any = 0;
#pragma omp parallel for num_threads(nthreads) schedule(static) reduction(| : err_any)
    for (int64_t p = 0; p < npix; ++p) {
        int err = 0;
        for (int n = 0; n < nmax; ++n) {
            const double k_n = k_row[n];
            double s = 0.0;
            for (int64_t q = offsets[p]; q < offsets[p + 1]; ++q) {
                const double z = k_n * r_sorted[q];
                s += interpolated ? co_lerp_eval(table, npts_tab, dx_inv, zmax, z, &err) : co_sbessel_jl(l, z);
            }
            map[p * nmax + n] = s;
        }
        err_any |= err;
    }
    free(table);
    return err_any ? 2 : 0;
}

int co_sfb_healpix(int64_t nside, const int64_t *offsets, const double *r_sorted, int lmax, int nmax, double rmax,
                   int interpolated, int nthreads, double *k_ln, double *c_ln, double *f_re, double *f_im)
{
    if (nthreads <= 0) {
#ifdef _OPENMP
        nthreads = omp_get_max_threads();
#else
        nthreads = 1;
#endif
    }
    int64_t npix = 12 * nside * nside;
    int64_t nrings = 4 * nside - 1;
    int64_t npoints = offsets[npix];
    double norm_factor = sqrt(2. / CO_PI) * (4. / 3.) * CO_PI;
    norm_factor *= rmax * rmax * rmax / (double)npoints;
    co_compute_kln(lmax, nmax, rmax, k_ln);
    memset(c_ln, 0, sizeof(double) * (size_t)lmax * nmax);

    int64_t *rstart = (int64_t *)malloc(sizeof(int64_t) * nrings);
    int64_t *rpixv = (int64_t *)malloc(sizeof(int64_t) * nrings);
    double *costh = (double *)malloc(sizeof(double) * nrings);
    double *phase = (double *)malloc(sizeof(double) * nrings);
    for (int64_t i = 0; i < nrings; ++i) {
        co_ring_info(nside, i + 1, &rstart[i], &rpixv[i]);
        double th, ph;
        co_pix2ang_ring(nside, rstart[i], &th, &ph);
        costh[i] = cos(th);
        phase[i] = ph;
    }
    int npts_tab = 1000 * nmax;
    double *table = interpolated ? (double *)malloc(sizeof(double) * npts_tab) : NULL;
    double *zl = (double *)malloc(sizeof(double) * (nmax + 1 > 2 ? nmax + 1 : 2));
    double *ylm = (double *)malloc(sizeof(double) * 2 * (size_t)nrings * lmax);
    double *acc = (double *)malloc(sizeof(double) * 2 * (size_t)nthreads * lmax);
    int err_any = 0;
    size_t foff = 0;

    for (int l = 0; l < lmax; ++l) {
        double dx_inv = 0.0, zmax = 0.0;
        if (interpolated) {
            co_sbessel_zeros((unsigned)l, nmax + 1, zl);
            zmax = zl[nmax];
            co_lerp_table(l, zmax, npts_tab, table, &dx_inv);
        }
        for (int64_t i = 0; i < nrings; ++i)
            for (int m = 0; m <= l; ++m) {
                double p = co_sph_plm(l, m, costh[i]);
                ylm[2 * (i * (l + 1) + m)] = p * cos(-m * phase[i]);
                ylm[2 * (i * (l + 1) + m) + 1] = p * sin(-m * phase[i]);
            }
        size_t fs = (size_t)(l + 1) * nmax;
        for (int n = 0; n < nmax; ++n) {
            double k_n = k_ln[(size_t)l * nmax + n];
            memset(acc, 0, sizeof(double) * 2 * (size_t)nthreads * (l + 1));
#pragma omp parallel num_threads(nthreads) reduction(| : err_any)
            {
                int tid = 0;
#ifdef _OPENMP
                tid = omp_get_thread_num();
#endif
                double *a = acc + (size_t)tid * 2 * (l + 1);
                int err = 0;
                double *map = (double *)malloc(sizeof(double) * 4 * nside);
#pragma omp for schedule(static)
                for (int64_t i = 0; i < nrings; ++i) {
                    int64_t rp = rpixv[i];
                    for (int64_t j = 0; j < rp; ++j) {
                        double s = 0.0;
                        int64_t p = rstart[i] + j;
                        for (int64_t q = offsets[p]; q < offsets[p + 1]; ++q) {
                            double z = k_n * r_sorted[q];
                            s += interpolated ? co_lerp_eval(table, npts_tab, dx_inv, zmax, z, &err)
                                              : co_sbessel_jl(l, z);
                        }
                        map[j] = s;
                    }
                    for (int m = 0; m <= l; ++m) {
                        int64_t mi = rp / 2 - (m % rp);
                        int sign = (m > 0) - (m < 0);
                        mi = rp / 2 - (mi < 0 ? -mi : mi);
                        /* F[mi] by direct DFT */
                        double fre = 0.0, fim = 0.0;
                        for (int64_t j = 0; j < rp; ++j) {
                            double ang = -2.0 * CO_PI * (double)((j * mi) % rp) / (double)rp;
                            fre += map[j] * cos(ang);
                            fim += map[j] * sin(ang);
                        }
                        fim *= sign;
                        double yre = ylm[2 * (i * (l + 1) + m)], yim = ylm[2 * (i * (l + 1) + m) + 1];
                        a[2 * m] += fre * yre - fim * yim;
                        a[2 * m + 1] += fre * yim + fim * yre;
                    }
                }
                free(map);
                err_any |= err;
            }
            double sq = 0.0, f0 = 0.0;
            for (int m = 0; m <= l; ++m) {
                double sre = 0.0, sim = 0.0;
                for (int t = 0; t < nthreads; ++t) {
                    sre += acc[(size_t)t * 2 * (l + 1) + 2 * m];
                    sim += acc[(size_t)t * 2 * (l + 1) + 2 * m + 1];
                }
                double a2 = sre * sre + sim * sim;
                sq += a2;
                if (m == 0) f0 = a2;
                if (f_re && f_im) {
                    f_re[foff + (size_t)m * nmax + n] = sre * k_n * norm_factor;
                    f_im[foff + (size_t)m * nmax + n] = sim * k_n * norm_factor;
                }
            }
            double c = 2 * sq - f0;
            double nk = norm_factor * k_n;
            c *= nk * nk / (2 * l + 1);
            c_ln[(size_t)l * nmax + n] = c;
        }
        foff += fs;
    }
    free(rstart);
    free(rpixv);
    free(costh);
    free(phase);
    free(table);
    free(zl);
    free(ylm);
    free(acc);
    return err_any ? 2 : 0;
}

/* _sfb_reverse (sfb_reverse.cpp:13-112): per l, Y(m, pix) = sphPlm(l, m, cos theta_pix)
 * e^{-i m phi_pix} at every pixel centre (:63-70), map(pix, n) = sum over the pixel's
 * radii of j_l(k_ln r) (:73-81), f_l = Y map (:88), C_ln = sum_{m=-l..l} |f_l|m|n|^2
 * (norm k)^2 / (2l+1) (:91-96), stored f = f k norm (:98-102); norm = sqrt(2/pi) 4/3 pi
 * rmax^3 / N (:29-30).  Interpolation as the raw path (:44-51). */
int co_sfb_reverse(int64_t nside, const int64_t *offsets, const double *r_sorted, int lmax, int nmax, double rmax,
                   int interpolated, int nthreads, double *k_ln, double *c_ln, double *f_re, double *f_im)
{
    if (!f_re || !f_im) return 3; /* f is needed for C_ln; callers always pass it */
    if (nthreads <= 0) {
#ifdef _OPENMP
        nthreads = omp_get_max_threads();
#else
        nthreads = 1;
#endif
    }
    int64_t npix = 12 * nside * nside;
    int64_t npoints = offsets[npix];
    double norm_factor = sqrt(2. / CO_PI) * (4. / 3.) * CO_PI;
    norm_factor *= rmax * rmax * rmax / (double)npoints;
    co_compute_kln(lmax, nmax, rmax, k_ln);
    memset(c_ln, 0, sizeof(double) * (size_t)lmax * nmax);
    double *th = (double *)malloc(sizeof(double) * npix);
    double *ph = (double *)malloc(sizeof(double) * npix);
    for (int64_t p = 0; p < npix; ++p) co_pix2ang_ring(nside, p, &th[p], &ph[p]);
    int npts_tab = 1000 * nmax;
    double *table = interpolated ? (double *)malloc(sizeof(double) * npts_tab) : NULL;
    double *zl = (double *)malloc(sizeof(double) * (nmax + 1 > 2 ? nmax + 1 : 2));
    double *map = (double *)malloc(sizeof(double) * (size_t)npix * (nmax > 0 ? nmax : 1));
    int err_any = 0;
    size_t foff = 0;
    for (int l = 0; l < lmax; ++l) {
        double dx_inv = 0.0, zmax = 0.0;
        if (interpolated) {
            co_sbessel_zeros((unsigned)l, nmax + 1, zl);
            zmax = zl[nmax];
            co_lerp_table(l, zmax, npts_tab, table, &dx_inv);
        }
#pragma omp parallel for num_threads(nthreads) reduction(| : err_any) schedule(static)
        for (int64_t p = 0; p < npix; ++p) {
            int err = 0;
            for (int n = 0; n < nmax; ++n) {
                double k_n = k_ln[(size_t)l * nmax + n], s = 0.0;
                for (int64_t q = offsets[p]; q < offsets[p + 1]; ++q) {
                    double z = k_n * r_sorted[q];
                    s += interpolated ? co_lerp_eval(table, npts_tab, dx_inv, zmax, z, &err) : co_sbessel_jl(l, z);
                }
                map[(size_t)p * nmax + n] = s;
            }
            err_any |= err;
        }
        /* f(m, n) = sum_pix Y(m, pix) map(pix, n), pixels in order */
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1)
        for (int m = 0; m <= l; ++m) {
            double *fr = (double *)calloc((size_t)nmax, sizeof(double));
            double *fi = (double *)calloc((size_t)nmax, sizeof(double));
            for (int64_t p = 0; p < npix; ++p) {
                double pl = co_sph_plm(l, m, cos(th[p]));
                double yr = pl * cos(-m * ph[p]), yi = pl * sin(-m * ph[p]);
                for (int n = 0; n < nmax; ++n) {
                    double v = map[(size_t)p * nmax + n];
                    fr[n] += yr * v;
                    fi[n] += yi * v;
                }
            }
            for (int n = 0; n < nmax; ++n) {
                size_t o = foff + (size_t)m * nmax + n;
                f_re[o] = fr[n];
                f_im[o] = fi[n];
            }
            free(fr);
            free(fi);
        }
        for (int n = 0; n < nmax; ++n) {
            double kk = k_ln[(size_t)l * nmax + n], c = 0.0;
            for (int m = -l; m <= l; ++m) {
                size_t o = foff + (size_t)(m < 0 ? -m : m) * nmax + n;
                c += f_re[o] * f_re[o] + f_im[o] * f_im[o];
            }
            c_ln[(size_t)l * nmax + n] = c * pow(norm_factor * kk, 2) / (2 * l + 1);
            for (int m = 0; m <= l; ++m) {
                size_t o = foff + (size_t)m * nmax + n;
                f_re[o] *= kk * norm_factor;
                f_im[o] *= kk * norm_factor;
            }
        }
        foff += (size_t)(l + 1) * nmax;
    }
    free(th);
    free(ph);
    free(table);
    free(zl);
    free(map);
    return err_any ? 2 : 0;
}

/* Point(x, y, z): Point.cpp:5-10 -- r = |v|, theta = atan2(rho, z),
 * phi = atan2(y, x) reduced into [0, 2 pi) (HEALPix pointing(vec3) + normalize). */
void co_cartesian_to_spherical(const double *xyz, int64_t n, double *rtp)
{
    for (int64_t i = 0; i < n; ++i) {
        double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
        double rho = sqrt(x * x + y * y);
        double r = sqrt(x * x + y * y + z * z);
        double th = atan2(rho, z);
        double ph = (x == 0.0 && y == 0.0) ? 0.0 : atan2(y, x);
        if (ph < 0.0) ph += 2.0 * CO_PI;
        ph = co_fmodulo(ph, 2.0 * CO_PI);
        rtp[3 * i] = r;
        rtp[3 * i + 1] = th;
        rtp[3 * i + 2] = ph;
    }
}

/* Ingest: record conversion (Point.cpp:5-10 for Cartesian records, as given for
 * spherical ones, Point.cpp:23-28) and the point filters -- tophat r < R0
 * (radial_filters.cpp:32-34), Gaussian exp(-(r/R0)^2) > u (:26-28), an interpolated
 * generic window w(r) > u (:12-24 with FunctionInterpolator.cpp:6-30), a RING angular
 * mask map[ang2pix] == 1 (angular_filters.cpp:11-13) -- with u of record i the
 * SplitMix64 hash of (seed, index0 + i).  Kept points in input order.  Returns 0, or 2
 * when a radius leaves the window's range / a theta leaves [0, pi] under a mask. */
static double co_ingest_uniform(uint64_t seed, uint64_t index)
{
    uint64_t z = seed + (index + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * 0x1.0p-53;
}

int co_ingest(const void *records, int64_t n, unsigned layout, double tophat_r0, double gauss_r0,
              const double *window, int64_t window_n, double window_min, double window_max, const float *mask,
              int64_t mask_nside, uint64_t seed, uint64_t index0, double *out, int64_t *n_out)
{
    int64_t k = 0;
    int err = 0;
    double dx_inv = 0.0;
    if (window) dx_inv = 1.0 / ((window_max - window_min) / (double)(window_n - 1));
    for (int64_t i = 0; i < n; ++i) {
        double a, b, c, r, th, ph;
        if (layout & 1u) {
            const float *p = (const float *)records + 3 * i;
            a = p[0];
            b = p[1];
            c = p[2];
        } else {
            const double *p = (const double *)records + 3 * i;
            a = p[0];
            b = p[1];
            c = p[2];
        }
        if (layout & 2u) {
            double v[3] = {a, b, c}, o[3];
            co_cartesian_to_spherical(v, 1, o);
            r = o[0];
            th = o[1];
            ph = o[2];
        } else {
            r = a;
            th = b;
            ph = c;
        }
        int keep = 1;
        if (tophat_r0 > 0.0 && !(r < tophat_r0)) keep = 0;
        if (keep && (gauss_r0 > 0.0 || window)) {
            double u = co_ingest_uniform(seed, index0 + (uint64_t)i);
            if (gauss_r0 > 0.0) {
                double q = r / gauss_r0;
                if (!(exp(-(q * q)) > u)) keep = 0;
            }
            if (keep && window) {
                if (r < window_min || r >= window_max) {
                    err = 2;
                    keep = 0;
                } else {
                    double x = r - window_min, ia = x * dx_inv;
                    unsigned ii = (unsigned)ia;
                    if (ii > (unsigned)(window_n - 2)) ii = (unsigned)(window_n - 2); /* r just below the top */
                    double w = window[ii] + (window[ii + 1] - window[ii]) * (ia - ii);
                    if (!(w > u)) keep = 0;
                }
            }
        }
        if (keep && mask) {
            int64_t pix = co_ang2pix_ring(mask_nside, th, ph);
            if (pix < 0) {
                err = 2;
                keep = 0;
            } else if (!(mask[pix] == 1.0f)) {
                keep = 0;
            }
        }
        if (keep) {
            out[3 * k] = r;
            out[3 * k + 1] = th;
            out[3 * k + 2] = ph;
            ++k;
        }
    }
    *n_out = k;
    return err;
}

/* Double spherical-Bessel integral int_0^rmax w(r) j_l(k1 r) j_l(k2 r) dr
 * (sbessel_integrator.cpp:53-110): breakpoints at the zeros of both factors inside
 * (0, rmax) (the reference's nested range generators, :113-133, visit the same merged
 * set) and at the nodes of the w table (w linear on every piece), adaptive
 * Gauss-Legendre on each piece (16 vs 32 nodes, bisection until they
 * agree to 1e-14) instead of QAG, over the whole range; w is a FunctionInterpolator
 * table (FunctionInterpolator.cpp:6-30).  Returns 0, or 2 when w is evaluated outside
 * its range. */
static void co_gl_nodes(int n, double *x, double *w)
{
    for (int i = 0; i < (n + 1) / 2; ++i) {
        double z = cos(CO_PI * (i + 0.75) / (n + 0.5)), pp = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p1 = 1.0, p2 = 0.0;
            for (int j = 1; j <= n; ++j) {
                double p3 = p2;
                p2 = p1;
                p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
            }
            pp = n * (z * p1 - p2) / (z * z - 1.0);
            double dz = p1 / pp;
            z -= dz;
            if (fabs(dz) < 1e-16) break;
        }
        x[i] = -z;
        x[n - 1 - i] = z;
        w[i] = w[n - 1 - i] = 2.0 / ((1.0 - z * z) * pp * pp);
    }
}

typedef struct {
    const double *wt;
    int64_t wn;
    double wmin, wmax, dxinv, k1, k2;
    int l, err;
    double x16[16], w16[16], x32[32], w32[32];
} co_dsb_ctx;

static double co_dsb_f(co_dsb_ctx *c, double x)
{
    /* x == wmax only from rounding at the range's end (the rule's nodes are interior):
     * the interpolator's last segment gives y[n-1] there */
    if (x < c->wmin || x > c->wmax) {
        c->err = 2;
        return 0.0;
    }
    double ia = (x - c->wmin) * c->dxinv;
    unsigned ii = (unsigned)ia;
    if (ii > (unsigned)(c->wn - 2)) ii = (unsigned)(c->wn - 2);
    double w = c->wt[ii] + (c->wt[ii + 1] - c->wt[ii]) * (ia - ii);
    return w * co_sbessel_jl(c->l, c->k1 * x) * co_sbessel_jl(c->l, c->k2 * x);
}

static double co_dsb_piece(co_dsb_ctx *c, double a, double b, int depth)
{
    double h = 0.5 * (b - a), s16 = 0.0, s32 = 0.0, a32 = 0.0;
    for (int i = 0; i < 16; ++i) s16 += c->w16[i] * co_dsb_f(c, a + h * (c->x16[i] + 1.0));
    for (int i = 0; i < 32; ++i) {
        double f = co_dsb_f(c, a + h * (c->x32[i] + 1.0));
        s32 += c->w32[i] * f;
        a32 += c->w32[i] * fabs(f);
    }
    s16 *= h;
    s32 *= h;
    a32 *= h;
    /* agreement to 1e-13 of the piece's integral of |f| (pieces that cancel to ~0 are
     * judged on that scale, not on their own tiny sum) */
    if (depth >= 12 || fabs(s32 - s16) <= 1e-13 * a32 + 1e-300) return s32;
    double m = 0.5 * (a + b);
    return co_dsb_piece(c, a, m, depth + 1) + co_dsb_piece(c, m, b, depth + 1);
}

int co_dsb_integral(const double *w_table, int64_t w_n, double w_min, double w_max, int l, double rmax, double k1,
                    double k2, double *out)
{
    co_dsb_ctx c;
    c.wt = w_table;
    c.wn = w_n;
    c.wmin = w_min;
    c.wmax = w_max;
    c.dxinv = 1.0 / ((w_max - w_min) / (double)(w_n - 1));
    c.l = l;
    c.err = 0;
    if (k1 > k2) {
        double t = k1;
        k1 = k2;
        k2 = t;
    }
    c.k1 = k1;
    c.k2 = k2;
    co_gl_nodes(16, c.x16, c.w16);
    co_gl_nodes(32, c.x32, c.w32);
    int nz = 2;
    double *z = NULL;
    for (;;) {
        free(z);
        z = (double *)malloc(sizeof(double) * nz);
        co_sbessel_zeros((unsigned)l, nz, z);
        if (z[nz - 1] > k2 * rmax) break;
        nz *= 2;
    }
    double lo = 0.0, acc = 0.0, wdx = (w_max - w_min) / (double)(w_n - 1);
    int i1 = 0, i2 = 0;
    int64_t it = (int64_t)floor((0.0 - w_min) / wdx) + 1;
    if (it < 1) it = 1;
    if (w_min > 0.0 || rmax > w_max) c.err = 2;
    while (lo < rmax && !c.err) {
        /* breakpoints: table nodes (w linear between them) and the zeros of both factors */
        double zt = (it < w_n) ? w_min + (double)it * wdx : INFINITY;
        double z1 = (k1 > 0.0 && i1 < nz) ? z[i1] / k1 : INFINITY;
        double z2 = (k2 > 0.0 && i2 < nz) ? z[i2] / k2 : INFINITY;
        double hi = fmin(fmin(fmin(z1, z2), zt), rmax);
        if (hi > lo) acc += co_dsb_piece(&c, lo, hi, 0);
        if (zt <= hi) ++it;
        if (z1 <= hi) ++i1;
        if (z2 <= hi) ++i2;
        if (hi >= rmax || (!(zt <= hi) && !(z1 <= hi) && !(z2 <= hi))) break;
        lo = hi;
    }
    free(z);
    *out = acc;
    return c.err;
}
