/*
 * catana_gpu.h -- C ABI of the GB300 (sm_103a) SFB decomposition library
 * (libcatana_gpu.so).
 *
 * Plain pointers and sizes only; every entry point returns a catana_status_t and
 * never throws.  Host-buffer entry points block until their results are in the
 * caller's buffers; the *_dev entry points take device pointers and only enqueue
 * work on the given stream (NULL = the legacy default stream).  The library keeps
 * one context per device (workspace, cached Bessel-zero and coefficient tables);
 * calls on one device are serialised by a mutex.
 *
 * Reference interfaces replaced (CatAna, paths relative to its repository):
 *   catana::sfb_decomposition(const PointContainer&, ...)   sfb_decomposition.hpp:29-30,
 *                                                            sfb_decomposition.cpp:15-19
 *   catana::_sfb_raw(...)                                    sfb_raw.hpp:11-12, sfb_raw.cpp:13-108
 *   catana::sfb_decomposition(const PixelizedPointContainer&, ...)
 *                                                            sfb_decomposition.hpp:46-47,
 *                                                            sfb_decomposition.cpp:22-26
 *   catana::_sfb_reverse_fft(...)                            sfb_reverse_fft.hpp, sfb_reverse_fft.cpp:43-172
 *   PixelizedPointContainer(nside, const PointContainer&)    PixelizedPointContainer.cpp:11-30
 *   catana::compute_kln / KClkk::KClkk                        return_types.cpp:10-23
 *   besseltools::SphericalBesselZeros::operator[]             SphericalBesselZeros.cpp:11-100
 */
#ifndef CATANA_GPU_H
#define CATANA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A cudaStream_t.  NULL selects the legacy default stream. */
typedef struct CUstream_st *catana_gpu_stream_t;

typedef enum {
    CATANA_OK = 0,
    CATANA_ERR_ARG = 1,         /* invalid argument (reference: std::invalid_argument -> ValueError) */
    CATANA_ERR_DOMAIN = 2,      /* j_l argument at or beyond the interpolation table's end
                                   (reference: std::domain_error -> ValueError) */
    CATANA_ERR_CUDA = 3,        /* CUDA runtime error; see catana_gpu_last_error() */
    CATANA_ERR_NOMEM = 4,       /* device or pinned allocation failed */
    CATANA_ERR_UNSUPPORTED = 5  /* the requested form needs a device this build does not target */
} catana_status_t;

/* ---- flags for the SFB entry points ------------------------------------ */
/* j_l evaluation.  AUTO is the reference's rule (sfb_decomposition.cpp:17,24):
 * interpolate iff the catalog holds more than 1000 points. */
#define CATANA_JL_AUTO 0u
#define CATANA_JL_INTERP 1u  /* linear table, 1000*nmax nodes up to z_{l,nmax} (SBesselInterpolator.cpp:10-26) */
#define CATANA_JL_EXACT 2u   /* direct j_l evaluation (the reference's gsl_sf_bessel_jl branch) */
/* Plain raw path only, no counterpart in the reference: j_l from piecewise FP64
 * polynomials (degree 11 in Chebyshev form, one per unit interval of z = k r centred
 * on an integer), within ~1e-14 of the envelope of j_l -- the accuracy of the
 * exact branch at the cost of the table branch.  It serves as the FP64 reference the
 * split form is measured against at full catalog sizes.  The healpix and
 * allocation-free entry points reject it (CATANA_ERR_ARG); negative or non-finite
 * radii are CATANA_ERR_DOMAIN. */
#define CATANA_JL_POLY 3u
#define CATANA_JL_MASK 3u
/* Contraction form.  PLAIN: FP64 on CUDA cores, the drop-in.  SPLIT: tensor-core
 * tcgen05 contraction of 3-term FP16 hi+lo products with FP32 accumulation,
 * folded per 32-point tile and reduced in FP64; j_l from piecewise degree-6
 * polynomials on unit intervals with FP32 coefficients, accurate to ~1e-7 of its
 * envelope (the JL flags do not apply); lmax <= 512, nmax <= 256 (above lmax 256
 * the Legendre rows carry a 2-bit exponent per value). */
#define CATANA_FORM_PLAIN 0u
#define CATANA_FORM_SPLIT 4u
#define CATANA_FORM_MASK 4u
/* Split form (no counterpart in the reference): the Legendre rows follow the
 * Reinsch-modified recurrence at |cos(theta)| for m < 128 (above lmax 256 always, with
 * or without this flag) -- rows P_l and
 * D_l = P_l - rho_l P_{l-1}, rho_l the ratio of consecutive P_lm / sin^m(theta) at the
 * pole -- so FP32 rounding no longer accumulates through the three-term recurrence's
 * cancellation near the poles.  About half the f_lmn error at high l of the default
 * split form, and up to ten times less for points near a pole, at ~12% lower
 * throughput at lmax 256 (one more row written per value).  Ignored by the plain form. */
#define CATANA_SPLIT_ACCURATE 32u
/* HEALPix path: 0 reproduces the reference's m-extraction, which reads
 * F[rpix - m%rpix] without conjugation when m%rpix > rpix/2
 * (sfb_reverse_fft.cpp:192-207); this flag conjugates it (the correct alias). */
#define CATANA_HEALPIX_CONJ_FIX 8u

/* ---- output layout -------------------------------------------------------
 * k_ln, c_ln: lmax x nmax, row-major (index l*nmax + n) -- the numpy view of the
 *             reference's KClkk.k_ln / c_ln (Eigen arrays exported to numpy).
 * f_lmn:      complex128 as interleaved (re, im) doubles, packed by l: the block of
 *             multipole l starts at complex index nmax*l*(l+1)/2 and holds the
 *             (l+1) x nmax row-major array f[l][m][n], m = 0..l (KClkk.f_lmn[l]).
 *             Total complex entries: catana_gpu_flmn_size(lmax, nmax).
 */
size_t catana_gpu_flmn_size(uint16_t lmax, uint16_t nmax);

/* Raw (direct-sum) SFB decomposition of a point catalog.
 *   f_lmn = sqrt(2/pi) * V/W * sum_i w_i k_ln j_l(k_ln r_i) Y*_lm(theta_i, phi_i),
 *   V = 4/3 pi rmax^3, W = sum_i w_i (= N without weights),
 *   C_ln  = sum_{m=-l..l} |f_l|m|n|^2 / (2l+1).
 * points: npoints x 3 row-major (r, theta, phi), host memory (the PointContainer
 *         buffer, py_basictypes.cpp:126-135).
 * weights: optional per-point weights (NULL = unit weights; an extension -- the
 *         reference's Point carries none).
 * k_ln, c_ln: host, lmax*nmax doubles.  f_lmn: host or NULL.
 * Replaces sfb_decomposition(const PointContainer&, lmax, nmax, rmax, store_flmn,
 * verbose) and _sfb_raw (sfb_raw.cpp:13-108). */
catana_status_t catana_gpu_sfb_raw(const double *points, const double *weights, int64_t npoints, uint16_t lmax,
                                   uint16_t nmax, double rmax, uint32_t flags, double *k_ln, double *c_ln,
                                   double *f_lmn, catana_gpu_stream_t stream);

/* Same computation on device-resident data: all pointers are device pointers,
 * the work is enqueued on `stream` and the call returns without synchronising
 * except where a domain check needs the host (JL_INTERP); *status_dev (device
 * int, may be NULL) receives CATANA_ERR_DOMAIN when an argument left the table. */
catana_status_t catana_gpu_sfb_raw_dev(const double *points_dev, const double *weights_dev, int64_t npoints,
                                       uint16_t lmax, uint16_t nmax, double rmax, uint32_t flags,
                                       double *k_ln_dev, double *c_ln_dev, double *f_lmn_dev,
                                       int *status_dev, catana_gpu_stream_t stream);

/* Allocation-free variant of catana_gpu_sfb_raw_dev (no counterpart in the
 * reference).  For callers that may not allocate device memory -- code that runs
 * under a caller-owned memory pool or a fixed memory budget, or that must not
 * trigger cudaMalloc's implicit device synchronisation -- it runs the plain FP64
 * raw path with every scratch buffer carved out of one static device array of
 * 32 MiB per device (held until the process exits) and calls no cudaMalloc,
 * cudaFree or allocating library routine.  The caller passes device inputs and
 * device outputs; k_ln_dev, c_ln_dev and f_lmn_dev are required (f_lmn_dev is also
 * the accumulator).  Plain form only (CATANA_FORM_SPLIT is rejected).  Sizes whose
 * interpolation tables and partial sums do not fit the array (lmax * nmax above
 * about 2000 with interpolated j_l -- lmax = nmax = 32 fits, 64 x 64 does not)
 * return CATANA_ERR_ARG with the reason.  The call
 * blocks until its results are ready.  The first call on a device resolves the
 * array's address (cudaGetSymbolAddress): make it before any stream capture.  All
 * calls share the array, so calls that overlap on the GPU race. */
catana_status_t catana_gpu_sfb_raw_noalloc(const double *points_dev, const double *weights_dev, int64_t npoints,
                                           uint16_t lmax, uint16_t nmax, double rmax, uint32_t flags,
                                           double *k_ln_dev, double *c_ln_dev, double *f_lmn_dev,
                                           catana_gpu_stream_t stream);

/* ---- batched raw decomposition (no counterpart in the reference) ---------
 * Many catalogs, each with its own size, lmax, nmax, rmax and an optional kmax cut,
 * decomposed in one call.  Each catalog's outputs are those of catana_gpu_sfb_raw
 * on that catalog alone, except that with kmax > 0 the modes with k_ln > kmax are
 * not computed: their f_lmn and c_ln are 0 (k_ln is still filled in full). */
typedef struct {
    const double *points;   /* npoints x 3 (r, theta, phi) */
    const double *weights;  /* optional per-point weights (NULL = unit) */
    int64_t npoints;
    double rmax;
    double kmax;            /* > 0: keep only modes with k_ln <= kmax */
    double *k_ln;           /* lmax x nmax, row-major [l][n] */
    double *c_ln;           /* lmax x nmax */
    double *f_lmn;          /* packed as for catana_gpu_sfb_raw, or NULL */
    uint16_t lmax, nmax;
    uint32_t reserved;      /* 0 */
} catana_catalog_t;

/* Batched flags (combine with CATANA_FORM_* and, for the plain form, CATANA_JL_*). */
#define CATANA_BATCH_NO_GRAPH 16u  /* split form: launch the level loop directly
                                      instead of capturing it as one CUDA graph */
#define CATANA_BATCH_MBLK64 64u    /* split form, fixed schedule (waves > 0): work items of
                                      at most 64 complex m instead of 128 */

/* Split form: the catalogs advance level by level together -- at each l one
 * grouped tcgen05 launch covers every catalog's (m-block, tile-slab) work items and
 * one grouped reduction folds them into each catalog's f -- and the whole level
 * loop is captured and launched as one CUDA graph.  `waves` sets how many CTAs per
 * SM each level's items are cut for, and the work items hold at most 128 complex m
 * (64 with CATANA_BATCH_MBLK64: the MMA tile's N, 2 m per column pair); waves <= 0
 * autotunes both -- the schedule and the tile shape -- by timing the contraction at
 * three sample levels for each candidate, once per distinct catalog set
 * (catana_gpu_batch_waves() and catana_gpu_batch_mblk() report the choice).  Plain form: the
 * catalogs run one after another through the FP64 path (waves ignored).
 * Host pointers in the catalog records; blocks until the results are in place. */
catana_status_t catana_gpu_sfb_raw_batched(const catana_catalog_t *cats, int32_t ncat, uint32_t flags, double waves,
                                           catana_gpu_stream_t stream);

/* The same with device pointers in the catalog records (the record array itself
 * stays on the host); enqueued on `stream`.  It synchronises once to read the
 * catalogs' extents and weight sums.  *status_dev as for catana_gpu_sfb_raw_dev. */
catana_status_t catana_gpu_sfb_raw_batched_dev(const catana_catalog_t *cats, int32_t ncat, uint32_t flags,
                                               double waves, int *status_dev, catana_gpu_stream_t stream);

/* Waves per SM the last split-form run used (the autotuned value when it tuned). */
double catana_gpu_batch_waves(void);
/* Most complex m per work item of the last split-form run (128 or 64). */
int32_t catana_gpu_batch_mblk(void);

/* ---- chunked accumulation of one large catalog (no counterpart in the reference) --
 * For catalogs streamed from disk or host memory in chunks (the reference's
 * FilterStream buffers the whole catalog before decomposing it,
 * FilterStream.cpp:100-124).  create() computes k_ln and zeroes the f sum on the
 * device; each add() copies one chunk from host memory (pinned memory makes the copy
 * asynchronous: the copy of chunk k+1 overlaps the decomposition of chunk k) and
 * decomposes it on the accumulator's own streams; finish() normalises with the total
 * point count (or weight sum), forms C_ln and writes k_ln, c_ln and optionally f_lmn
 * (host, layouts as catana_gpu_sfb_raw).  Flags: CATANA_FORM_* (and CATANA_JL_EXACT
 * for the plain form; JL_AUTO takes the table form, the reference's rule for any
 * catalog of more than 1000 points).  A host chunk may be reused once the second
 * add() after it, or finish(), has returned (pageable memory: at once).  Chunks must
 * all carry weights or none.  finish() ends the accumulation.  An accumulator is
 * used from one thread at a time. */
typedef struct catana_gpu_accum *catana_gpu_accum_t;
typedef struct catana_ingest catana_ingest_t;  /* record layout and filters, defined below */
catana_status_t catana_gpu_accum_create(uint16_t lmax, uint16_t nmax, double rmax, uint32_t flags,
                                        catana_gpu_accum_t *out);
/* chunk of n float32 (r, theta, phi) records (the SphericalRecord<float> layout that
 * RawBinarySource reads, record_types.hpp:82-160) and optional float32 weights */
catana_status_t catana_gpu_accum_add_f32(catana_gpu_accum_t acc, const float *points, const float *weights,
                                         int64_t n);
/* chunk of n float64 (r, theta, phi) records and optional weights */
catana_status_t catana_gpu_accum_add(catana_gpu_accum_t acc, const double *points, const double *weights,
                                     int64_t n);
/* chunk of n raw records converted and filtered on the device (catana_ingest_t;
 * index0 counts records across chunks for the random windows), the kept points
 * decomposed; no weights */
catana_status_t catana_gpu_accum_add_records(catana_gpu_accum_t acc, const void *records, int64_t n,
                                             const catana_ingest_t *spec);
/* records [first_record, first_record + max_records) of a raw binary file (the
 * RawBinarySource format, RawBinarySource.cpp:6-61: consecutive records of 3 floats or
 * 3 doubles, Cartesian or spherical per spec->layout; max_records < 0 = to the end),
 * read chunk_records at a time into pinned buffers by a reader thread while the
 * previous chunk is filtered and decomposed as in add_records (index0 of the random
 * windows advances with the record number).  *records_read receives the count. */
catana_status_t catana_gpu_accum_add_file(catana_gpu_accum_t acc, const char *path, int64_t first_record,
                                          int64_t max_records, int64_t chunk_records, const catana_ingest_t *spec,
                                          int64_t *records_read);
catana_status_t catana_gpu_accum_finish(catana_gpu_accum_t acc, double *k_ln, double *c_ln, double *f_lmn);
catana_status_t catana_gpu_accum_destroy(catana_gpu_accum_t acc);

/* ---- catalog ingest on the device (no counterpart in the reference's API) ----
 * Record conversion and the reference's point filters, run on the GPU ahead of a
 * decomposition: the parts of its FilterStream pipeline (FilterStream.cpp:100-124)
 * that touch every point. */
#define CATANA_REC_FLOAT64 0u    /* records are 3 doubles */
#define CATANA_REC_FLOAT32 1u    /* records are 3 floats (RawBinarySource<...Record<float>>) */
#define CATANA_REC_SPHERICAL 0u  /* (r, theta, phi), taken as given (Point.cpp:23-28) */
#define CATANA_REC_CARTESIAN 2u  /* (x, y, z) -> Point(x, y, z) (Point.cpp:5-10) */

struct catana_ingest {
    uint32_t layout;        /* CATANA_REC_* */
    uint32_t reserved;      /* 0 */
    double tophat_r0;       /* > 0: TophatRadialWindowFunctionFilter: keep r < R0 (radial_filters.cpp:32-34) */
    double gauss_r0;        /* > 0: GaussianRadialWindowFunctionFilter: keep if exp(-(r/R0)^2) > u (:26-28) */
    const double *window;   /* GenericRadialWindowFunctionFilter with an interpolated window: keep if w(r) > u;
                               w on window_n equally spaced nodes of [window_min, window_max], evaluated as
                               FunctionInterpolator (FunctionInterpolator.cpp:6-30; r outside -> CATANA_ERR_DOMAIN);
                               host array, NULL = off */
    int64_t window_n;
    double window_min, window_max;
    const float *mask;      /* AngularMaskFilter: RING map of 12 mask_nside^2 floats, keep if map[ang2pix] == 1
                               (angular_filters.cpp:11-13); host array, NULL = off */
    int64_t mask_nside;
    uint64_t seed;          /* u of record i = SplitMix64 hash of (seed, index0 + i), uniform in [0, 1) */
    uint64_t index0;
};

/* Convert and filter n host records; the kept points, (r, theta, phi) float64 in input
 * order, go to points_out (host, room for n x 3) and their number to *n_out.  The
 * reference's Filter swaps each rejected point with the last unread one (Filter.cpp:
 * 25-35), so its survivors come out permuted; the SFB does not depend on the order
 * beyond rounding. */
catana_status_t catana_gpu_ingest(const void *records, int64_t n, const catana_ingest_t *spec, double *points_out,
                                  int64_t *n_out, catana_gpu_stream_t stream);

/* HEALPix (pixelized) SFB decomposition.  The catalog is given binned: pixel p
 * (RING scheme) holds the radii r_sorted[pix_offsets[p] .. pix_offsets[p+1]), in
 * the order the points were added.  npix = 12 nside^2; pix_offsets has npix+1
 * entries.  Host pointers.  Replaces sfb_decomposition(const
 * PixelizedPointContainer&, ...) and _sfb_reverse_fft (sfb_reverse_fft.cpp:43-209). */
catana_status_t catana_gpu_sfb_healpix(int64_t nside, const int64_t *pix_offsets, const double *r_sorted,
                                       uint16_t lmax, uint16_t nmax, double rmax, uint32_t flags, double *k_ln,
                                       double *c_ln, double *f_lmn, catana_gpu_stream_t stream);

/* Pixelized SFB without FFT: the reference's _sfb_reverse (sfb_reverse.cpp:13-112),
 * which the public wrappers do not call.  Same arguments and outputs as
 * catana_gpu_sfb_healpix; f_lmn = sum over pixels of Y*_lm(pixel centre) times the
 * pixel's sum of j_l(k_ln r), with the C_ln and f normalisation of that file.  The
 * JL flag picks the j_l branch (the reference passes `interpolated` explicitly;
 * CATANA_JL_AUTO applies the N > 1000 rule). */
catana_status_t catana_gpu_sfb_reverse(int64_t nside, const int64_t *pix_offsets, const double *r_sorted,
                                       uint16_t lmax, uint16_t nmax, double rmax, uint32_t flags, double *k_ln,
                                       double *c_ln, double *f_lmn, catana_gpu_stream_t stream);

/* Bin a catalog into RING pixels: the PixelizedPointContainer(nside, pc)
 * constructor (PixelizedPointContainer.cpp:11-30).  points: host npoints x 3
 * (r, theta, phi).  Outputs (host): pix_offsets[npix+1] and r_sorted[npoints],
 * radii grouped by pixel in point order.  nside must be a power of two
 * (CATANA_ERR_ARG otherwise, like the reference); theta outside [0, pi] is
 * CATANA_ERR_ARG (HEALPix asserts there). */
catana_status_t catana_gpu_bin_points(int64_t nside, const double *points, int64_t npoints, int64_t *pix_offsets,
                                      double *r_sorted, catana_gpu_stream_t stream);

/* HEALPix RING ang2pix for n angles (host arrays in, host array out):
 * Healpix_Base::ang2pix(pointing) as used at PixelizedPointContainer.cpp:28. */
catana_status_t catana_gpu_ang2pix_ring(int64_t nside, const double *theta, const double *phi, int64_t n,
                                        int64_t *pix, catana_gpu_stream_t stream);

/* HEALPix RING pix2ang for n pixel indices: Healpix_Base::pix2ang as used at
 * PixelizedPointContainer.cpp:17-19 (pixel centres). */
catana_status_t catana_gpu_pix2ang_ring(int64_t nside, const int64_t *pix, int64_t n, double *theta, double *phi,
                                        catana_gpu_stream_t stream);

/* Zeros 0..count-1 of j_l, computed on the host exactly as
 * besseltools::SphericalBesselZeros (SphericalBesselZeros.cpp:11-100), including
 * its Newton stopping rule.  Cached per process. */
catana_status_t catana_gpu_sbessel_zeros(uint32_t l, int32_t count, double *out);

/* Batched double spherical-Bessel integrals (the shot-noise integrals):
 *   out[p] = int_0^r_max w(r) j_l(k1[p] r) j_l(k2[p] r) dr,  p < npairs,
 * replacing besseltools::double_sbessel_integrator (sbessel_integrator.cpp:45-110,
 * vectorised over k1, k2 in py_besseltools.cpp:45-84).  w is a FunctionInterpolator
 * table: w_n values on equally spaced nodes of [w_min, w_max], linear in between
 * (FunctionInterpolator.cpp:6-30); [0, r_max) must lie inside it (CATANA_ERR_DOMAIN
 * otherwise, as the interpolator throws).  32-point Gauss-Legendre between the zeros of
 * both Bessel factors.  Host arrays. */
catana_status_t catana_gpu_sbessel_integrals(const double *w_table, int64_t w_n, double w_min, double w_max,
                                             uint32_t l, double r_max, const double *k1, const double *k2,
                                             int64_t npairs, double *out, catana_gpu_stream_t stream);

/* k_ln = z_{l,n} / rmax for l < lmax, n < nmax, row-major (return_types.cpp:10-20). */
catana_status_t catana_gpu_compute_kln(uint16_t lmax, uint16_t nmax, double rmax, double *k_ln);

/* Kernel timing for roofline reports.  While enabled, the library brackets every
 * launch of the dominant contraction kernel (the tcgen05 split kernel or the FP64
 * plain kernel) with CUDA events on the launching stream and records the launch's
 * algorithmic work (4 flops per point-mode).  catana_gpu_profile_report()
 * synchronises, returns the summed kernel time (ms), the number of timed launches
 * and the summed algorithmic flops, and clears the record.  No counterpart in the
 * reference (it has no GPU). */
void catana_gpu_profile_enable(int enable);
catana_status_t catana_gpu_profile_report(double *kernel_ms, uint64_t *launches, double *algo_flops);

/* FP64 FMA throughput of the current device as its clocks stand (TFLOP/s, 2 flops
 * per FMA): independent FMA chains, 8 CTAs of 256 threads per SM, about `ms`
 * milliseconds in three timed launches, the best one reported.  The denominator of
 * the plain path's roofline.  No counterpart in the reference. */
catana_status_t catana_gpu_fp64_peak(int32_t ms, double *tflops);

/* Test hook for the split kernel's bounded waits (no counterpart in the reference,
 * whose GSL errors are switched off, sfb_raw.cpp:26).  Arms the next split-form run
 * only: every work item withholds the hand-off of its first tile's operands, so the
 * tensor-core warps' wait on it -- limited to wait_us microseconds for that run
 * instead of 1 s -- runs out.  The kernel then stops issuing work, lets copies and
 * MMAs already in flight land, frees its tensor memory and records CATANA_ERR_CUDA,
 * which the entry point returns; the context stays usable.  wait_us in [1, 1e6]. */
catana_status_t catana_gpu_test_split_stall(uint32_t wait_us);

/* Message of the last failing call on this thread ("" if none). */
const char *catana_gpu_last_error(void);

/* Number of kernel launches the library issued since process start (all devices). */
uint64_t catana_gpu_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* CATANA_GPU_H */
