// common.cuh -- shared declarations of the catana_gpu library (host side).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/catana_gpu.h"

namespace catana_gpu {

// Launch counter behind catana_gpu_launch_count().
extern std::atomic<uint64_t> g_launches;
inline void count_launch(uint64_t n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

void set_error(const std::string &msg);

// Kernel timing (catana_gpu_profile_*): prof_begin/prof_end bracket one launch of
// the dominant kernel when profiling is enabled.
void prof_begin(cudaStream_t st);
void prof_end(cudaStream_t st, double algo_flops);

// Grow-only device buffer.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need) {
        if (need <= bytes) return cudaSuccess;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        size_t cap = need + need / 4;
        cudaError_t e = cudaMalloc(&ptr, cap);
        if (e == cudaSuccess) bytes = cap;
        return e;
    }
    template <class T> T *as() const { return reinterpret_cast<T *>(ptr); }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
};

// Cached split-form tables (per device): j_l piecewise polynomials, recurrence
// coefficients and the largest |j_l| per l.
struct SplitCache {
    int lmax = -1, nmax = -1, nint = -1;
    std::vector<double> maxj;   // 1.05 max |j_l| (first maximum)
    std::vector<double> zpeak;  // where that maximum sits (j_l rises monotonically below)
};

// Per-device state: workspace and cached tables.  Guarded by `mu`.
struct DeviceContext {
    std::mutex mu;
    int device = 0;
    int sm_count = 0;
    int cc_major = 0, cc_minor = 0;
    // workspace
    DevBuf soa;        // point SoA (r, x, w, cos phi, sin phi, phase fraction) of the current chunk
    DevBuf state;      // Legendre recurrence rows
    DevBuf partial;    // per-slab partial sums
    DevBuf flmn;       // f_lmn accumulator (complex, packed)
    DevBuf kln;        // k_ln on device
    DevBuf coef;       // Legendre recurrence coefficients
    DevBuf tables;     // j_l interpolation tables (FP64 lerp)
    DevBuf misc;       // error word, small scalars (never grown past 256 bytes: callers hold pointers into it)
    DevBuf cat_scratch;  // per-catalog scalars of batched runs (extents, weight sums)
    DevBuf io_points;  // staging of host inputs
    DevBuf io_out;     // staging of outputs
    DevBuf split_ws;   // split-form workspace
    DevBuf split_tab;  // split-form tables
    DevBuf split_plan; // split-form plan (catalog descriptors, items, reductions)
    SplitCache split_cache;
    std::map<std::string, std::pair<double, int>> split_tuned;  // autotuned (waves, m-block cap) per catalog set
    double split_last_waves = 0.0;
    int split_last_mblk = 0;
    cudaStream_t capture_stream = nullptr;      // stream the split level loop is captured on
    cudaEvent_t split_ws_event = nullptr;       // end of the last split run (orders workspace reuse across streams)
    DevBuf hp_ws;      // HEALPix workspace
    DevBuf ingest_ws;  // ingest: converted records, keep flags, block counts, window, mask
    // kernels whose shared-memory limit this device's context has raised (the
    // attribute is per device, so it is tracked here rather than per process)
    bool attr_fp64 = false, attr_split = false, attr_healpix = false;
    // cache keys
    int coef_lmax = -1;
    int tab_lmax = -1, tab_nmax = -1;
    std::vector<double> tab_dxinv, tab_zmax;  // per l
    DevBuf poly;       // piecewise FP64 j_l polynomials [l][interval][12] (CATANA_JL_POLY)
    int poly_lmax = -1, poly_nint = -1;
};

DeviceContext *get_context(int *status);

// Bessel zeros (host, cached): z[l][n] for n < count.  Thread-safe.
const double *zeros_for(unsigned l, int count);
// k_ln table row-major (lmax x nmax), host.
void kln_table(int lmax, int nmax, double rmax, double *out);

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

#define CG_CUDA_TRY(expr)                                                                        \
    do {                                                                                         \
        cudaError_t _e = (expr);                                                                 \
        if (_e != cudaSuccess) {                                                                 \
            ::catana_gpu::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));         \
            return _e == cudaErrorMemoryAllocation ? CATANA_ERR_NOMEM : CATANA_ERR_CUDA;          \
        }                                                                                        \
    } while (0)

// j_l evaluation of the FP64 plain path: the reference's linear table, the direct
// evaluation, or the piecewise FP64 polynomials (CATANA_JL_POLY).
enum JlMode { JL_MODE_LERP = 0, JL_MODE_EXACT = 1, JL_MODE_POLY = 2 };

// FP64 plain raw path (sfb_fp64.cu).  All pointers device.  Accumulates into
// f_acc (complex, packed by l, un-normalised); the caller normalises.
catana_status_t fp64_raw_accumulate(DeviceContext *ctx, const double *points_dev, const double *weights_dev,
                                    int64_t npoints, int lmax, int nmax, JlMode jl, const double *kln_dev,
                                    double *f_acc_dev, int *err_dev, cudaStream_t st);
// f *= norm; c_ln from f (device).
catana_status_t finish_flmn_cln(double *f_dev, double norm, int lmax, int nmax, double *c_ln_dev,
                                cudaStream_t st);
// FP64 lerp tables (1000*nmax nodes per l) for l < lmax, cached in ctx->tables.
catana_status_t ensure_lerp_tables(DeviceContext *ctx, int lmax, int nmax, cudaStream_t st);
// Legendre coefficients for l < lmax, cached in ctx->coef.
catana_status_t ensure_coefs(DeviceContext *ctx, int lmax, cudaStream_t st);

// One catalog of a split-form run (device pointers; f_acc zeroed by the caller).
struct SplitCatInput {
    const double *pts = nullptr;  // n x 3 (r, theta, phi)
    const double *w = nullptr;    // optional weights
    const float *pts32 = nullptr; // or: float32 records (r, theta, phi) and weights
    const float *w32 = nullptr;
    double max_r = -1.0, max_w = -1.0;  // >= 0: extents known to the caller (skips a read-back)
    int64_t n = 0;
    int lmax = 0, nmax = 0;
    double rmax = 1.0;
    double kmax = 0.0;            // > 0: keep only k_ln <= kmax
    double *kln_dev = nullptr;    // k_ln (lmax x nmax), already on the device
    double *f_acc = nullptr;      // packed complex f_lmn accumulator
    bool accurate = false;        // CATANA_SPLIT_ACCURATE: Reinsch-modified Legendre rows (always above lmax 256)
};
// Split form over several catalogs: level-synchronous launches over all of them,
// optionally captured as one CUDA graph.  `waves` = CTAs per SM each level's work
// items are cut for, `mblk` the most complex m per work item (128 or 64); waves <= 0
// autotunes both (timed sample levels, cached per catalog set).
catana_status_t split_run(DeviceContext *ctx, std::vector<SplitCatInput> &cats, bool use_graph, double waves,
                          int mblk, int *err_dev, cudaStream_t st);

// Convert, filter and compact n device records (ingest.cu); *n_out kept, in order.
catana_status_t ingest_dev(DeviceContext *ctx, const void *rec_dev, int64_t n, const catana_ingest_t &spec,
                           double *out_dev, int64_t *n_out, cudaStream_t st);

// Split (tensor-core) raw path (sfb_split.cu).
catana_status_t split_raw_accumulate(DeviceContext *ctx, const double *points_dev, const double *weights_dev,
                                     int64_t npoints, int lmax, int nmax, double rmax, const double *kln_dev,
                                     double *f_acc_dev, int *err_dev, cudaStream_t st, bool accurate);

// Stable radix sort of (key, index) pairs by the low key_bits bits (sort.cu).
catana_status_t radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *tmp_keys, uint32_t *tmp_vals, int64_t n,
                                 int key_bits, uint32_t *hist_scratch, cudaStream_t st);

// In-place exclusive scan of uint32 words (sort.cu).
catana_status_t scan_u32(uint32_t *data, int64_t count, cudaStream_t st);

// HEALPix (healpix.cu).
catana_status_t healpix_bin_dev(DeviceContext *ctx, int64_t nside, const double *points_dev, int64_t npoints,
                                int64_t *offsets_dev, double *r_sorted_dev, int *err_dev, cudaStream_t st);
catana_status_t healpix_ang2pix_dev(int64_t nside, const double *theta, const double *phi, int64_t n,
                                    int64_t *pix, int *err_dev, cudaStream_t st);
catana_status_t healpix_pix2ang_dev(int64_t nside, const int64_t *pix, int64_t n, double *theta, double *phi,
                                    cudaStream_t st);
// kln_host (L x M, may be null) and the radii's range [r_min, r_max] (r_min NaN when a
// radius is NaN) let levels that lie inside the j_l table skip the per-point range test
catana_status_t healpix_sfb_dev(DeviceContext *ctx, int64_t nside, const int64_t *offsets_dev,
                                const double *r_sorted_dev, int64_t npoints, int lmax, int nmax, bool interpolated,
                                bool conj_fix, const double *kln_dev, const double *kln_host, double r_min,
                                double r_max, double norm, double *f_dev, double *c_ln_dev, int *err_dev,
                                cudaStream_t st);

}  // namespace catana_gpu
