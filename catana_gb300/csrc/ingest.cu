// ingest.cu -- catalog ingest on the device: record conversion, the reference's point
// filters and order-keeping compaction, ahead of a decomposition.
//
// Per record (float32 or float64; Cartesian x, y, z or spherical r, theta, phi):
//   * Cartesian: Point(x, y, z) (Point.cpp:5-10): r = |v|, theta = atan2(rho, z),
//     phi = atan2(y, x) normalised into [0, 2 pi) (0 when x = y = 0);
//     spherical: taken as given (point_from_spherical_position, Point.cpp:23-28);
//   * TophatRadialWindowFunctionFilter (radial_filters.cpp:32-34): keep r < R0;
//   * GaussianRadialWindowFunctionFilter (:26-28) / GenericRadialWindowFunctionFilter
//     with an interpolated window (:12-24, FunctionInterpolator.cpp:6-30): keep when
//     w(r) > u, u uniform in [0, 1);
//   * AngularMaskFilter (angular_filters.cpp:11-13): keep when map[ang2pix(theta, phi)]
//     == 1 on a RING map.
// Kept records come out in input order.  (The reference's Filter swaps each rejected
// point with the last unread one, Filter.cpp:25-35, so its survivors are permuted; the
// SFB sums do not depend on the order beyond rounding.)  The uniform of record i is a
// SplitMix64 hash of (seed, index0 + i) -- a counter-based stream, so the decision for
// a record does not depend on the chunking or on the other filters (the reference draws
// from one global std::mt19937 in filter order).
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "hpx_ring.cuh"
#include "special.cuh"

namespace catana_gpu {

namespace {

constexpr int IG_BLOCK = 1024;

struct IngestDev {
    uint32_t layout;
    int has_tophat, has_gauss, has_window, has_mask;
    double tophat_r0, gauss_r0;
    const double *window;
    int64_t window_n;
    double window_min, window_max, window_dx_inv;
    const float *mask;
    int64_t mask_nside;
    uint64_t seed, index0;
};

__host__ __device__ inline double ingest_uniform(uint64_t seed, uint64_t index) {
    uint64_t z = seed + (index + 1) * 0x9E3779B97F4A7C15ull;  // SplitMix64
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * 0x1.0p-53;
}

__device__ inline void load_record(const void *rec, uint32_t layout, int64_t i, double &a, double &b, double &c) {
    if (layout & CATANA_REC_FLOAT32) {
        const float *p = reinterpret_cast<const float *>(rec) + 3 * i;
        a = (double)p[0];
        b = (double)p[1];
        c = (double)p[2];
    } else {
        const double *p = reinterpret_cast<const double *>(rec) + 3 * i;
        a = p[0];
        b = p[1];
        c = p[2];
    }
}

// convert + filter; keep flag per record, kept count per block (flags: 1 window domain, 2 mask theta)
__global__ void __launch_bounds__(IG_BLOCK) k_ingest_mark(const void *__restrict__ rec, int64_t n, IngestDev sp,
                                                           double *__restrict__ tmp, uint8_t *__restrict__ keepv,
                                                           uint32_t *__restrict__ bcount, int *__restrict__ err) {
    const int64_t i = blockIdx.x * (int64_t)IG_BLOCK + threadIdx.x;
    int keep = 0;
    if (i < n) {
        double r, th, ph;
        double a, b, c;
        load_record(rec, sp.layout, i, a, b, c);
        if (sp.layout & CATANA_REC_CARTESIAN) {
            r = sqrt(a * a + b * b + c * c);
            th = atan2(sqrt(a * a + b * b), c);
            ph = (a == 0.0 && b == 0.0) ? 0.0 : atan2(b, a);
            if (ph < 0.0) ph += 2.0 * kPi;
            if (ph >= 2.0 * kPi) ph = fmod(ph, 2.0 * kPi);
        } else {
            r = a;
            th = b;
            ph = c;
        }
        keep = 1;
        if (sp.has_tophat && !(r < sp.tophat_r0)) keep = 0;
        if (keep && (sp.has_gauss || sp.has_window)) {
            const double u = ingest_uniform(sp.seed, sp.index0 + (uint64_t)i);
            if (sp.has_gauss) {
                const double q = r / sp.gauss_r0;
                if (!(exp(-(q * q)) > u)) keep = 0;
            }
            if (keep && sp.has_window) {
                if (r < sp.window_min || r >= sp.window_max) {
                    atomicOr(err, 1);
                    keep = 0;
                } else {
                    const double x = r - sp.window_min;
                    const double ia = x * sp.window_dx_inv;
                    const unsigned ii = min((unsigned)ia, (unsigned)(sp.window_n - 2));  // r just below the top
                    const double w = sp.window[ii] + (sp.window[ii + 1] - sp.window[ii]) * (ia - ii);
                    if (!(w > u)) keep = 0;
                }
            }
        }
        if (keep && sp.has_mask) {
            const int64_t pix = ang2pix_ring_dev(sp.mask_nside, th, ph);
            if (pix < 0) {
                atomicOr(err, 2);
                keep = 0;
            } else if (!(sp.mask[pix] == 1.0f)) {
                keep = 0;
            }
        }
        tmp[3 * i] = r;
        tmp[3 * i + 1] = th;
        tmp[3 * i + 2] = ph;
        keepv[i] = (uint8_t)keep;
    }
    const int cnt = __syncthreads_count(keep);
    if (threadIdx.x == 0) bcount[blockIdx.x] = (uint32_t)cnt;
}

// kept records to out[boff[block] + rank within the block], input order
__global__ void __launch_bounds__(IG_BLOCK) k_ingest_scatter(const double *__restrict__ tmp,
                                                              const uint8_t *__restrict__ keepv, int64_t n,
                                                              const uint32_t *__restrict__ boff,
                                                              double *__restrict__ out) {
    __shared__ uint32_t wsum[IG_BLOCK / 32];
    const int64_t i = blockIdx.x * (int64_t)IG_BLOCK + threadIdx.x;
    const int keep = (i < n) ? keepv[i] : 0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) wsum[warp] = __popc(bal);
    __syncthreads();
    if (warp == 0) {  // exclusive scan of the 32 warp counts
        const uint32_t v = wsum[lane];
        uint32_t s = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        wsum[lane] = s - v;
    }
    __syncthreads();
    if (keep) {
        const uint64_t dst = (uint64_t)boff[blockIdx.x] + wsum[warp] + __popc(bal & ((1u << lane) - 1u));
        out[3 * dst] = tmp[3 * i];
        out[3 * dst + 1] = tmp[3 * i + 1];
        out[3 * dst + 2] = tmp[3 * i + 2];
    }
}

bool spec_valid(const catana_ingest_t &s, std::string &why) {
    if (s.layout & ~(CATANA_REC_FLOAT32 | CATANA_REC_CARTESIAN)) {
        why = "unknown record layout bits";
        return false;
    }
    if (s.tophat_r0 < 0.0 || s.gauss_r0 < 0.0 || !std::isfinite(s.tophat_r0) || !std::isfinite(s.gauss_r0)) {
        why = "tophat_r0 and gauss_r0 must be >= 0 and finite (0 = off)";
        return false;
    }
    if (s.window && (s.window_n < 2 || !(s.window_max > s.window_min))) {
        why = "window: window_n >= 2 nodes on window_min < window_max";
        return false;
    }
    if (s.mask && (s.mask_nside < 1 || (s.mask_nside & (s.mask_nside - 1)) != 0)) {
        why = "mask_nside must be a power of 2";
        return false;
    }
    return true;
}

}  // namespace

// Convert, filter and compact n device records into out_dev (n x 3 float64 capacity);
// the kept count is returned through *n_out (one read-back).  window and mask in
// `spec` are host arrays (copied here).
catana_status_t ingest_dev(DeviceContext *ctx, const void *rec_dev, int64_t n, const catana_ingest_t &spec,
                           double *out_dev, int64_t *n_out, cudaStream_t st) {
    std::string why;
    if (!spec_valid(spec, why)) {
        set_error("ingest: " + why);
        return CATANA_ERR_ARG;
    }
    *n_out = 0;
    if (n <= 0) return CATANA_OK;
    const int64_t nb = (n + IG_BLOCK - 1) / IG_BLOCK;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t tb = al((size_t)n * 3 * sizeof(double)), kb = al((size_t)n), cb = al((size_t)(nb + 1) * 4),
                 wb = spec.window ? al((size_t)spec.window_n * sizeof(double)) : 0,
                 mb = spec.mask ? al((size_t)12 * spec.mask_nside * spec.mask_nside * sizeof(float)) : 0;
    CG_CUDA_TRY(ctx->ingest_ws.ensure(tb + kb + cb + wb + mb + 256));
    char *w = ctx->ingest_ws.as<char>();
    double *tmp = reinterpret_cast<double *>(w);
    uint8_t *keepv = reinterpret_cast<uint8_t *>(w + tb);
    uint32_t *cnt = reinterpret_cast<uint32_t *>(w + tb + kb);
    double *win = reinterpret_cast<double *>(w + tb + kb + cb);
    float *msk = reinterpret_cast<float *>(w + tb + kb + cb + wb);
    IngestDev sp;
    memset(&sp, 0, sizeof(sp));
    sp.layout = spec.layout;
    sp.has_tophat = spec.tophat_r0 > 0.0;
    sp.tophat_r0 = spec.tophat_r0;
    sp.has_gauss = spec.gauss_r0 > 0.0;
    sp.gauss_r0 = spec.gauss_r0;
    if (spec.window) {
        CG_CUDA_TRY(cudaMemcpyAsync(win, spec.window, (size_t)spec.window_n * sizeof(double), cudaMemcpyHostToDevice,
                                    st));
        sp.has_window = 1;
        sp.window = win;
        sp.window_n = spec.window_n;
        sp.window_min = spec.window_min;
        sp.window_max = spec.window_max;
        sp.window_dx_inv = 1.0 / ((spec.window_max - spec.window_min) / (double)(spec.window_n - 1));
    }
    if (spec.mask) {
        CG_CUDA_TRY(cudaMemcpyAsync(msk, spec.mask, (size_t)12 * spec.mask_nside * spec.mask_nside * sizeof(float),
                                    cudaMemcpyHostToDevice, st));
        sp.has_mask = 1;
        sp.mask = msk;
        sp.mask_nside = spec.mask_nside;
    }
    sp.seed = spec.seed;
    sp.index0 = spec.index0;
    CG_CUDA_TRY(ctx->misc.ensure(256));
    int *err = reinterpret_cast<int *>(ctx->misc.as<char>() + 128);
    CG_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
    CG_CUDA_TRY(cudaMemsetAsync(cnt + nb, 0, sizeof(uint32_t), st));
    k_ingest_mark<<<(unsigned)nb, IG_BLOCK, 0, st>>>(rec_dev, n, sp, tmp, keepv, cnt, err);
    count_launch();
    CG_CUDA_TRY(cudaGetLastError());
    catana_status_t s = scan_u32(cnt, nb + 1, st);
    if (s != CATANA_OK) return s;
    k_ingest_scatter<<<(unsigned)nb, IG_BLOCK, 0, st>>>(tmp, keepv, n, cnt, out_dev);
    count_launch();
    CG_CUDA_TRY(cudaGetLastError());
    uint32_t tot = 0;
    int err_h = 0;
    CG_CUDA_TRY(cudaMemcpyAsync(&tot, cnt + nb, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CG_CUDA_TRY(cudaMemcpyAsync(&err_h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CG_CUDA_TRY(cudaStreamSynchronize(st));
    if (err_h & 1) {
        set_error("argument outside range for which this FunctionInterpolator is defined");
        return CATANA_ERR_DOMAIN;
    }
    if (err_h & 2) {
        set_error("angular mask: theta outside [0, pi]");
        return CATANA_ERR_DOMAIN;
    }
    *n_out = (int64_t)tot;
    return CATANA_OK;
}

}  // namespace catana_gpu

using namespace catana_gpu;

extern "C" {

catana_status_t catana_gpu_ingest(const void *records, int64_t n, const catana_ingest_t *spec, double *points_out,
                                  int64_t *n_out, catana_gpu_stream_t stream) {
    if (!spec || !n_out || n < 0 || (n > 0 && (!records || !points_out))) {
        set_error("ingest: null argument or n < 0");
        return CATANA_ERR_ARG;
    }
    if (n > (int64_t)0xFFFFFFF0ll) {
        set_error("ingest: at most 2^32 - 16 records per call");
        return CATANA_ERR_ARG;
    }
    *n_out = 0;
    std::string why;
    if (!spec_valid(*spec, why)) {
        set_error("ingest: " + why);
        return CATANA_ERR_ARG;
    }
    int cs;
    DeviceContext *ctx = get_context(&cs);
    if (!ctx) return (catana_status_t)cs;
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const size_t rb = (size_t)n * 3 * ((spec->layout & CATANA_REC_FLOAT32) ? 4 : 8);
    CG_CUDA_TRY(ctx->io_points.ensure(rb + (size_t)n * 3 * sizeof(double) + 512));
    char *in_d = ctx->io_points.as<char>();
    double *out_d = reinterpret_cast<double *>(in_d + ((rb + 255) & ~size_t(255)));
    if (n) CG_CUDA_TRY(cudaMemcpyAsync(in_d, records, rb, cudaMemcpyHostToDevice, st));
    int64_t kept = 0;
    catana_status_t s = ingest_dev(ctx, in_d, n, *spec, out_d, &kept, st);
    if (s != CATANA_OK) return s;
    if (kept) {
        CG_CUDA_TRY(cudaMemcpyAsync(points_out, out_d, (size_t)kept * 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
        CG_CUDA_TRY(cudaStreamSynchronize(st));
    }
    *n_out = kept;
    return CATANA_OK;
}

}  // extern "C"
