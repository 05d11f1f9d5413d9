// catana_gpu.cu -- C ABI of libcatana_gpu (declared in include/catana_gpu.h):
// device contexts, the host-side Bessel-zero cache and the entry points that move
// host catalogs to the device and results back.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "special.cuh"

namespace catana_gpu {

std::atomic<uint64_t> g_launches{0};
static thread_local std::string t_last_error;

void set_error(const std::string &msg) { t_last_error = msg; }

// ---------------------------------------------------------------------------
// Kernel timing
// ---------------------------------------------------------------------------
static std::atomic<int> g_prof_on{0};
static std::mutex g_prof_mu;
struct ProfRec {
    cudaEvent_t a, b;
    double flops;
};
static std::vector<ProfRec> g_prof;
static std::vector<cudaEvent_t> g_prof_free;

static cudaEvent_t prof_event() {
    if (!g_prof_free.empty()) {
        cudaEvent_t e = g_prof_free.back();
        g_prof_free.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void prof_begin(cudaStream_t st) {
    if (!g_prof_on.load()) return;
    std::lock_guard<std::mutex> g(g_prof_mu);
    ProfRec r;
    r.a = prof_event();
    r.b = nullptr;
    r.flops = 0.0;
    cudaEventRecord(r.a, st);
    g_prof.push_back(r);
}

void prof_end(cudaStream_t st, double algo_flops) {
    if (!g_prof_on.load()) return;
    std::lock_guard<std::mutex> g(g_prof_mu);
    if (g_prof.empty() || g_prof.back().b) return;
    g_prof.back().b = prof_event();
    g_prof.back().flops = algo_flops;
    cudaEventRecord(g_prof.back().b, st);
}

// ---------------------------------------------------------------------------
// Bessel zeros: SphericalBesselZeros.cpp:11-68.  Asymptotic guesses for the first
// two zeros (:17-47), Newton iterations that stop as soon as delta/z <= 1e-15 --
// which includes every negative step (:49-62) -- and linear extrapolation
// 2 z_{n-1} - z_{n-2} as the guess for later zeros (:64-68).  The quirky stop is
// kept on purpose: the reference's k_ln are these values, not converged roots.
// ---------------------------------------------------------------------------
static double newton(unsigned l, double z) {
    double delta, jl;
    do {
        jl = sbessel_jl((int)l, z);
        delta = jl / ((double)l / z * jl - sbessel_jl((int)l + 1, z));
        z -= delta;
    } while (delta / z > 1e-15);
    return z;
}

static void zeros_extend(unsigned l, std::vector<double> &z, int count) {
    if (z.empty()) {
        double z0, z1;
        if (l == 0) {
            z0 = 3.141592653589793238463;
            z1 = 6.283185307179586476925;
        } else {
            const double lh = l + 0.5;
            z0 = l + 0.5 + 1.8557571 * std::pow(lh, 1. / 3.) + 1.033150 * std::pow(lh, -1. / 3.) -
                 0.00397 * std::pow(lh, -1.) - 0.0908 * std::pow(lh, -5. / 3.) + 0.043 * std::pow(lh, -7. / 3.);
            z1 = l + 0.5 + 3.2446076 * std::pow(lh, 1. / 3.) + 3.158244 * std::pow(lh, -1. / 3.) -
                 0.08331 * std::pow(lh, -1.) - 0.8437 * std::pow(lh, -5. / 3.) + 0.864 * std::pow(lh, -7. / 3.);
        }
        z.push_back(newton(l, z0));
        z.push_back(newton(l, z1));
    }
    while ((int)z.size() < count) {
        const double g = 2 * z[z.size() - 1] - z[z.size() - 2];
        z.push_back(newton(l, g));
    }
}

static std::mutex g_zero_mu;
static std::map<unsigned, std::unique_ptr<std::vector<double>>> g_zeros;

// Make sure zeros 0..count-1 exist for every l in ls (parallel over l).
static void zeros_prepare(const std::vector<unsigned> &ls, int count) {
    std::vector<std::vector<double> *> todo;
    std::vector<unsigned> todo_l;
    {
        std::lock_guard<std::mutex> g(g_zero_mu);
        for (unsigned l : ls) {
            auto &p = g_zeros[l];
            if (!p) p.reset(new std::vector<double>());
            if ((int)p->size() < count) {
                todo.push_back(p.get());
                todo_l.push_back(l);
            }
        }
    }
    if (todo.empty()) return;
    // The vectors are owned by the map and never erased, so workers can fill them
    // without holding the lock; concurrent callers extending the same l would
    // race, which the per-device mutex of every entry point prevents.
    unsigned nt = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), (unsigned)todo.size()));
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (size_t k = next.fetch_add(1); k < todo.size(); k = next.fetch_add(1))
            zeros_extend(todo_l[k], *todo[k], count);
    };
    std::vector<std::thread> th;
    for (unsigned t = 1; t < nt; ++t) th.emplace_back(work);
    work();
    for (auto &t : th) t.join();
}

const double *zeros_for(unsigned l, int count) {
    zeros_prepare({l}, count);
    std::lock_guard<std::mutex> g(g_zero_mu);
    return g_zeros[l]->data();
}

void kln_table(int lmax, int nmax, double rmax, double *out) {
    std::vector<unsigned> ls(lmax);
    for (int l = 0; l < lmax; ++l) ls[l] = l;
    zeros_prepare(ls, std::max(nmax, 2));
    for (int l = 0; l < lmax; ++l) {
        const double *z = zeros_for(l, std::max(nmax, 2));
        for (int n = 0; n < nmax; ++n) out[(size_t)l * nmax + n] = z[n] / rmax;  // return_types.cpp:15
    }
}

// ---------------------------------------------------------------------------
// Device contexts
// ---------------------------------------------------------------------------
static std::mutex g_ctx_mu;
static std::map<int, std::unique_ptr<DeviceContext>> g_ctx;

DeviceContext *get_context(int *status) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
        *status = CATANA_ERR_CUDA;
        return nullptr;
    }
    std::lock_guard<std::mutex> g(g_ctx_mu);
    auto &p = g_ctx[dev];
    if (!p) {
        std::unique_ptr<DeviceContext> c(new DeviceContext());
        c->device = dev;
        cudaDeviceProp prop;
        e = cudaGetDeviceProperties(&prop, dev);
        if (e != cudaSuccess) {
            set_error(std::string("cudaGetDeviceProperties: ") + cudaGetErrorString(e));
            *status = CATANA_ERR_CUDA;
            return nullptr;
        }
        c->sm_count = prop.multiProcessorCount;
        c->cc_major = prop.major;
        c->cc_minor = prop.minor;
        p = std::move(c);
    }
    *status = CATANA_OK;
    return p.get();
}

}  // namespace catana_gpu

using namespace catana_gpu;

namespace {

double norm_factor(double rmax, double wsum) {
    // sfb_raw.cpp:29-30: sqrt(2/pi) * (4/3) * pi * rmax^3 / N  (N -> sum of weights)
    double nf = std::sqrt(2. / kPi) * (4. / 3.) * kPi;
    nf *= rmax * rmax * rmax / wsum;
    return nf;
}

bool resolve_interp(uint32_t flags, int64_t npoints) {
    const uint32_t j = flags & CATANA_JL_MASK;
    if (j == CATANA_JL_INTERP) return true;
    if (j == CATANA_JL_EXACT) return false;
    return npoints > 1000;  // sfb_decomposition.cpp:17 (BESSELINTERPOLATIONPOINTS_PER_ZERO)
}

// j_l mode of the raw FP64 path: the reference's rule, or the polynomial tables
JlMode resolve_jl(uint32_t flags, int64_t npoints) {
    if ((flags & CATANA_JL_MASK) == CATANA_JL_POLY) return JL_MODE_POLY;
    return resolve_interp(flags, npoints) ? JL_MODE_LERP : JL_MODE_EXACT;
}

catana_status_t check_args(int64_t npoints, uint16_t lmax, uint16_t nmax, double rmax) {
    if (npoints < 0) {
        set_error("npoints must be >= 0");
        return CATANA_ERR_ARG;
    }
    if (!(rmax > 0.0) || !std::isfinite(rmax)) {
        set_error("rmax must be positive and finite");
        return CATANA_ERR_ARG;
    }
    (void)lmax;
    (void)nmax;
    return CATANA_OK;
}

// Weighted sum on device for the normalisation (sum of weights).
__global__ void k_wsum(const double *w, int64_t n, double *out) {
    // single CTA, fixed-order tree: deterministic
    __shared__ double sh[1024];
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += w[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

// Core of both raw entry points: device inputs, device outputs.  `wsum_host` < 0
// means "compute the weight sum on the device".
catana_status_t raw_device(DeviceContext *ctx, const double *pts_d, const double *w_d, int64_t npoints, int lmax,
                           int nmax, double rmax, uint32_t flags, double *kln_d, double *cln_d, double *f_d,
                           int *err_d, cudaStream_t st) {
    const bool split = (flags & CATANA_FORM_MASK) == CATANA_FORM_SPLIT;
    // k_ln on the host (cached zeros), then to the device
    std::vector<double> kh((size_t)lmax * nmax);
    kln_table(lmax, nmax, rmax, kh.data());
    CG_CUDA_TRY(cudaMemcpyAsync(kln_d, kh.data(), kh.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    const size_t fbytes = catana_gpu_flmn_size(lmax, nmax) * 2 * sizeof(double);
    double *facc = f_d;
    if (!facc) {
        CG_CUDA_TRY(ctx->flmn.ensure(fbytes));
        facc = ctx->flmn.as<double>();
    }
    CG_CUDA_TRY(cudaMemsetAsync(facc, 0, fbytes, st));
    catana_status_t s;
    if (split) {
        if (ctx->cc_major != 10 || ctx->cc_minor != 3) {
            set_error("the split (tcgen05) form needs an sm_103 device");
            return CATANA_ERR_UNSUPPORTED;
        }
        s = split_raw_accumulate(ctx, pts_d, w_d, npoints, lmax, nmax, rmax, kln_d, facc, err_d, st,
                                 (flags & CATANA_SPLIT_ACCURATE) != 0);
    } else {
        s = fp64_raw_accumulate(ctx, pts_d, w_d, npoints, lmax, nmax, resolve_jl(flags, npoints), kln_d, facc,
                                err_d, st);
    }
    if (s != CATANA_OK) return s;
    double wsum = (double)npoints;
    if (w_d && npoints > 0) {
        CG_CUDA_TRY(ctx->misc.ensure(256));
        double *ws = reinterpret_cast<double *>(ctx->misc.as<char>() + 64);
        k_wsum<<<1, 1024, 0, st>>>(w_d, npoints, ws);
        count_launch();
        CG_CUDA_TRY(cudaGetLastError());
        CG_CUDA_TRY(cudaMemcpyAsync(&wsum, ws, sizeof(double), cudaMemcpyDeviceToHost, st));
        CG_CUDA_TRY(cudaStreamSynchronize(st));
    }
    // an empty catalog divides by zero like the reference (f = 0 * inf = NaN)
    const double nf = norm_factor(rmax, wsum);
    return finish_flmn_cln(facc, nf, lmax, nmax, cln_d, st);
}

// FP64 FMA throughput: 8 independent dependent chains per thread (the result feeds a
// conditional store so no chain can be dropped).
__global__ void k_fp64_fma_chains(int iters, double b, double c, double *sink) {
    double a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = 1.0 + 1e-3 * (threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
    }
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) t += a[k];
    if (t == 1234.5) *sink = t;
}

// Zero the f entries of modes with k_ln > kmax (plain form of the kmax cut).
__global__ void k_kcut(double2 *f, const double *kln, int nmax, double kmax) {
    const int l = blockIdx.y;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (l + 1) * nmax) return;
    const int n = t % nmax;
    if (kln[(size_t)l * nmax + n] > kmax) f[(size_t)nmax * l * (l + 1) / 2 + t] = make_double2(0.0, 0.0);
}

catana_status_t check_catalogs(const catana_catalog_t *cats, int32_t ncat) {
    if (ncat < 0 || (ncat > 0 && !cats)) {
        set_error("ncat must be >= 0 and cats non-null");
        return CATANA_ERR_ARG;
    }
    for (int c = 0; c < ncat; ++c) {
        const catana_catalog_t &C = cats[c];
        catana_status_t s = check_args(C.npoints, C.lmax, C.nmax, C.rmax);
        if (s != CATANA_OK) return s;
        if ((C.npoints > 0 && !C.points) || ((size_t)C.lmax * C.nmax && (!C.k_ln || !C.c_ln))) {
            set_error("catalog " + std::to_string(c) + ": null buffer");
            return CATANA_ERR_ARG;
        }
        if (!(C.kmax >= 0.0) || std::isinf(C.kmax)) {
            set_error("catalog " + std::to_string(c) + ": kmax must be >= 0 and finite (0 = no cut)");
            return CATANA_ERR_ARG;
        }
    }
    return CATANA_OK;
}

// Core of both batched entry points: device pointers in the records.
catana_status_t batched_device(DeviceContext *ctx, const catana_catalog_t *cats, int ncat, uint32_t flags,
                               double waves, int *err_d, cudaStream_t st) {
    const bool split = (flags & CATANA_FORM_MASK) == CATANA_FORM_SPLIT;
    if (split && (ctx->cc_major != 10 || ctx->cc_minor != 3)) {
        set_error("the split (tcgen05) form needs an sm_103 device");
        return CATANA_ERR_UNSUPPORTED;
    }
    // k_ln (host, cached zeros) and zeroed accumulators; internal f where none is given
    size_t fin = 0;
    for (int c = 0; c < ncat; ++c)
        if (!cats[c].f_lmn) fin += catana_gpu_flmn_size(cats[c].lmax, cats[c].nmax) * 2;
    if (fin) CG_CUDA_TRY(ctx->flmn.ensure(fin * sizeof(double)));
    std::vector<double *> facc(ncat);
    std::vector<std::vector<double>> kh(ncat);
    size_t fo = 0;
    for (int c = 0; c < ncat; ++c) {
        const catana_catalog_t &C = cats[c];
        const size_t fc = catana_gpu_flmn_size(C.lmax, C.nmax) * 2;
        facc[c] = C.f_lmn ? C.f_lmn : ctx->flmn.as<double>() + fo;
        if (!C.f_lmn) fo += fc;
        kh[c].resize((size_t)C.lmax * C.nmax);
        kln_table(C.lmax, C.nmax, C.rmax, kh[c].data());
        if (!kh[c].empty())
            CG_CUDA_TRY(cudaMemcpyAsync(C.k_ln, kh[c].data(), kh[c].size() * sizeof(double), cudaMemcpyHostToDevice,
                                        st));
        if (fc) CG_CUDA_TRY(cudaMemsetAsync(facc[c], 0, fc * sizeof(double), st));
    }
    catana_status_t s;
    if (split) {
        // catalogs whose Legendre rows exceed 16 GB enter as chunks (same accumulator)
        std::vector<SplitCatInput> v;
        for (int c = 0; c < ncat; ++c) {
            const catana_catalog_t &C = cats[c];
            if (C.npoints == 0 || C.lmax == 0 || C.nmax == 0) continue;
            const int64_t chunk =
                std::max<int64_t>(32, std::min<int64_t>(C.npoints, (int64_t)(16e9 / (12.0 * C.lmax))));
            for (int64_t p0 = 0; p0 < C.npoints; p0 += chunk) {
                SplitCatInput in;
                in.pts = C.points + 3 * p0;
                in.w = C.weights ? C.weights + p0 : nullptr;
                in.n = std::min(chunk, C.npoints - p0);
                in.lmax = C.lmax;
                in.nmax = C.nmax;
                in.rmax = C.rmax;
                in.kmax = C.kmax;
                in.kln_dev = C.k_ln;
                in.f_acc = facc[c];
                in.accurate = (flags & CATANA_SPLIT_ACCURATE) != 0;
                v.push_back(in);
            }
        }
        s = split_run(ctx, v, !(flags & CATANA_BATCH_NO_GRAPH), waves, (flags & CATANA_BATCH_MBLK64) ? 64 : 128,
                      err_d, st);
        if (s != CATANA_OK) return s;
    } else {
        for (int c = 0; c < ncat; ++c) {
            const catana_catalog_t &C = cats[c];
            s = fp64_raw_accumulate(ctx, C.points, C.weights, C.npoints, C.lmax, C.nmax,
                                    resolve_jl(flags, C.npoints), C.k_ln, facc[c], err_d, st);
            if (s != CATANA_OK) return s;
            if (C.kmax > 0.0 && C.lmax > 0 && C.nmax > 0) {
                k_kcut<<<dim3(ceil_div((int64_t)C.lmax * C.nmax, 256), C.lmax), 256, 0, st>>>(
                    reinterpret_cast<double2 *>(facc[c]), C.k_ln, C.nmax, C.kmax);
                count_launch();
                CG_CUDA_TRY(cudaGetLastError());
            }
        }
    }
    // weight sums (one read-back for all catalogs), then normalise and form C_ln
    std::vector<double> wsum(ncat);
    bool any_w = false;
    for (int c = 0; c < ncat; ++c) {
        wsum[c] = (double)cats[c].npoints;
        any_w |= (cats[c].weights && cats[c].npoints > 0);
    }
    if (any_w) {
        CG_CUDA_TRY(ctx->cat_scratch.ensure((size_t)8 * ncat));
        double *ws = ctx->cat_scratch.as<double>();
        for (int c = 0; c < ncat; ++c)
            if (cats[c].weights && cats[c].npoints > 0) {
                k_wsum<<<1, 1024, 0, st>>>(cats[c].weights, cats[c].npoints, ws + c);
                count_launch();
            }
        CG_CUDA_TRY(cudaGetLastError());
        std::vector<double> wh(ncat);
        CG_CUDA_TRY(cudaMemcpyAsync(wh.data(), ws, (size_t)8 * ncat, cudaMemcpyDeviceToHost, st));
        CG_CUDA_TRY(cudaStreamSynchronize(st));
        for (int c = 0; c < ncat; ++c)
            if (cats[c].weights && cats[c].npoints > 0) wsum[c] = wh[c];
    }
    for (int c = 0; c < ncat; ++c) {
        const catana_catalog_t &C = cats[c];
        s = finish_flmn_cln(facc[c], norm_factor(C.rmax, wsum[c]), C.lmax, C.nmax, C.c_ln, st);
        if (s != CATANA_OK) return s;
    }
    return CATANA_OK;
}

}  // namespace

extern "C" {

size_t catana_gpu_flmn_size(uint16_t lmax, uint16_t nmax) {
    return (size_t)nmax * (size_t)lmax * ((size_t)lmax + 1) / 2;
}

const char *catana_gpu_last_error(void) { return t_last_error.c_str(); }

uint64_t catana_gpu_launch_count(void) { return g_launches.load(); }

void catana_gpu_profile_enable(int enable) { g_prof_on.store(enable ? 1 : 0); }

catana_status_t catana_gpu_profile_report(double *kernel_ms, uint64_t *launches, double *algo_flops) {
    std::lock_guard<std::mutex> g(g_prof_mu);
    double ms = 0.0, fl = 0.0;
    uint64_t n = 0;
    for (auto &r : g_prof) {
        if (!r.b) continue;
        cudaError_t e = cudaEventSynchronize(r.b);
        if (e != cudaSuccess) {
            set_error(std::string("cudaEventSynchronize: ") + cudaGetErrorString(e));
            return CATANA_ERR_CUDA;
        }
        float t = 0.f;
        cudaEventElapsedTime(&t, r.a, r.b);
        ms += t;
        fl += r.flops;
        ++n;
    }
    for (auto &r : g_prof) {
        g_prof_free.push_back(r.a);
        if (r.b) g_prof_free.push_back(r.b);
    }
    g_prof.clear();
    if (kernel_ms) *kernel_ms = ms;
    if (launches) *launches = n;
    if (algo_flops) *algo_flops = fl;
    return CATANA_OK;
}

catana_status_t catana_gpu_fp64_peak(int32_t ms, double *tflops) {
    if (!tflops || ms < 1) {
        set_error("fp64_peak: ms >= 1 and a result pointer are required");
        return CATANA_ERR_ARG;
    }
    int cs;
    DeviceContext *ctx = get_context(&cs);
    if (!ctx) return (catana_status_t)cs;
    std::lock_guard<std::mutex> g(ctx->mu);
    CG_CUDA_TRY(ctx->misc.ensure(256));
    double *sink = reinterpret_cast<double *>(ctx->misc.as<char>() + 128);
    cudaStream_t st = nullptr;
    cudaEvent_t e0, e1;
    CG_CUDA_TRY(cudaEventCreate(&e0));
    CG_CUDA_TRY(cudaEventCreate(&e1));
    const int blocks = 8 * ctx->sm_count, threads = 256;
    auto timed = [&](int iters, float *msec) -> cudaError_t {
        cudaEventRecord(e0, st);
        k_fp64_fma_chains<<<blocks, threads, 0, st>>>(iters, 0.9999999999, 1e-10, sink);
        count_launch();
        cudaEventRecord(e1, st);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventElapsedTime(msec, e0, e1);
        return e;
    };
    float t = 0.f;
    cudaError_t e = timed(2000, &t);  // calibration (and warm-up)
    double best = 0.0;
    if (e == cudaSuccess) {
        const int iters = std::max(2000, (int)(2000.0 * (ms / 3.0) / std::max(1e-3, (double)t)));
        for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
            e = timed(iters, &t);
            const double fl = 2.0 * 8.0 * (double)iters * blocks * threads;
            if (e == cudaSuccess && t > 0.f) best = std::max(best, fl / (t * 1e-3) / 1e12);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CG_CUDA_TRY(e);
    *tflops = best;
    return CATANA_OK;
}

catana_status_t catana_gpu_sbessel_zeros(uint32_t l, int32_t count, double *out) {
    if (count < 0 || !out) {
        set_error("count must be >= 0 and out non-null");
        return CATANA_ERR_ARG;
    }
    if (count == 0) return CATANA_OK;
    const double *z = zeros_for(l, std::max(count, 2));
    memcpy(out, z, sizeof(double) * count);
    return CATANA_OK;
}

catana_status_t catana_gpu_compute_kln(uint16_t lmax, uint16_t nmax, double rmax, double *k_ln) {
    if (!k_ln && (size_t)lmax * nmax) {
        set_error("k_ln must be non-null");
        return CATANA_ERR_ARG;
    }
    kln_table(lmax, nmax, rmax, k_ln);
    return CATANA_OK;
}

catana_status_t catana_gpu_sfb_raw_dev(const double *points_dev, const double *weights_dev, int64_t npoints,
                                       uint16_t lmax, uint16_t nmax, double rmax, uint32_t flags,
                                       double *k_ln_dev, double *c_ln_dev, double *f_lmn_dev, int *status_dev,
                                       catana_gpu_stream_t stream) {
    catana_status_t s = check_args(npoints, lmax, nmax, rmax);
    if (s != CATANA_OK) return s;
    int cs;
    DeviceContext *ctx = get_context(&cs);
    if (!ctx) return (catana_status_t)cs;
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    int *err_d = status_dev;
    if (!err_d) {
        CG_CUDA_TRY(ctx->misc.ensure(256));
        err_d = ctx->misc.as<int>();
        CG_CUDA_TRY(cudaMemsetAsync(err_d, 0, sizeof(int), st));
    }
    return raw_device(ctx, points_dev, weights_dev, npoints, lmax, nmax, rmax, flags, k_ln_dev, c_ln_dev, f_lmn_dev,
                      err_d, st);
}

catana_status_t catana_gpu_sfb_raw(const double *points, const double *weights, int64_t npoints, uint16_t lmax,
                                   uint16_t nmax, double rmax, uint32_t flags, double *k_ln, double *c_ln,
                                   double *f_lmn, catana_gpu_stream_t stream) {
    catana_status_t s = check_args(npoints, lmax, nmax, rmax);
    if (s != CATANA_OK) return s;
    if ((npoints > 0 && !points) || ((size_t)lmax * nmax && (!k_ln || !c_ln))) {
        set_error("null buffer");
        return CATANA_ERR_ARG;
    }
    int cs;
    DeviceContext *ctx = get_context(&cs);
    if (!ctx) return (catana_status_t)cs;
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const size_t lm = (size_t)lmax * nmax;
    const size_t fc = catana_gpu_flmn_size(lmax, nmax);
    const size_t in_bytes = (size_t)npoints * 3 * sizeof(double) + (weights ? (size_t)npoints * sizeof(double) : 0);
    CG_CUDA_TRY(ctx->io_points.ensure(in_bytes + 256));
    CG_CUDA_TRY(ctx->io_out.ensure((2 * lm + 2 * fc) * sizeof(double) + 256));
    CG_CUDA_TRY(ctx->misc.ensure(256));
    double *pts_d = ctx->io_points.as<double>();
    double *w_d = weights ? pts_d + (size_t)npoints * 3 : nullptr;
    double *kln_d = ctx->io_out.as<double>();
    double *cln_d = kln_d + lm;
    double *f_d = cln_d + lm;
    int *err_d = ctx->misc.as<int>();
    CG_CUDA_TRY(cudaMemsetAsync(err_d, 0, sizeof(int), st));
    if (npoints > 0)
        CG_CUDA_TRY(cudaMemcpyAsync(pts_d, points, (size_t)npoints * 3 * sizeof(double), cudaMemcpyHostToDevice, st));
    if (weights && npoints > 0)
        CG_CUDA_TRY(cudaMemcpyAsync(w_d, weights, (size_t)npoints * sizeof(double), cudaMemcpyHostToDevice, st));
    s = raw_device(ctx, pts_d, w_d, npoints, lmax, nmax, rmax, flags, kln_d, cln_d, f_d, err_d, st);
    if (s != CATANA_OK) return s;
    int err_h = 0;
    CG_CUDA_TRY(cudaMemcpyAsync(&err_h, err_d, sizeof(int), cudaMemcpyDeviceToHost, st));
    CG_CUDA_TRY(cudaMemcpyAsync(k_ln, kln_d, lm * sizeof(double), cudaMemcpyDeviceToHost, st));
    CG_CUDA_TRY(cudaMemcpyAsync(c_ln, cln_d, lm * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (f_lmn) CG_CUDA_TRY(cudaMemcpyAsync(f_lmn, f_d, fc * 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    CG_CUDA_TRY(cudaStreamSynchronize(st));
    if (err_h == CATANA_ERR_DOMAIN) {
        set_error("argument (z) outside of defined range.");
        return CATANA_ERR_DOMAIN;
    }
    if (err_h != 0) {
        set_error("split kernel reported a timed-out wait");
        return CATANA_ERR_CUDA;
    }
    return CATANA_OK;
}

catana_status_t catana_gpu_sfb_raw_batched_dev(const catana_catalog_t *cats, int32_t ncat, uint32_t flags,
                                               double waves, int *status_dev, catana_gpu_stream_t stream) {
    catana_status_t s = check_catalogs(cats, ncat);
    if (s != CATANA_OK || ncat == 0) return s;
    int cs;
    DeviceContext *ctx = get_context(&cs);
    if (!ctx) return (catana_status_t)cs;
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    int *err_d = status_dev;
    if (!err_d) {
        CG_CUDA_TRY(ctx->misc.ensure(256));
        err_d = ctx->misc.as<int>();
        CG_CUDA_TRY(cudaMemsetAsync(err_d, 0, sizeof(int), st));
    }
    return batched_device(ctx, cats, ncat, flags, waves, err_d, st);
}

catana_status_t catana_gpu_sfb_raw_batched(const catana_catalog_t *cats, int32_t ncat, uint32_t flags, double waves,
                                           catana_gpu_stream_t stream) {
    catana_status_t s = check_catalogs(cats, ncat);
    if (s != CATANA_OK || ncat == 0) return s;
    int cs;
    DeviceContext *ctx = get_context(&cs);
    if (!ctx) return (catana_status_t)cs;
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    // staging: inputs packed into io_points, outputs into io_out (256-byte aligned pieces)
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    size_t in_bytes = 0, out_bytes = 0;
    for (int c = 0; c < ncat; ++c) {
        const catana_catalog_t &C = cats[c];
        in_bytes += al((size_t)C.npoints * 3 * sizeof(double)) + (C.weights ? al((size_t)C.npoints * sizeof(double)) : 0);
        const size_t lm = (size_t)C.lmax * C.nmax;
        out_bytes += 2 * al(lm * sizeof(double)) + al(catana_gpu_flmn_size(C.lmax, C.nmax) * 2 * sizeof(double));
    }
    CG_CUDA_TRY(ctx->io_points.ensure(in_bytes + 256));
    CG_CUDA_TRY(ctx->io_out.ensure(out_bytes + 256));
    CG_CUDA_TRY(ctx->misc.ensure(256));
    int *err_d = ctx->misc.as<int>();
    CG_CUDA_TRY(cudaMemsetAsync(err_d, 0, sizeof(int), st));
    std::vector<catana_catalog_t> dc(cats, cats + ncat);
    char *ip = ctx->io_points.as<char>(), *op = ctx->io_out.as<char>();
    for (int c = 0; c < ncat; ++c) {
        const catana_catalog_t &C = cats[c];
        const size_t pb = (size_t)C.npoints * 3 * sizeof(double), wb = (size_t)C.npoints * sizeof(double);
        dc[c].points = reinterpret_cast<const double *>(ip);
        if (pb) CG_CUDA_TRY(cudaMemcpyAsync(ip, C.points, pb, cudaMemcpyHostToDevice, st));
        ip += al(pb);
        if (C.weights) {
            dc[c].weights = reinterpret_cast<const double *>(ip);
            if (wb) CG_CUDA_TRY(cudaMemcpyAsync(ip, C.weights, wb, cudaMemcpyHostToDevice, st));
            ip += al(wb);
        }
        const size_t lmb = (size_t)C.lmax * C.nmax * sizeof(double);
        dc[c].k_ln = reinterpret_cast<double *>(op);
        op += al(lmb);
        dc[c].c_ln = reinterpret_cast<double *>(op);
        op += al(lmb);
        dc[c].f_lmn = reinterpret_cast<double *>(op);
        op += al(catana_gpu_flmn_size(C.lmax, C.nmax) * 2 * sizeof(double));
    }
    s = batched_device(ctx, dc.data(), ncat, flags, waves, err_d, st);
    if (s != CATANA_OK) return s;
    int err_h = 0;
    CG_CUDA_TRY(cudaMemcpyAsync(&err_h, err_d, sizeof(int), cudaMemcpyDeviceToHost, st));
    for (int c = 0; c < ncat; ++c) {
        const catana_catalog_t &C = cats[c];
        const size_t lmb = (size_t)C.lmax * C.nmax * sizeof(double);
        if (lmb) {
            CG_CUDA_TRY(cudaMemcpyAsync(C.k_ln, dc[c].k_ln, lmb, cudaMemcpyDeviceToHost, st));
            CG_CUDA_TRY(cudaMemcpyAsync(C.c_ln, dc[c].c_ln, lmb, cudaMemcpyDeviceToHost, st));
        }
        if (C.f_lmn && lmb)
            CG_CUDA_TRY(cudaMemcpyAsync(C.f_lmn, dc[c].f_lmn, catana_gpu_flmn_size(C.lmax, C.nmax) * 2 * sizeof(double),
                                        cudaMemcpyDeviceToHost, st));
    }
    CG_CUDA_TRY(cudaStreamSynchronize(st));
    if (err_h == CATANA_ERR_DOMAIN) {
        set_error("argument (z) outside of defined range.");
        return CATANA_ERR_DOMAIN;
    }
    if (err_h != 0) {
        set_error("split kernel reported a timed-out wait");
        return CATANA_ERR_CUDA;
    }
    return CATANA_OK;
}

double catana_gpu_batch_waves(void) {
    int cs;
    DeviceContext *ctx = get_context(&cs);
    return ctx ? ctx->split_last_waves : 0.0;
}

int32_t catana_gpu_batch_mblk(void) {
    int cs;
    DeviceContext *ctx = get_context(&cs);
    return ctx ? ctx->split_last_mblk : 0;
}

catana_status_t catana_gpu_ang2pix_ring(int64_t nside, const double *theta, const double *phi, int64_t n, int64_t *pix,
                                        catana_gpu_stream_t stream) {
    if (nside < 1 || (nside & (nside - 1)) != 0) {
        set_error("argument (nside) must be a power of 2");
        return CATANA_ERR_ARG;
    }
    if (n < 0 || (n > 0 && (!theta || !phi || !pix))) {
        set_error("invalid buffers");
        return CATANA_ERR_ARG;
    }
    if (n == 0) return CATANA_OK;
    int cs;
    DeviceContext *ctx = get_context(&cs);
    if (!ctx) return (catana_status_t)cs;
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    CG_CUDA_TRY(ctx->hp_ws.ensure((size_t)n * 3 * sizeof(double) + 256));
    double *th_d = ctx->hp_ws.as<double>();
    double *ph_d = th_d + n;
    int64_t *pix_d = reinterpret_cast<int64_t *>(ph_d + n);
    CG_CUDA_TRY(ctx->misc.ensure(256));
    int *err_d = ctx->misc.as<int>();
    CG_CUDA_TRY(cudaMemsetAsync(err_d, 0, sizeof(int), st));
    CG_CUDA_TRY(cudaMemcpyAsync(th_d, theta, n * sizeof(double), cudaMemcpyHostToDevice, st));
    CG_CUDA_TRY(cudaMemcpyAsync(ph_d, phi, n * sizeof(double), cudaMemcpyHostToDevice, st));
    catana_status_t s = healpix_ang2pix_dev(nside, th_d, ph_d, n, pix_d, err_d, st);
    if (s != CATANA_OK) return s;
    int err_h = 0;
    CG_CUDA_TRY(cudaMemcpyAsync(pix, pix_d, n * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CG_CUDA_TRY(cudaMemcpyAsync(&err_h, err_d, sizeof(int), cudaMemcpyDeviceToHost, st));
    CG_CUDA_TRY(cudaStreamSynchronize(st));
    if (err_h) {
        set_error("invalid theta value");
        return CATANA_ERR_ARG;
    }
    return CATANA_OK;
}

catana_status_t catana_gpu_pix2ang_ring(int64_t nside, const int64_t *pix, int64_t n, double *theta, double *phi,
                                        catana_gpu_stream_t stream) {
    if (nside < 1 || (nside & (nside - 1)) != 0) {
        set_error("argument (nside) must be a power of 2");
        return CATANA_ERR_ARG;
    }
    if (n < 0 || (n > 0 && (!theta || !phi || !pix))) {
        set_error("invalid buffers");
        return CATANA_ERR_ARG;
    }
    const int64_t npix = 12 * nside * nside;
    for (int64_t i = 0; i < n; ++i)
        if (pix[i] < 0 || pix[i] >= npix) {
            set_error("pixel index out of range");
            return CATANA_ERR_ARG;
        }
    if (n == 0) return CATANA_OK;
    int cs;
    DeviceContext *ctx = get_context(&cs);
    if (!ctx) return (catana_status_t)cs;
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    CG_CUDA_TRY(ctx->hp_ws.ensure((size_t)n * 3 * sizeof(double) + 256));
    double *th_d = ctx->hp_ws.as<double>();
    double *ph_d = th_d + n;
    int64_t *pix_d = reinterpret_cast<int64_t *>(ph_d + n);
    CG_CUDA_TRY(cudaMemcpyAsync(pix_d, pix, n * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    catana_status_t s = healpix_pix2ang_dev(nside, pix_d, n, th_d, ph_d, st);
    if (s != CATANA_OK) return s;
    CG_CUDA_TRY(cudaMemcpyAsync(theta, th_d, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    CG_CUDA_TRY(cudaMemcpyAsync(phi, ph_d, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    CG_CUDA_TRY(cudaStreamSynchronize(st));
    return CATANA_OK;
}

catana_status_t catana_gpu_sfb_reverse(int64_t nside, const int64_t *pix_offsets, const double *r_sorted,
                                       uint16_t lmax, uint16_t nmax, double rmax, uint32_t flags, double *k_ln,
                                       double *c_ln, double *f_lmn, catana_gpu_stream_t stream) {
    // _sfb_reverse's dense sum over pixels, f(m, n) = sum_pix Y_lm(pix) map(pix, n), splits
    // over rings: a ring's pixels share theta and have equally spaced phi, so its part is
    // P_lm(theta_ring) e^{-i m phi_0} times the ring DFT of the map at m mod rpix -- read as
    // the conjugate of F[rpix - m mod rpix] past rpix/2 (the corrected alias).
    return catana_gpu_sfb_healpix(nside, pix_offsets, r_sorted, lmax, nmax, rmax, flags | CATANA_HEALPIX_CONJ_FIX,
                                  k_ln, c_ln, f_lmn, stream);
}

catana_status_t catana_gpu_bin_points(int64_t nside, const double *points, int64_t npoints, int64_t *pix_offsets,
                                      double *r_sorted, catana_gpu_stream_t stream) {
    if (nside < 1 || (nside & (nside - 1)) != 0) {
        set_error("argument (nside) must be a power of 2");  // PixelizedPointContainer.cpp:13-15
        return CATANA_ERR_ARG;
    }
    if (npoints < 0 || !pix_offsets || (npoints > 0 && (!points || !r_sorted))) {
        set_error("invalid buffers");
        return CATANA_ERR_ARG;
    }
    const int64_t npix = 12 * nside * nside;
    int cs;
    DeviceContext *ctx = get_context(&cs);
    if (!ctx) return (catana_status_t)cs;
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const size_t pbytes = (size_t)npoints * 3 * sizeof(double);
    const size_t obytes = (size_t)(npix + 1) * sizeof(int64_t);
    const size_t rbytes = (size_t)npoints * sizeof(double);
    CG_CUDA_TRY(ctx->io_points.ensure(pbytes + 256));
    CG_CUDA_TRY(ctx->io_out.ensure(obytes + rbytes + 256));
    CG_CUDA_TRY(ctx->misc.ensure(256));
    double *pts_d = ctx->io_points.as<double>();
    int64_t *off_d = ctx->io_out.as<int64_t>();
    double *rs_d = reinterpret_cast<double *>(off_d + npix + 1);
    int *err_d = ctx->misc.as<int>();
    CG_CUDA_TRY(cudaMemsetAsync(err_d, 0, sizeof(int), st));
    if (npoints > 0) CG_CUDA_TRY(cudaMemcpyAsync(pts_d, points, pbytes, cudaMemcpyHostToDevice, st));
    catana_status_t s = healpix_bin_dev(ctx, nside, pts_d, npoints, off_d, rs_d, err_d, st);
    if (s != CATANA_OK) return s;
    int err_h = 0;
    CG_CUDA_TRY(cudaMemcpyAsync(&err_h, err_d, sizeof(int), cudaMemcpyDeviceToHost, st));
    CG_CUDA_TRY(cudaMemcpyAsync(pix_offsets, off_d, obytes, cudaMemcpyDeviceToHost, st));
    if (npoints > 0) CG_CUDA_TRY(cudaMemcpyAsync(r_sorted, rs_d, rbytes, cudaMemcpyDeviceToHost, st));
    CG_CUDA_TRY(cudaStreamSynchronize(st));
    if (err_h) {
        set_error("invalid theta value");  // HEALPix asserts 0 <= theta <= pi
        return CATANA_ERR_ARG;
    }
    return CATANA_OK;
}

catana_status_t catana_gpu_sfb_healpix(int64_t nside, const int64_t *pix_offsets, const double *r_sorted,
                                       uint16_t lmax, uint16_t nmax, double rmax, uint32_t flags, double *k_ln,
                                       double *c_ln, double *f_lmn, catana_gpu_stream_t stream) {
    if (nside < 1 || (nside & (nside - 1)) != 0) {
        set_error("argument (nside) must be a power of 2");
        return CATANA_ERR_ARG;
    }
    if ((flags & CATANA_JL_MASK) == CATANA_JL_POLY) {
        set_error("the pixelized path takes the table or exact j_l, not CATANA_JL_POLY");
        return CATANA_ERR_ARG;
    }
    const int64_t npix = 12 * nside * nside;
    if (!pix_offsets || ((size_t)lmax * nmax && (!k_ln || !c_ln))) {
        set_error("null buffer");
        return CATANA_ERR_ARG;
    }
    const int64_t npoints = pix_offsets[npix];
    catana_status_t s = check_args(npoints, lmax, nmax, rmax);
    if (s != CATANA_OK) return s;
    if (pix_offsets[0] != 0) {
        set_error("pix_offsets[0] must be 0");
        return CATANA_ERR_ARG;
    }
    for (int64_t p = 0; p < npix; ++p)
        if (pix_offsets[p + 1] < pix_offsets[p]) {
            set_error("pix_offsets must be non-decreasing");
            return CATANA_ERR_ARG;
        }
    if (npoints > 0 && !r_sorted) {
        set_error("null r_sorted");
        return CATANA_ERR_ARG;
    }
    int cs;
    DeviceContext *ctx = get_context(&cs);
    if (!ctx) return (catana_status_t)cs;
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const size_t lm = (size_t)lmax * nmax;
    const size_t fc = catana_gpu_flmn_size(lmax, nmax);
    const size_t obytes = (size_t)(npix + 1) * sizeof(int64_t);
    CG_CUDA_TRY(ctx->io_points.ensure(obytes + (size_t)npoints * sizeof(double) + 256));
    CG_CUDA_TRY(ctx->io_out.ensure((2 * lm + 2 * fc) * sizeof(double) + 256));
    CG_CUDA_TRY(ctx->misc.ensure(256));
    int64_t *off_d = ctx->io_points.as<int64_t>();
    double *rs_d = reinterpret_cast<double *>(off_d + npix + 1);
    double *kln_d = ctx->io_out.as<double>();
    double *cln_d = kln_d + lm;
    double *f_d = cln_d + lm;
    int *err_d = ctx->misc.as<int>();
    CG_CUDA_TRY(cudaMemsetAsync(err_d, 0, sizeof(int), st));
    CG_CUDA_TRY(cudaMemcpyAsync(off_d, pix_offsets, obytes, cudaMemcpyHostToDevice, st));
    if (npoints > 0)
        CG_CUDA_TRY(cudaMemcpyAsync(rs_d, r_sorted, (size_t)npoints * sizeof(double), cudaMemcpyHostToDevice, st));
    std::vector<double> kh(lm);
    kln_table(lmax, nmax, rmax, kh.data());
    CG_CUDA_TRY(cudaMemcpyAsync(kln_d, kh.data(), lm * sizeof(double), cudaMemcpyHostToDevice, st));
    CG_CUDA_TRY(cudaMemsetAsync(f_d, 0, fc * 2 * sizeof(double), st));
    const double nf = norm_factor(rmax, (double)npoints);
    double r_lo = 0.0, r_hi = 0.0;  // range of the radii; r_lo NaN when any radius is NaN
    for (int64_t i = 0; i < npoints; ++i) {
        const double r = r_sorted[i];
        if (std::isnan(r)) {
            r_lo = NAN;
            break;
        }
        if (i == 0 || r < r_lo) r_lo = r;
        if (i == 0 || r > r_hi) r_hi = r;
    }
    s = healpix_sfb_dev(ctx, nside, off_d, rs_d, npoints, lmax, nmax, resolve_interp(flags, npoints),
                        (flags & CATANA_HEALPIX_CONJ_FIX) != 0, kln_d, kh.data(), r_lo, r_hi, nf, f_d, cln_d, err_d,
                        st);
    if (s != CATANA_OK) return s;
    int err_h = 0;
    CG_CUDA_TRY(cudaMemcpyAsync(&err_h, err_d, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (lm) {
        CG_CUDA_TRY(cudaMemcpyAsync(k_ln, kln_d, lm * sizeof(double), cudaMemcpyDeviceToHost, st));
        CG_CUDA_TRY(cudaMemcpyAsync(c_ln, cln_d, lm * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    if (f_lmn && fc) CG_CUDA_TRY(cudaMemcpyAsync(f_lmn, f_d, fc * 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    CG_CUDA_TRY(cudaStreamSynchronize(st));
    if (err_h == CATANA_ERR_DOMAIN) {
        set_error("argument (z) outside of defined range.");
        return CATANA_ERR_DOMAIN;
    }
    return CATANA_OK;
}

}  // extern "C"
