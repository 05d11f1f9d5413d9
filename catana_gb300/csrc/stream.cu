// stream.cu -- chunked accumulation of one large catalog (no counterpart in the
// reference, whose FilterStream buffers a whole catalog in a PointContainer before
// sfb_decomposition runs, FilterStream.cpp:100-124).
//
// An accumulator owns the f_lmn sum of one decomposition on the device.  Each added
// chunk of points (float32 SphericalRecord-style (r, theta, phi) records, as
// RawBinarySource reads them, or float64) is copied from host memory into one of two
// device staging slots on the accumulator's copy stream and decomposed on its compute
// stream; a chunk's copy waits only for the compute that last used its slot, so the
// copy of chunk k+1 runs while chunk k is being decomposed (pinned host memory makes
// the copies asynchronous).  finish() normalises with the total point count (or
// weight sum) and forms C_ln exactly as the one-shot call does.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"

namespace catana_gpu {

namespace {

__global__ void k_f32_to_f64(const float *__restrict__ in, double *__restrict__ out, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (double)in[i];
}

}  // namespace

struct Accum {
    DeviceContext *ctx = nullptr;
    int lmax = 0, nmax = 0;
    double rmax = 1.0;
    uint32_t flags = 0;
    bool split = false;
    DevBuf kln, facc, err;
    DevBuf slot[2], slot64[2];
    cudaStream_t copy_st = nullptr, comp_st = nullptr;
    cudaEvent_t copied[2] = {nullptr, nullptr}, consumed[2] = {nullptr, nullptr};
    int next = 0;
    int64_t npoints = 0;
    double wsum = 0.0;
    bool weighted = false, unweighted = false;
    bool finished = false;
    ~Accum() {
        kln.release();
        facc.release();
        err.release();
        for (int k = 0; k < 2; ++k) {
            slot[k].release();
            slot64[k].release();
        }
        for (int k = 0; k < 2; ++k) {
            if (copied[k]) cudaEventDestroy(copied[k]);
            if (consumed[k]) cudaEventDestroy(consumed[k]);
        }
        if (copy_st) cudaStreamDestroy(copy_st);
        if (comp_st) cudaStreamDestroy(comp_st);
    }
};

namespace {

// one chunk: stage it in slot `k`, then decompose it on the compute stream
template <typename T>
catana_status_t accum_add(Accum *A, const T *points, const T *weights, int64_t n) {
    if (n < 0 || (n > 0 && !points)) {
        set_error("n must be >= 0 and points non-null");
        return CATANA_ERR_ARG;
    }
    if (A->finished) {
        set_error("the accumulation is finished");
        return CATANA_ERR_ARG;
    }
    if (n == 0) return CATANA_OK;
    if ((weights && A->unweighted) || (!weights && A->weighted)) {
        set_error("all chunks of an accumulation must either carry weights or not");
        return CATANA_ERR_ARG;
    }
    (weights ? A->weighted : A->unweighted) = true;
    // extents and weight sum on the host (the chunk is in host memory already)
    double max_r = 0.0, max_w = weights ? 0.0 : 1.0, ws = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        const double r = (double)points[3 * i];
        if (!(r >= 0.0) || !std::isfinite(r)) {
            set_error("argument (z) outside of defined range.");
            return CATANA_ERR_DOMAIN;
        }
        if (r > max_r) max_r = r;
        if (weights) {
            const double w = (double)weights[i];
            ws += w;
            if (std::fabs(w) > max_w) max_w = std::fabs(w);
        }
    }
    DeviceContext *ctx = A->ctx;
    std::lock_guard<std::mutex> g(ctx->mu);
    const int k = A->next;
    A->next ^= 1;
    const size_t pb = (size_t)n * 3 * sizeof(T), wb = weights ? (size_t)n * sizeof(T) : 0;
    // the slot's previous chunk must be consumed before it is overwritten (and before
    // a reallocation frees it)
    CG_CUDA_TRY(cudaEventSynchronize(A->consumed[k]));
    CG_CUDA_TRY(A->slot[k].ensure(pb + wb + 256));
    char *dst = A->slot[k].as<char>();
    CG_CUDA_TRY(cudaMemcpyAsync(dst, points, pb, cudaMemcpyHostToDevice, A->copy_st));
    if (weights) CG_CUDA_TRY(cudaMemcpyAsync(dst + ((pb + 255) & ~size_t(255)), weights, wb, cudaMemcpyHostToDevice, A->copy_st));
    CG_CUDA_TRY(cudaEventRecord(A->copied[k], A->copy_st));
    CG_CUDA_TRY(cudaStreamWaitEvent(A->comp_st, A->copied[k], 0));
    const T *pd = reinterpret_cast<const T *>(dst);
    const T *wd = weights ? reinterpret_cast<const T *>(dst + ((pb + 255) & ~size_t(255))) : nullptr;
    int *err_d = A->err.as<int>();
    catana_status_t s = CATANA_OK;
    if (A->split) {
        if (ctx->cc_major != 10 || ctx->cc_minor != 3) {
            set_error("the split (tcgen05) form needs an sm_103 device");
            return CATANA_ERR_UNSUPPORTED;
        }
        // pieces whose Legendre rows stay under ~24 GB (they share f: run one after another)
        const int64_t piece =
            std::max<int64_t>(32, std::min<int64_t>(n, (int64_t)(24e9 / ((A->lmax > 256 ? 15.0 : 12.0) * A->lmax))));
        std::vector<SplitCatInput> v;
        for (int64_t p0 = 0; p0 < n; p0 += piece) {
            SplitCatInput in;
            if (sizeof(T) == 4) {
                in.pts32 = reinterpret_cast<const float *>(pd) + 3 * p0;
                in.w32 = wd ? reinterpret_cast<const float *>(wd) + p0 : nullptr;
            } else {
                in.pts = reinterpret_cast<const double *>(pd) + 3 * p0;
                in.w = wd ? reinterpret_cast<const double *>(wd) + p0 : nullptr;
            }
            in.n = std::min(piece, n - p0);
            in.lmax = A->lmax;
            in.nmax = A->nmax;
            in.rmax = A->rmax;
            in.max_r = max_r;
            in.max_w = max_w;
            in.kln_dev = A->kln.as<double>();
            in.f_acc = A->facc.as<double>();
            in.accurate = (A->flags & CATANA_SPLIT_ACCURATE) != 0;
            v.push_back(in);
        }
        s = split_run(ctx, v, false, 1.0, 128, err_d, A->comp_st);
    } else {
        const double *p64 = reinterpret_cast<const double *>(pd), *w64 = reinterpret_cast<const double *>(wd);
        if (sizeof(T) == 4) {  // the FP64 path reads float64 records
            CG_CUDA_TRY(A->slot64[k].ensure((size_t)n * 4 * sizeof(double) + 256));
            double *c = A->slot64[k].as<double>();
            k_f32_to_f64<<<ceil_div(3 * n, 256), 256, 0, A->comp_st>>>(reinterpret_cast<const float *>(pd), c, 3 * n);
            count_launch();
            if (wd) {
                k_f32_to_f64<<<ceil_div(n, 256), 256, 0, A->comp_st>>>(reinterpret_cast<const float *>(wd), c + 3 * n,
                                                                       n);
                count_launch();
            }
            CG_CUDA_TRY(cudaGetLastError());
            p64 = c;
            w64 = wd ? c + 3 * n : nullptr;
        }
        // the reference's j_l rule applies to the whole catalog, not to a chunk:
        // JL_AUTO picks the table form here (streamed catalogs are large)
        const uint32_t jl = A->flags & CATANA_JL_MASK;
        const JlMode mode = jl == CATANA_JL_POLY ? JL_MODE_POLY : jl == CATANA_JL_EXACT ? JL_MODE_EXACT : JL_MODE_LERP;
        s = fp64_raw_accumulate(ctx, p64, w64, n, A->lmax, A->nmax, mode, A->kln.as<double>(),
                                A->facc.as<double>(), err_d, A->comp_st);
    }
    if (s != CATANA_OK) return s;
    CG_CUDA_TRY(cudaEventRecord(A->consumed[k], A->comp_st));
    A->npoints += n;
    A->wsum += ws;
    return CATANA_OK;
}

// one chunk of raw records: stage in slot `k`, convert + filter + compact into slot64[k],
// decompose the kept points
catana_status_t accum_add_records(Accum *A, const void *records, int64_t n, const catana_ingest_t &spec) {
    if (n < 0 || (n > 0 && !records)) {
        set_error("n must be >= 0 and records non-null");
        return CATANA_ERR_ARG;
    }
    if (A->finished) {
        set_error("the accumulation is finished");
        return CATANA_ERR_ARG;
    }
    if (A->weighted) {
        set_error("all chunks of an accumulation must either carry weights or not");
        return CATANA_ERR_ARG;
    }
    if (n == 0) return CATANA_OK;
    A->unweighted = true;
    DeviceContext *ctx = A->ctx;
    std::lock_guard<std::mutex> g(ctx->mu);
    const int k = A->next;
    A->next ^= 1;
    const size_t rb = (size_t)n * 3 * ((spec.layout & CATANA_REC_FLOAT32) ? 4 : 8);
    CG_CUDA_TRY(cudaEventSynchronize(A->consumed[k]));
    CG_CUDA_TRY(A->slot[k].ensure(rb + 256));
    CG_CUDA_TRY(A->slot64[k].ensure((size_t)n * 3 * sizeof(double) + 256));
    CG_CUDA_TRY(cudaMemcpyAsync(A->slot[k].ptr, records, rb, cudaMemcpyHostToDevice, A->copy_st));
    CG_CUDA_TRY(cudaEventRecord(A->copied[k], A->copy_st));
    CG_CUDA_TRY(cudaStreamWaitEvent(A->comp_st, A->copied[k], 0));
    int64_t kept = 0;
    double *pts = A->slot64[k].as<double>();
    catana_status_t s = ingest_dev(ctx, A->slot[k].ptr, n, spec, pts, &kept, A->comp_st);
    if (s != CATANA_OK) return s;
    int *err_d = A->err.as<int>();
    if (kept > 0) {
        if (A->split) {
            if (ctx->cc_major != 10 || ctx->cc_minor != 3) {
                set_error("the split (tcgen05) form needs an sm_103 device");
                return CATANA_ERR_UNSUPPORTED;
            }
            const int64_t piece = std::max<int64_t>(
                32, std::min<int64_t>(kept, (int64_t)(24e9 / ((A->lmax > 256 ? 15.0 : 12.0) * A->lmax))));
            std::vector<SplitCatInput> v;
            for (int64_t p0 = 0; p0 < kept; p0 += piece) {
                SplitCatInput in;
                in.pts = pts + 3 * p0;
                in.n = std::min(piece, kept - p0);
                in.lmax = A->lmax;
                in.nmax = A->nmax;
                in.rmax = A->rmax;
                in.kln_dev = A->kln.as<double>();
                in.f_acc = A->facc.as<double>();
                in.accurate = (A->flags & CATANA_SPLIT_ACCURATE) != 0;
                v.push_back(in);
            }
            s = split_run(ctx, v, false, 1.0, 128, err_d, A->comp_st);
        } else {
            const uint32_t jl = A->flags & CATANA_JL_MASK;
            const JlMode mode =
                jl == CATANA_JL_POLY ? JL_MODE_POLY : jl == CATANA_JL_EXACT ? JL_MODE_EXACT : JL_MODE_LERP;
            s = fp64_raw_accumulate(ctx, pts, nullptr, kept, A->lmax, A->nmax, mode,
                                    A->kln.as<double>(), A->facc.as<double>(), err_d, A->comp_st);
        }
        if (s != CATANA_OK) return s;
    }
    CG_CUDA_TRY(cudaEventRecord(A->consumed[k], A->comp_st));
    A->npoints += kept;
    return CATANA_OK;
}

}  // namespace

}  // namespace catana_gpu

using namespace catana_gpu;

extern "C" {

catana_status_t catana_gpu_accum_create(uint16_t lmax, uint16_t nmax, double rmax, uint32_t flags,
                                        catana_gpu_accum_t *out) {
    if (!out) {
        set_error("out must be non-null");
        return CATANA_ERR_ARG;
    }
    *out = nullptr;
    if (!(rmax > 0.0) || !std::isfinite(rmax)) {
        set_error("rmax must be positive and finite");
        return CATANA_ERR_ARG;
    }
    int cs;
    DeviceContext *ctx = get_context(&cs);
    if (!ctx) return (catana_status_t)cs;
    Accum *A = new Accum();
    A->ctx = ctx;
    A->lmax = lmax;
    A->nmax = nmax;
    A->rmax = rmax;
    A->flags = flags;
    A->split = (flags & CATANA_FORM_MASK) == CATANA_FORM_SPLIT;
    auto fail = [&](cudaError_t e, const char *what) {
        set_error(std::string(what) + ": " + cudaGetErrorString(e));
        delete A;
        return CATANA_ERR_CUDA;
    };
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&A->copy_st, cudaStreamNonBlocking)) != cudaSuccess) return fail(e, "stream");
    if ((e = cudaStreamCreateWithFlags(&A->comp_st, cudaStreamNonBlocking)) != cudaSuccess) return fail(e, "stream");
    for (int k = 0; k < 2; ++k) {
        if ((e = cudaEventCreateWithFlags(&A->copied[k], cudaEventDisableTiming)) != cudaSuccess) return fail(e, "event");
        if ((e = cudaEventCreateWithFlags(&A->consumed[k], cudaEventDisableTiming)) != cudaSuccess)
            return fail(e, "event");
    }
    const size_t lm = (size_t)lmax * nmax, fb = catana_gpu_flmn_size(lmax, nmax) * 2 * sizeof(double);
    std::vector<double> kh(lm);
    kln_table(lmax, nmax, rmax, kh.data());
    if ((e = A->kln.ensure(lm * sizeof(double) + 8)) != cudaSuccess) return fail(e, "cudaMalloc");
    if ((e = A->facc.ensure(fb + 16)) != cudaSuccess) return fail(e, "cudaMalloc");
    if ((e = A->err.ensure(256)) != cudaSuccess) return fail(e, "cudaMalloc");
    if (lm && (e = cudaMemcpyAsync(A->kln.ptr, kh.data(), lm * sizeof(double), cudaMemcpyHostToDevice, A->comp_st)) !=
                  cudaSuccess)
        return fail(e, "cudaMemcpyAsync");
    if ((e = cudaMemsetAsync(A->facc.ptr, 0, fb + 16, A->comp_st)) != cudaSuccess) return fail(e, "cudaMemsetAsync");
    if ((e = cudaMemsetAsync(A->err.ptr, 0, 256, A->comp_st)) != cudaSuccess) return fail(e, "cudaMemsetAsync");
    if ((e = cudaStreamSynchronize(A->comp_st)) != cudaSuccess) return fail(e, "cudaStreamSynchronize");
    *out = reinterpret_cast<catana_gpu_accum_t>(A);
    return CATANA_OK;
}

catana_status_t catana_gpu_accum_add_f32(catana_gpu_accum_t acc, const float *points, const float *weights,
                                         int64_t n) {
    if (!acc) {
        set_error("null accumulator");
        return CATANA_ERR_ARG;
    }
    return accum_add<float>(reinterpret_cast<Accum *>(acc), points, weights, n);
}

catana_status_t catana_gpu_accum_add(catana_gpu_accum_t acc, const double *points, const double *weights,
                                     int64_t n) {
    if (!acc) {
        set_error("null accumulator");
        return CATANA_ERR_ARG;
    }
    return accum_add<double>(reinterpret_cast<Accum *>(acc), points, weights, n);
}

catana_status_t catana_gpu_accum_add_records(catana_gpu_accum_t acc, const void *records, int64_t n,
                                             const catana_ingest_t *spec) {
    if (!acc || !spec) {
        set_error("null accumulator or spec");
        return CATANA_ERR_ARG;
    }
    return accum_add_records(reinterpret_cast<Accum *>(acc), records, n, *spec);
}

catana_status_t catana_gpu_accum_add_file(catana_gpu_accum_t acc, const char *path, int64_t first_record,
                                          int64_t max_records, int64_t chunk_records, const catana_ingest_t *spec,
                                          int64_t *records_read) {
    // RawBinarySource (RawBinarySource.cpp:6-61): a file of consecutive fixed-size records
    // read in chunks; here a reader thread fills one of two pinned host buffers while the
    // previous chunk is copied, filtered and decomposed.
    if (records_read) *records_read = 0;
    if (!acc || !path || !spec || first_record < 0 || chunk_records <= 0) {
        set_error("add_file: null argument, negative first_record or non-positive chunk");
        return CATANA_ERR_ARG;
    }
    const size_t rsz = (size_t)3 * ((spec->layout & CATANA_REC_FLOAT32) ? 4 : 8);
    FILE *fp = std::fopen(path, "rb");
    if (!fp) {
        set_error(std::string("add_file: cannot open ") + path);
        return CATANA_ERR_ARG;
    }
    std::fseek(fp, 0, SEEK_END);
    const long long bytes = std::ftell(fp);
    int64_t ntot = bytes > 0 ? (int64_t)(bytes / (long long)rsz) : 0;  // trailing partial record ignored
    int64_t n = std::max<int64_t>(0, ntot - first_record);
    if (max_records >= 0) n = std::min(n, max_records);
    if (n == 0) {
        std::fclose(fp);
        return CATANA_OK;
    }
    std::fseek(fp, (long)((long long)first_record * (long long)rsz), SEEK_SET);
    const int64_t chunk = std::min(chunk_records, n);
    void *buf[2] = {nullptr, nullptr};
    for (int k = 0; k < 2; ++k)
        if (cudaHostAlloc(&buf[k], (size_t)chunk * rsz, cudaHostAllocDefault) != cudaSuccess) {
            if (buf[0]) cudaFreeHost(buf[0]);
            std::fclose(fp);
            set_error("add_file: cudaHostAlloc failed");
            return CATANA_ERR_NOMEM;
        }
    auto read_into = [&](int k, int64_t cnt) -> int64_t {
        return (int64_t)std::fread(buf[k], rsz, (size_t)cnt, fp);
    };
    catana_status_t s = CATANA_OK;
    int64_t done = 0, got = read_into(0, std::min(chunk, n));
    int cur = 0;
    while (got > 0 && s == CATANA_OK) {
        const int64_t todo = std::min(chunk, n - done - got);
        int64_t got_next = 0;
        std::thread reader;
        if (todo > 0) reader = std::thread([&, cur, todo]() { got_next = read_into(cur ^ 1, todo); });
        catana_ingest_t sp = *spec;
        sp.index0 = spec->index0 + (uint64_t)(first_record + done);
        s = accum_add_records(reinterpret_cast<Accum *>(acc), buf[cur], got, sp);
        if (reader.joinable()) reader.join();
        done += got;
        // the chunk in buf[cur] is read by the copy of the next add (pinned, asynchronous):
        // wait for the device to be done with it before it is refilled
        Accum *A = reinterpret_cast<Accum *>(acc);
        cudaStreamSynchronize(A->copy_st);
        got = got_next;
        cur ^= 1;
    }
    Accum *A = reinterpret_cast<Accum *>(acc);
    cudaStreamSynchronize(A->copy_st);
    cudaStreamSynchronize(A->comp_st);
    cudaFreeHost(buf[0]);
    cudaFreeHost(buf[1]);
    std::fclose(fp);
    if (records_read) *records_read = done;
    return s;
}

catana_status_t catana_gpu_accum_finish(catana_gpu_accum_t acc, double *k_ln, double *c_ln, double *f_lmn) {
    if (!acc) {
        set_error("null accumulator");
        return CATANA_ERR_ARG;
    }
    Accum *A = reinterpret_cast<Accum *>(acc);
    const size_t lm = (size_t)A->lmax * A->nmax;
    if (A->finished) {
        set_error("the accumulation is finished");
        return CATANA_ERR_ARG;
    }
    if (lm && (!k_ln || !c_ln)) {
        set_error("k_ln and c_ln must be non-null");
        return CATANA_ERR_ARG;
    }
    DeviceContext *ctx = A->ctx;
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaStream_t st = A->comp_st;
    const double wsum = A->weighted ? A->wsum : (double)A->npoints;
    // sqrt(2/pi) (4/3) pi rmax^3 / N (sfb_raw.cpp:29-30), N -> sum of weights
    const double nf = std::sqrt(2.0 / 3.14159265358979323846) * (4.0 / 3.0) * 3.14159265358979323846 * A->rmax *
                      A->rmax * A->rmax / wsum;
    CG_CUDA_TRY(ctx->io_out.ensure(lm * sizeof(double) + 256));
    double *cln_d = ctx->io_out.as<double>();
    catana_status_t s = finish_flmn_cln(A->facc.as<double>(), nf, A->lmax, A->nmax, cln_d, st);
    if (s != CATANA_OK) return s;
    A->finished = true;  // f is normalised in place
    int err_h = 0;
    CG_CUDA_TRY(cudaMemcpyAsync(&err_h, A->err.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (lm) {
        CG_CUDA_TRY(cudaMemcpyAsync(k_ln, A->kln.ptr, lm * sizeof(double), cudaMemcpyDeviceToHost, st));
        CG_CUDA_TRY(cudaMemcpyAsync(c_ln, cln_d, lm * sizeof(double), cudaMemcpyDeviceToHost, st));
        if (f_lmn)
            CG_CUDA_TRY(cudaMemcpyAsync(f_lmn, A->facc.ptr, catana_gpu_flmn_size(A->lmax, A->nmax) * 2 * sizeof(double),
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

catana_status_t catana_gpu_accum_destroy(catana_gpu_accum_t acc) {
    if (!acc) return CATANA_OK;
    Accum *A = reinterpret_cast<Accum *>(acc);
    cudaStreamSynchronize(A->comp_st);
    cudaStreamSynchronize(A->copy_st);
    delete A;
    return CATANA_OK;
}

}  // extern "C"
