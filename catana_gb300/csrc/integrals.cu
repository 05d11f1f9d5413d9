// integrals.cu -- batched double spherical-Bessel integrals (the shot-noise integrals
// of the SFB power spectrum):
//
//   I(k1, k2) = int_0^rmax w(r) j_l(k1 r) j_l(k2 r) dr      (sbessel_integrator.cpp:53-110)
//
// The reference integrates with GSL's adaptive Gauss-Kronrod (QAG, 21-point rule,
// epsrel 1e-7) over the sub-intervals between consecutive zeros of j_l(k1 r) and, inside
// each, of j_l(k2 r) (SBesselIntegrationRangeGenerator, :113-133), stopping once an outer
// interval adds less than 1e-10 of the total.  Here one warp integrates one (k1, k2) pair
// over the same breakpoints -- the merged zero sets z_{l,i}/k1 and z_{l,j}/k2 inside
// (0, rmax) -- plus the nodes of the w table, so that w is linear on every piece (w is a
// FunctionInterpolator table, FunctionInterpolator.cpp:6-30: linear on equally spaced
// nodes, domain error outside [x_min, x_max); its kinks would otherwise cost GL its
// accuracy).  Between consecutive zeros the warp spreads the table segments over its
// lanes with a Gauss-Legendre rule chosen by the segment length L: 2 points for
// k2 L <= 0.02, 4 for <= 0.1, 8 for <= 0.25, else 32 (error below 1e-10 of the
// segment's integral in every case); the whole range is summed.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <vector>

#include "common.cuh"
#include "special.cuh"

namespace catana_gpu {

namespace {


// GL rules packed in one array: 2 points at [0, 2), 4 at [2, 6), 8 at [6, 14), 32 at [14, 46)
constexpr int GL_OFF2 = 0, GL_OFF4 = 2, GL_OFF8 = 6, GL_OFF32 = 14, GL_TOT = 46;

__device__ __forceinline__ double dsb_w(const double *__restrict__ wt, int64_t wn, double wmin, double wdxinv,
                                        double x) {
    const double ia = (x - wmin) * wdxinv;  // FunctionInterpolator form; x may round onto wmax at the end
    unsigned ii = (unsigned)ia;
    if (ii > (unsigned)(wn - 2)) ii = (unsigned)(wn - 2);
    return wt[ii] + (wt[ii + 1] - wt[ii]) * (ia - ii);
}

__global__ void k_dsb_integrals(const double *__restrict__ zeros, int nz, const double *__restrict__ glx,
                                const double *__restrict__ glw, const double *__restrict__ wt, int64_t wn,
                                double wmin, double wmax, double wdx, double wdxinv, int l, double rmax,
                                const double *__restrict__ k1v, const double *__restrict__ k2v, int64_t np,
                                double *__restrict__ out, int *__restrict__ err) {
    const int64_t p = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (p >= np) return;  // warp-uniform
    double a = k1v[p], b = k2v[p];
    if (a > b) {
        const double t = a;
        a = b;
        b = t;
    }
    double acc = 0.0;
    int i1 = 0, i2 = 0;
    double lo = 0.0;
    const int bad = (wmin > 0.0 || rmax > wmax) ? 1 : 0;
    while (lo < rmax && !bad) {
        // the next zero of either factor: the Bessel product keeps its sign up to there
        const double z1 = (a > 0.0 && i1 < nz) ? zeros[i1] / a : INFINITY;
        const double z2 = (b > 0.0 && i2 < nz) ? zeros[i2] / b : INFINITY;
        const double hi = fmin(fmin(z1, z2), rmax);
        if (hi > lo) {
            // table nodes strictly inside (lo, hi) split it into segments on which w is linear
            int64_t ilo = (int64_t)floor((lo - wmin) * wdxinv) + 1;
            while (ilo > 0 && wmin + (double)(ilo - 1) * wdx > lo) --ilo;
            while (wmin + (double)ilo * wdx <= lo) ++ilo;
            int64_t ihi = ilo - 1;
            {
                int64_t c = (int64_t)ceil((hi - wmin) * wdxinv) - 1;
                while (c >= ilo && wmin + (double)c * wdx >= hi) --c;
                while (wmin + (double)(c + 1) * wdx < hi && c + 1 < wn) ++c;
                ihi = c;
            }
            const int64_t nseg = (ihi >= ilo) ? ihi - ilo + 2 : 1;
            const double seglen = (nseg > 1) ? wdx : (hi - lo);
            // rule per segment length (k2 len: <= 0.02 -> 2 points, 0.1 -> 4, 0.25 -> 8, else 32)
            const double kl = b * seglen;
            const int npg = kl <= 0.02 ? 2 : (kl <= 0.1 ? 4 : (kl <= 0.25 ? 8 : 32));
            const int goff = npg == 2 ? GL_OFF2 : (npg == 4 ? GL_OFF4 : (npg == 8 ? GL_OFF8 : GL_OFF32));
            const int per = 32 / npg;  // segments per warp pass
            const int j = lane % npg;
            const double xg = glx[goff + j], wg = glw[goff + j];
            for (int64_t s0 = 0; s0 < nseg; s0 += per) {
                const int64_t sgi = s0 + lane / npg;
                if (sgi < nseg) {
                    const double sa = (sgi == 0) ? lo : wmin + (double)(ilo + sgi - 1) * wdx;
                    const double sb = (sgi == nseg - 1) ? hi : wmin + (double)(ilo + sgi) * wdx;
                    const double half = 0.5 * (sb - sa);
                    const double x = sa + half * (xg + 1.0);
                    acc += wg * half * dsb_w(wt, wn, wmin, wdxinv, x) * sbessel_jl(l, a * x) * sbessel_jl(l, b * x);
                }
            }
        }
        if (z1 <= hi) ++i1;
        if (z2 <= hi) ++i2;
        if (hi >= rmax || (!(z1 <= hi) && !(z2 <= hi))) break;
        lo = hi;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
        out[p] = acc;
        if (bad) atomicOr(err, 1);
    }
}

// Gauss-Legendre nodes and weights on [-1, 1] (Newton on P_n from the asymptotic guesses
// cos(pi (i - 1/4) / (n + 1/2)); Abramowitz & Stegun 25.4.29)
void gauss_legendre(int n, double *x, double *w) {
    for (int i = 0; i < (n + 1) / 2; ++i) {
        double z = std::cos(kPi * (i + 0.75) / (n + 0.5)), pp = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p1 = 1.0, p2 = 0.0;
            for (int j = 1; j <= n; ++j) {
                const double p3 = p2;
                p2 = p1;
                p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
            }
            pp = n * (z * p1 - p2) / (z * z - 1.0);
            const double dz = p1 / pp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        x[i] = -z;
        x[n - 1 - i] = z;
        w[i] = w[n - 1 - i] = 2.0 / ((1.0 - z * z) * pp * pp);
    }
}

}  // namespace

}  // namespace catana_gpu

using namespace catana_gpu;

extern "C" {

catana_status_t catana_gpu_sbessel_integrals(const double *w_table, int64_t w_n, double w_min, double w_max,
                                             uint32_t l, double r_max, const double *k1, const double *k2,
                                             int64_t npairs, double *out, catana_gpu_stream_t stream) {
    if (!w_table || w_n < 2 || !(w_max > w_min) || !(r_max > 0.0) || !std::isfinite(r_max) || npairs < 0 ||
        (npairs > 0 && (!k1 || !k2 || !out))) {
        set_error("sbessel_integrals: need a w table of >= 2 nodes on w_min < w_max, r_max > 0, k1/k2/out");
        return CATANA_ERR_ARG;
    }
    if (npairs == 0) return CATANA_OK;
    double kmax = 0.0;
    for (int64_t i = 0; i < npairs; ++i) {
        if (!(k1[i] >= 0.0) || !(k2[i] >= 0.0) || !std::isfinite(k1[i]) || !std::isfinite(k2[i])) {
            set_error("sbessel_integrals: k1 and k2 must be >= 0 and finite");
            return CATANA_ERR_ARG;
        }
        kmax = std::max(kmax, std::max(k1[i], k2[i]));
    }
    // zeros of j_l up to kmax rmax (plus one beyond)
    int nz = 2;
    const double *z = zeros_for(l, nz);
    while (z[nz - 1] <= kmax * r_max) {
        nz *= 2;
        z = zeros_for(l, nz);
    }
    int cs;
    DeviceContext *ctx = get_context(&cs);
    if (!ctx) return (catana_status_t)cs;
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    std::vector<double> glx(GL_TOT), glw(GL_TOT);
    gauss_legendre(2, glx.data() + GL_OFF2, glw.data() + GL_OFF2);
    gauss_legendre(4, glx.data() + GL_OFF4, glw.data() + GL_OFF4);
    gauss_legendre(8, glx.data() + GL_OFF8, glw.data() + GL_OFF8);
    gauss_legendre(32, glx.data() + GL_OFF32, glw.data() + GL_OFF32);
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t zb = al((size_t)nz * 8), gb = al(2 * GL_TOT * 8), wb = al((size_t)w_n * 8), kb = al((size_t)npairs * 8);
    CG_CUDA_TRY(ctx->io_points.ensure(zb + gb + wb + 3 * kb + 256));
    char *d = ctx->io_points.as<char>();
    double *zd = reinterpret_cast<double *>(d), *gd = reinterpret_cast<double *>(d + zb),
           *wd = reinterpret_cast<double *>(d + zb + gb), *k1d = reinterpret_cast<double *>(d + zb + gb + wb),
           *k2d = reinterpret_cast<double *>(d + zb + gb + wb + kb),
           *od = reinterpret_cast<double *>(d + zb + gb + wb + 2 * kb);
    CG_CUDA_TRY(cudaMemcpyAsync(zd, z, (size_t)nz * 8, cudaMemcpyHostToDevice, st));
    CG_CUDA_TRY(cudaMemcpyAsync(gd, glx.data(), GL_TOT * 8, cudaMemcpyHostToDevice, st));
    CG_CUDA_TRY(cudaMemcpyAsync(gd + GL_TOT, glw.data(), GL_TOT * 8, cudaMemcpyHostToDevice, st));
    CG_CUDA_TRY(cudaMemcpyAsync(wd, w_table, (size_t)w_n * 8, cudaMemcpyHostToDevice, st));
    CG_CUDA_TRY(cudaMemcpyAsync(k1d, k1, (size_t)npairs * 8, cudaMemcpyHostToDevice, st));
    CG_CUDA_TRY(cudaMemcpyAsync(k2d, k2, (size_t)npairs * 8, cudaMemcpyHostToDevice, st));
    CG_CUDA_TRY(ctx->misc.ensure(256));
    int *err = reinterpret_cast<int *>(ctx->misc.as<char>() + 160);
    CG_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
    const double wdx = (w_max - w_min) / (double)(w_n - 1), wdxinv = 1.0 / wdx;
    const int64_t threads = npairs * 32;
    k_dsb_integrals<<<ceil_div(threads, 256), 256, 0, st>>>(zd, nz, gd, gd + GL_TOT, wd, w_n, w_min, w_max, wdx,
                                                            wdxinv, (int)l, r_max, k1d, k2d, npairs, od, err);
    count_launch();
    CG_CUDA_TRY(cudaGetLastError());
    int err_h = 0;
    CG_CUDA_TRY(cudaMemcpyAsync(out, od, (size_t)npairs * 8, cudaMemcpyDeviceToHost, st));
    CG_CUDA_TRY(cudaMemcpyAsync(&err_h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CG_CUDA_TRY(cudaStreamSynchronize(st));
    if (err_h) {
        set_error("argument outside range for which this FunctionInterpolator is defined");
        return CATANA_ERR_DOMAIN;
    }
    return CATANA_OK;
}

}  // extern "C"
