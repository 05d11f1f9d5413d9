// healpix.cu -- HEALPix RING binning and the pixelized SFB (FP64).
//
// Binning (PixelizedPointContainer.cpp:11-30): ang2pix per point (RING scheme, the
// published algorithm of Gorski et al. 2005, ApJ 622:759, sec. 4, evaluated in the
// same operation order as the CPU restatement with every product and sum rounded
// separately -- no FMA contraction -- so both give the same pixel), then a stable
// radix sort of (pixel, point index) and a histogram scan give CSR offsets; radii are
// gathered in point order within each pixel, as the reference's push_back does.
//
// SFB (sfb_reverse_fft.cpp:43-209), per multipole l:
//   k_hp_map    map[pix][n] = sum_{p in pix} j_l(k_ln r_p), points in order
//   k_hp_ylm    Y_lm(ring) = P_lm(cos theta_ring) e^{-i m phi_0(ring)} (phi_0: the ring's
//               first pixel centre, as the reference's RingInfo)
//   k_hp_ring   per ring: the real DFT F[s] = sum_j map_j e^{-2 pi i j s / rpix} at the
//               frequencies the m-extraction reads, s = rpix/2 - |rpix/2 - (m mod rpix)|;
//               the reference never conjugates (sign = (m > 0) scales only ... the sign
//               of the imaginary part, which is +1 for every m > 0), so for
//               m mod rpix > rpix/2 it uses F[rpix - m mod rpix] itself; the
//               CATANA_HEALPIX_CONJ_FIX flag conjugates it.  Times Y_lm(ring) -> per-ring
//               partial sums [ring][m][n]
//   k_hp_reduce sum over rings (interleaved per warp, fixed order);
//               C_ln = (2 sum_m |f|^2 - |f_0|^2) (norm k)^2 / (2l+1) and f stored as
//               f k norm (sfb_reverse_fft.cpp:147-153)
// The ring transform: rings whose length is a power of two (all equatorial rings when
// nside is one, and the polar rings of 4, 8, 16, ... pixels) take a batched FP64 FFT
// (k_hp_fft: two radial orders packed as one complex sequence, radix-4 passes in
// shared memory) once l is large enough that the FFT's N log N beats the direct sum;
// the other rings take a direct DFT of only the needed frequencies over the ring's
// quarter-orbits (N/4 + 1 folded terms per frequency, folded chunks and twiddles staged
// in shared memory).  Both end in the same m-extraction and per-ring partial sums.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "special.cuh"
#include "hpx_ring.cuh"

namespace catana_gpu {

namespace {

__global__ void k_ang2pix(int64_t nside, const double *theta, const double *phi, int64_t n, int64_t *pix, int *err) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t p = ang2pix_ring_dev(nside, theta[i], phi[i]);
    if (p < 0) *err = CATANA_ERR_ARG;
    pix[i] = p < 0 ? 0 : p;
}

__global__ void k_pix2ang(int64_t nside, const int64_t *pix, int64_t n, double *theta, double *phi) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    pix2ang_ring_dev(nside, pix[i], &theta[i], &phi[i]);
}

// keys = RING pixel of each point, vals = point index; counts[pix] += 1
__global__ void k_bin_keys(int64_t nside, const double *pts, int64_t n, uint32_t *keys, uint32_t *vals,
                           uint32_t *counts, int *err) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t p = ang2pix_ring_dev(nside, pts[3 * i + 1], pts[3 * i + 2]);
    if (p < 0) {
        *err = CATANA_ERR_ARG;
        p = 0;
    }
    keys[i] = (uint32_t)p;
    vals[i] = (uint32_t)i;
    atomicAdd(&counts[p], 1u);
}

__global__ void k_bin_gather(const double *pts, const uint32_t *perm, int64_t n, const uint32_t *offs32,
                             int64_t npix, double *r_sorted, int64_t *offs) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) r_sorted[i] = pts[3 * (int64_t)perm[i]];
    if (i <= npix) offs[i] = (i == npix) ? n : (int64_t)offs32[i];
}

// map[pix][n] = sum over the pixel's points (in order) of j_l(k_ln r).  CHECKED: every
// argument k r is tested against the table's range [0, zmax) (a domain error otherwise);
// unchecked launches are made only when the host has shown that the whole level lies in
// range (0 <= r_min and k_max r_max < zmax, the same FP64 product as here), and form the
// table position as r (k / dx) with kd[n] = k_ln / dx from the host -- one rounding away
// from (k r) / dx, a change of the interpolated value far below 1e-10 of the table's
// scale.
template <bool CHECKED>
__global__ void k_hp_map(const int64_t *__restrict__ offs, const double *__restrict__ r, int64_t npix, int nmax,
                         const double *__restrict__ kln, const double *__restrict__ kdl,
                         const double *__restrict__ tab, int npts_tab, double dx_inv, double zmax, int l,
                         double *__restrict__ map, int *err) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= npix * nmax) return;
    const int64_t pix = t / nmax;
    const int n = (int)(t - pix * nmax);
    const double k = kln[n];
    const double kd = CHECKED ? 0.0 : kdl[n];
    double s = 0.0;
    for (int64_t q = offs[pix]; q < offs[pix + 1]; ++q) {
        double j;
        if (tab) {
            double ia;
            if (CHECKED) {
                const double z = k * r[q];
                if (!(z >= 0.0) || z >= zmax) {
                    *err = CATANA_ERR_DOMAIN;
                    ia = 0.0;
                } else {
                    ia = z * dx_inv;
                }
            } else {
                ia = r[q] * kd;
            }
            int ii = (int)ia;
            if (ii > npts_tab - 2) ii = npts_tab - 2;
            j = tab[ii] + (tab[ii + 1] - tab[ii]) * (ia - ii);
        } else {
            j = sbessel_jl(l, k * r[q]);
        }
        s += j;
    }
    map[t] = s;
}

// Y_lm(ring) = P_lm(x_ring) e^{-i m phi_0}, thread per (ring, m)
__global__ void k_hp_ylm(const double *__restrict__ ring_x, const double *__restrict__ ring_phi, int nrings, int l,
                         const double2 *__restrict__ coef /* all rows, triangular */, double2 *__restrict__ ylm) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nrings * (l + 1)) return;
    const int r = t / (l + 1), m = t - r * (l + 1);
    const double x = ring_x[r];
    // sectoral seed P_m^m, then the l-recurrence up to l (same coefficients as the raw path)
    const double somx2 = sqrt((1.0 - x) * (1.0 + x));
    double pmm = 0.28209479177387814347403972578038630;  // 1/sqrt(4 pi)
    for (int i = 1; i <= m; ++i) pmm *= coef[(size_t)i * (i + 1) / 2 + i].x * somx2;
    double p = pmm;
    if (l > m) {
        double p2 = pmm, p1 = coef[(size_t)(m + 1) * (m + 2) / 2 + m].x * (x * pmm);
        for (int ll = m + 2; ll <= l; ++ll) {
            const double2 c = coef[(size_t)ll * (ll + 1) / 2 + m];
            const double pn = c.x * (x * p1 - c.y * p2);
            p2 = p1;
            p1 = pn;
        }
        p = p1;
    }
    double sn, cs;
    sincos((double)m * ring_phi[r], &sn, &cs);
    ylm[t] = make_double2(p * cs, -p * sn);
}

constexpr int HP_NB = 32;     // n per CTA
constexpr int HP_MS = 8;      // m slots (threads) per n
constexpr int HP_MPT = 8;     // m per thread -> 64 m per CTA
constexpr int HP_JC = 32;     // folded quarter-ring positions per staged chunk
constexpr int HP_MAXPIX = 4096;  // twiddle table capacity (ring length, 4 nside <= 4096)

// per ring: G(m, n) = F_ring[s(m)](n) with the reference's extraction, times Y_lm(ring).
// A ring of N = 4 i pixels is real, so the pixels j, N-j, N/2-j, N/2+j share |cos| and
// |sin| of 2 pi j s / N: with a = x_j + x_{N-j}, b = x_{N/2-j} + x_{N/2+j},
// c = x_j - x_{N-j}, d = x_{N/2+j} - x_{N/2-j},
//   Re F[s] = sum_{j=0}^{N/4} cos(2 pi j s / N) (a + (-1)^s b)
//   Im F[s] = -sum_{j=0}^{N/4} sin(2 pi j s / N) (c + (-1)^s d)
// (j = 0: a + b -> x_0 + (-1)^s x_{N/2}, no sine; j = N/4: the orbit {N/4, 3N/4}), so
// the sum over N pixels becomes N/4 + 1 terms, folded once per chunk and shared by
// every frequency of the CTA.
__global__ void __launch_bounds__(HP_NB *HP_MS) k_hp_ring(const double *__restrict__ map, int nmax, int l,
                                                         const int *__restrict__ rings,
                                                         const int64_t *__restrict__ ring_start,
                                                         const int *__restrict__ ring_pix,
                                                         const double2 *__restrict__ tw_all,
                                                         const int64_t *__restrict__ tw_off,
                                                         const double2 *__restrict__ ylm, int conj_fix,
                                                         double2 *__restrict__ partial /* [ring][m][n] */) {
    extern __shared__ double hp_smem[];
    double2 *s_tw = reinterpret_cast<double2 *>(hp_smem);          // [rpix]
    double *s_fold = hp_smem + 2 * HP_MAXPIX;                       // [4][HP_JC][HP_NB]: even/odd cos, even/odd sin
    const int r = rings[blockIdx.x];
    const int n0 = blockIdx.y * HP_NB, m0 = blockIdx.z * (HP_MS * HP_MPT);
    const int rpix = ring_pix[r], quarter = rpix >> 2, halfp = rpix >> 1;
    const int64_t rs = ring_start[r];
    const int tid = threadIdx.x, nl = tid % HP_NB, ms = tid / HP_NB;
    const int n = n0 + nl;
    for (int k = tid; k < rpix; k += blockDim.x) s_tw[k] = tw_all[tw_off[r] + k];
    // accumulators k < kval hold valid m = m0 + ms + HP_MS k <= l
    const int kval = (l - m0 - ms) < 0 ? 0 : min(HP_MPT, (l - m0 - ms) / HP_MS + 1);
    int sidx[HP_MPT], cur[HP_MPT];
    double gr[HP_MPT], gi[HP_MPT];
#pragma unroll
    for (int k = 0; k < HP_MPT; ++k) {
        const int m = m0 + ms + HP_MS * k;
        const int mm = m % rpix;
        int s = rpix / 2 - mm;
        s = rpix / 2 - (s < 0 ? -s : s);
        sidx[k] = s;
        cur[k] = 0;
        gr[k] = gi[k] = 0.0;
    }
    for (int j0 = 0; j0 <= quarter; j0 += HP_JC) {
        const int jn = min(HP_JC, quarter + 1 - j0);
        __syncthreads();
        for (int e = tid; e < HP_JC * HP_NB; e += blockDim.x) {
            const int jj = e / HP_NB, nn = e % HP_NB, j = j0 + jj;
            double ce = 0.0, co = 0.0, se = 0.0, so = 0.0;
            if (jj < jn && n0 + nn < nmax) {
                const double *col = map + rs * nmax + n0 + nn;
                if (j == 0) {
                    const double x0 = col[0], xh = col[(int64_t)halfp * nmax];
                    ce = x0 + xh;
                    co = x0 - xh;
                } else if (j == quarter) {
                    const double xa = col[(int64_t)quarter * nmax], xb = col[(int64_t)(3 * quarter) * nmax];
                    ce = co = xa + xb;
                    se = so = xa - xb;
                } else {
                    const double xj = col[(int64_t)j * nmax], xn = col[(int64_t)(rpix - j) * nmax];
                    const double xm = col[(int64_t)(halfp - j) * nmax], xp = col[(int64_t)(halfp + j) * nmax];
                    const double a = xj + xn, b = xm + xp, c = xj - xn, d = xp - xm;
                    ce = a + b;
                    co = a - b;
                    se = c + d;
                    so = c - d;
                }
            }
            s_fold[e] = ce;
            s_fold[HP_JC * HP_NB + e] = co;
            s_fold[2 * HP_JC * HP_NB + e] = se;
            s_fold[3 * HP_JC * HP_NB + e] = so;
        }
        __syncthreads();
        for (int jj = 0; jj < jn; ++jj) {
            const int o = jj * HP_NB + nl;
            const double ce = s_fold[o], co = s_fold[HP_JC * HP_NB + o];
            const double se = s_fold[2 * HP_JC * HP_NB + o], so = s_fold[3 * HP_JC * HP_NB + o];
#pragma unroll
            for (int k = 0; k < HP_MPT; ++k) {
                if (k < kval) {
                    const double2 w = s_tw[cur[k]];  // (cos, -sin) of 2 pi j s / N
                    const bool odd = sidx[k] & 1;
                    gr[k] = fma(odd ? co : ce, w.x, gr[k]);
                    gi[k] = fma(odd ? so : se, w.y, gi[k]);
                    const int c = cur[k] + sidx[k];
                    cur[k] = c >= rpix ? c - rpix : c;
                }
            }
        }
    }
    if (n >= nmax) return;
#pragma unroll
    for (int k = 0; k < HP_MPT; ++k) {
        const int m = m0 + ms + HP_MS * k;
        if (m > l) continue;
        const int mm = m % rpix;
        double fr = gr[k], fi = gi[k];
        if (m == 0) fi = 0.0;                                // sign = 0 at m = 0
        if (conj_fix && 2 * mm > rpix) fi = -fi;             // the alias is the conjugate
        const double2 y = ylm[(size_t)r * (l + 1) + m];
        partial[((size_t)r * (l + 1) + m) * nmax + n] = make_double2(fr * y.x - fi * y.y, fr * y.y + fi * y.x);
    }
}

constexpr int HF_G = 2;    // complex sequences (radial-order pairs) per CTA
constexpr int HF_T = 256;  // threads per CTA

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}

// Power-of-two ring of N pixels: the complex sequence z_j = map_j(n) + i map_j(n + 1)
// (two radial orders) goes through an in-place decimation-in-time FFT, loaded in
// bit-reversed order, radix-4 passes (each two radix-2 stages of half-lengths h and 2h
// fused into one butterfly: inputs 1, 2, 3 times W_4h^2j, W_4h^j, W_4h^3j, then sums with
// +-1 and +-i) and one radix-2 pass when log2 N is odd.  The two real transforms are A[s] = (Z[s] + conj Z[N-s]) / 2 and
// B[s] = (Z[s] - conj Z[N-s]) / 2i; the m-extraction, the sign rules and the product
// with Y_lm(ring) are those of k_hp_ring.
__global__ void __launch_bounds__(HF_T) k_hp_fft(const double *__restrict__ map, int nmax, int l,
                                                const int *__restrict__ rings,
                                                const int64_t *__restrict__ ring_start,
                                                const int *__restrict__ ring_pix,
                                                const double2 *__restrict__ tw_all,
                                                const int64_t *__restrict__ tw_off,
                                                const double2 *__restrict__ ylm, int conj_fix,
                                                double2 *__restrict__ partial /* [ring][m][n] */) {
    extern __shared__ double2 hf_x[];  // [HF_G][N]
    const int r = rings[blockIdx.x];
    const int N = ring_pix[r], logn = __ffs(N) - 1;
    const int64_t rs = ring_start[r];
    const double2 *__restrict__ tw = tw_all + tw_off[r];  // tw[k] = e^{-2 pi i k / N}
    const int q0 = blockIdx.y * HF_G, tid = threadIdx.x;
    // map columns n = 2 q0 .. 2 q0 + 2 HF_G - 1 of the ring's pixels, bit-reversed
    for (int e = tid; e < N * 2 * HF_G; e += HF_T) {
        const int j = e / (2 * HF_G), t = e - j * (2 * HF_G);
        const int n = 2 * q0 + t;
        const double v = n < nmax ? __ldg(map + (rs + j) * nmax + n) : 0.0;
        const int jr = logn ? (int)(__brev((unsigned)j) >> (32 - logn)) : 0;
        reinterpret_cast<double *>(hf_x + (t >> 1) * N + jr)[t & 1] = v;
    }
    const int nb4 = N >> 2;
    int h = 1;
    for (; 4 * h <= N; h *= 4) {
        __syncthreads();
        for (int e = tid; e < HF_G * nb4; e += HF_T) {
            const int g = e >> (logn - 2), k = e & (nb4 - 1);
            const int j = k & (h - 1);
            double2 *xs = hf_x + g * N + ((k - j) << 2) + j;
            const double2 x0 = xs[0];
            double2 t1 = xs[h], t2 = xs[2 * h], t3 = xs[3 * h];
            if (h > 1) {  // t1 W^2j, t2 W^j, t3 W^3j with W = W_4h
                const int st = N / (4 * h);
                t1 = cmul(t1, __ldg(tw + 2 * j * st));
                t2 = cmul(t2, __ldg(tw + j * st));
                t3 = cmul(t3, __ldg(tw + 3 * j * st));
            }
            const double2 a0 = make_double2(x0.x + t1.x, x0.y + t1.y), a1 = make_double2(x0.x - t1.x, x0.y - t1.y);
            const double2 b0 = make_double2(t2.x + t3.x, t2.y + t3.y);
            const double2 b1 = make_double2(t2.y - t3.y, t3.x - t2.x);  // -i (t2 - t3)
            xs[0] = make_double2(a0.x + b0.x, a0.y + b0.y);
            xs[2 * h] = make_double2(a0.x - b0.x, a0.y - b0.y);
            xs[h] = make_double2(a1.x + b1.x, a1.y + b1.y);
            xs[3 * h] = make_double2(a1.x - b1.x, a1.y - b1.y);
        }
    }
    if (h < N) {  // N = 2 h: the last radix-2 stage
        __syncthreads();
        const int nb2 = N >> 1;
        for (int e = tid; e < HF_G * nb2; e += HF_T) {
            const int g = e >> (logn - 1), j = e & (nb2 - 1);
            double2 *xs = hf_x + g * N + j;
            const double2 u = xs[0], v = cmul(xs[h], __ldg(tw + j));
            xs[0] = make_double2(u.x + v.x, u.y + v.y);
            xs[h] = make_double2(u.x - v.x, u.y - v.y);
        }
    }
    __syncthreads();
    const int half = N >> 1;
    for (int e = tid; e < (l + 1) * HF_G; e += HF_T) {
        const int m = e / HF_G, g = e - m * HF_G;
        const int n = 2 * (q0 + g);
        if (n >= nmax) continue;
        const int mm = m & (N - 1);
        const int d = half - mm;
        const int s = half - (d < 0 ? -d : d);
        const double2 zs = hf_x[g * N + s], zn = hf_x[g * N + ((N - s) & (N - 1))];
        double ar = zs.x + zn.x, ai = zs.y - zn.y;  // 2 A[s]
        double br = zs.y + zn.y, bi = zn.x - zs.x;  // 2 B[s]
        if (m == 0) ai = bi = 0.0;                  // sign = 0 at m = 0
        if (conj_fix && 2 * mm > N) {               // the alias is the conjugate
            ai = -ai;
            bi = -bi;
        }
        const double2 y = ylm[(size_t)r * (l + 1) + m];
        const double yr = 0.5 * y.x, yi = 0.5 * y.y;
        double2 *out = partial + ((size_t)r * (l + 1) + m) * nmax + n;
        out[0] = make_double2(ar * yr - ai * yi, ar * yi + ai * yr);
        if (n + 1 < nmax) out[1] = make_double2(br * yr - bi * yi, br * yi + bi * yr);
    }
}

// f(m, n) = sum over rings (ring order), stored as f k norm (sfb_reverse_fft.cpp:152-153)
constexpr int HR_W = 8;  // warps per reduction block, each over every HR_W-th ring

// CTA per (m, 32 radial orders): warp w sums rings w, w + HR_W, ... (lane = n), then
// warp 0 adds the HR_W sums in warp order -- a fixed order, so repeated calls agree bit
// for bit
__global__ void __launch_bounds__(32 * HR_W) k_hp_reduce(const double2 *__restrict__ partial, int nrings, int l,
                                                         int nmax, const double *__restrict__ kln, double norm,
                                                         double2 *__restrict__ fl) {
    __shared__ double2 s_sum[HR_W][32];
    const int m = blockIdx.x, n = blockIdx.y * 32 + (threadIdx.x & 31), w = threadIdx.x >> 5;
    double sr = 0.0, si = 0.0;
    if (n < nmax) {
        for (int r = w; r < nrings; r += HR_W) {
            const double2 v = partial[((size_t)r * (l + 1) + m) * nmax + n];
            sr += v.x;
            si += v.y;
        }
    }
    s_sum[w][threadIdx.x & 31] = make_double2(sr, si);
    __syncthreads();
    if (w != 0 || n >= nmax) return;
    double tr = 0.0, ti = 0.0;
#pragma unroll
    for (int k = 0; k < HR_W; ++k) {
        tr += s_sum[k][threadIdx.x].x;
        ti += s_sum[k][threadIdx.x].y;
    }
    const double k = kln[n];
    fl[(size_t)m * nmax + n] = make_double2(tr * k * norm, ti * k * norm);
}

// C_ln = (2 sum_m |f|^2 - |f_0|^2) / (2l+1) of the stored f (sfb_reverse_fft.cpp:147-150)
__global__ void k_hp_cln(const double2 *__restrict__ fl, int l, int nmax, double *__restrict__ c_row) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nmax) return;
    double sq = 0.0, f0 = 0.0;
    for (int m = 0; m <= l; ++m) {
        const double2 v = fl[(size_t)m * nmax + n];
        const double a2 = v.x * v.x + v.y * v.y;
        sq += a2;
        if (m == 0) f0 = a2;
    }
    c_row[n] = (2 * sq - f0) / (2 * l + 1);
}

struct RingTables {
    int64_t nside = -1;
    int nrings = 0;
    DevBuf buf;
    size_t off_start = 0, off_pix = 0, off_x = 0, off_phi = 0, off_tw = 0, off_twoff = 0, off_order = 0;
    // ring order: power-of-two rings by increasing length, then the others; the rings
    // taking the FFT at multipole l are the prefix of fft_count[l] entries
    int max_pow2 = 0;                // longest power-of-two ring
    std::vector<int> pow2_log;       // log2 length of the power-of-two rings, in order
};

// the FFT (about 2 N log2 N FP64 operations per radial order, measured) beats the folded
// direct sum (N/2 (l + 1) + 2 N) from l + 1 > 4 log2 N - 4 on
int fft_count(const RingTables &R, int l) {
    int c = 0;
    while (c < (int)R.pow2_log.size() && l + 1 > 4 * R.pow2_log[c] - 4) ++c;
    return c;
}
RingTables g_rings;

// host copies of the HEALPix ring geometry (same formulas as the device functions)
double fmodulo_h(double v1, double v2) {
    if (v1 >= 0) return (v1 < v2) ? v1 : std::fmod(v1, v2);
    const double tmp = std::fmod(v1, v2) + v2;
    return (tmp == v2) ? 0. : tmp;
}

int64_t isqrt_h(int64_t v) {
    int64_t r = (int64_t)std::sqrt((double)v + 0.5);
    while (r * r > v) --r;
    while ((r + 1) * (r + 1) <= v) ++r;
    return r;
}

void pix2ang_h(int64_t nside, int64_t pix, double *theta, double *phi) {
    const int64_t npix = 12 * nside * nside, ncap = 2 * nside * (nside - 1);
    const double fact2 = 4. / npix, fact1 = (nside << 1) * fact2;
    double z, ph, sth = 0.0;
    bool have_sth = false;
    if (pix < ncap) {
        const int64_t iring = (1 + isqrt_h(1 + 2 * pix)) >> 1;
        const int64_t iphi = (pix + 1) - 2 * iring * (iring - 1);
        const double tmp = (iring * iring) * fact2;
        z = 1.0 - tmp;
        if (z > 0.99) {
            sth = std::sqrt(tmp * (2.0 - tmp));
            have_sth = true;
        }
        ph = (iphi - 0.5) * (0.5 * kPi) / iring;
    } else if (pix < (npix - ncap)) {
        const int64_t nl4 = 4 * nside, ip = pix - ncap;
        const int64_t tmp = ip / nl4;
        const int64_t iring = tmp + nside, iphi = ip - nl4 * tmp + 1;
        const double fodd = ((iring + nside) & 1) ? 1 : 0.5;
        z = (2 * nside - iring) * fact1;
        ph = (iphi - fodd) * kPi * 0.75 * fact1;
    } else {
        const int64_t ip = npix - pix;
        const int64_t iring = (1 + isqrt_h(2 * ip - 1)) >> 1;
        const int64_t iphi = 4 * iring + 1 - (ip - 2 * iring * (iring - 1));
        const double tmp = (iring * iring) * fact2;
        z = tmp - 1.0;
        if (z < -0.99) {
            sth = std::sqrt(tmp * (2.0 - tmp));
            have_sth = true;
        }
        ph = (iphi - 0.5) * (0.5 * kPi) / iring;
    }
    *theta = have_sth ? std::atan2(sth, z) : std::acos(z);
    *phi = ph;
}

catana_status_t ensure_rings(int64_t nside, cudaStream_t st) {
    RingTables &R = g_rings;
    if (R.nside == nside) return CATANA_OK;
    const int nrings = (int)(4 * nside - 1);
    const int64_t npix = 12 * nside * nside, ncap = 2 * nside * (nside - 1);
    std::vector<int64_t> start(nrings), twoff(nrings);
    std::vector<int> rp(nrings);
    std::vector<double> x(nrings), ph(nrings);
    // twiddles, one table per ring length 4 i (i = 1 .. nside), offset 2 i (i - 1)
    std::vector<double2> tw((size_t)2 * nside * (nside + 1));
    for (int64_t i = 1; i <= nside; ++i) {
        const int64_t len = 4 * i, off = 2 * i * (i - 1);
        for (int64_t k = 0; k < len; ++k) {
            const double a = -2.0 * kPi * (double)k / (double)len;
            tw[off + k] = make_double2(std::cos(a), std::sin(a));
        }
    }
    for (int r = 0; r < nrings; ++r) {  // get_ring_info_small(r + 1)
        const int64_t ring = r + 1;
        int64_t s, len;
        if (ring < nside) {
            len = 4 * ring;
            s = 2 * ring * (ring - 1);
        } else if (ring < 3 * nside) {
            len = 4 * nside;
            s = ncap + (ring - nside) * 4 * nside;
        } else {
            const int64_t nr = 4 * nside - ring;
            len = 4 * nr;
            s = npix - 2 * nr * (nr + 1);
        }
        start[r] = s;
        rp[r] = (int)len;
        const int64_t i = len / 4;
        twoff[r] = 2 * i * (i - 1);
        double th, phi;
        pix2ang_h(nside, s, &th, &phi);
        x[r] = std::cos(th);  // RingInfo: cos(theta) of the first pixel (sfb_reverse_fft.cpp:21)
        ph[r] = phi;
    }
    std::vector<int> order(nrings);
    for (int r = 0; r < nrings; ++r) order[r] = r;
    auto is_pow2 = [&](int r) { return (rp[r] & (rp[r] - 1)) == 0; };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        const bool pa = is_pow2(a), pb = is_pow2(b);
        if (pa != pb) return pa;
        return pa && rp[a] < rp[b];
    });
    R.pow2_log.clear();
    R.max_pow2 = 0;
    for (int r : order) {
        if (!is_pow2(r)) break;
        int lg = 0;
        while ((1 << lg) < rp[r]) ++lg;
        R.pow2_log.push_back(lg);
        R.max_pow2 = std::max(R.max_pow2, rp[r]);
    }
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    R.off_start = 0;
    R.off_pix = al(R.off_start + nrings * sizeof(int64_t));
    R.off_x = al(R.off_pix + nrings * sizeof(int));
    R.off_phi = al(R.off_x + nrings * sizeof(double));
    R.off_twoff = al(R.off_phi + nrings * sizeof(double));
    R.off_order = al(R.off_twoff + nrings * sizeof(int64_t));
    R.off_tw = al(R.off_order + nrings * sizeof(int));
    const size_t total = R.off_tw + tw.size() * sizeof(double2);
    CG_CUDA_TRY(R.buf.ensure(total));
    char *b = R.buf.as<char>();
    CG_CUDA_TRY(cudaMemcpyAsync(b + R.off_start, start.data(), nrings * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    CG_CUDA_TRY(cudaMemcpyAsync(b + R.off_pix, rp.data(), nrings * sizeof(int), cudaMemcpyHostToDevice, st));
    CG_CUDA_TRY(cudaMemcpyAsync(b + R.off_x, x.data(), nrings * sizeof(double), cudaMemcpyHostToDevice, st));
    CG_CUDA_TRY(cudaMemcpyAsync(b + R.off_phi, ph.data(), nrings * sizeof(double), cudaMemcpyHostToDevice, st));
    CG_CUDA_TRY(cudaMemcpyAsync(b + R.off_twoff, twoff.data(), nrings * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    CG_CUDA_TRY(cudaMemcpyAsync(b + R.off_order, order.data(), nrings * sizeof(int), cudaMemcpyHostToDevice, st));
    CG_CUDA_TRY(cudaMemcpyAsync(b + R.off_tw, tw.data(), tw.size() * sizeof(double2), cudaMemcpyHostToDevice, st));
    CG_CUDA_TRY(cudaStreamSynchronize(st));
    R.nside = nside;
    R.nrings = nrings;
    return CATANA_OK;
}

}  // namespace

catana_status_t healpix_ang2pix_dev(int64_t nside, const double *theta, const double *phi, int64_t n, int64_t *pix,
                                    int *err_dev, cudaStream_t st) {
    if (n == 0) return CATANA_OK;
    k_ang2pix<<<ceil_div(n, 256), 256, 0, st>>>(nside, theta, phi, n, pix, err_dev);
    count_launch();
    CG_CUDA_TRY(cudaGetLastError());
    return CATANA_OK;
}

catana_status_t healpix_pix2ang_dev(int64_t nside, const int64_t *pix, int64_t n, double *theta, double *phi,
                                    cudaStream_t st) {
    if (n == 0) return CATANA_OK;
    k_pix2ang<<<ceil_div(n, 256), 256, 0, st>>>(nside, pix, n, theta, phi);
    count_launch();
    CG_CUDA_TRY(cudaGetLastError());
    return CATANA_OK;
}

catana_status_t healpix_bin_dev(DeviceContext *ctx, int64_t nside, const double *points_dev, int64_t npoints,
                                int64_t *offsets_dev, double *r_sorted_dev, int *err_dev, cudaStream_t st) {
    const int64_t npix = 12 * nside * nside;
    if (npoints > (int64_t)0xFFFFFFFFll - 1) {
        set_error("bin_points: at most 2^32 - 2 points");
        return CATANA_ERR_ARG;
    }
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t nb = al((size_t)std::max<int64_t>(npoints, 1) * sizeof(uint32_t));
    const size_t cb = al((size_t)(npix + 1) * sizeof(uint32_t));
    const size_t hb = al((size_t)256 * ((npoints + 4095) / 4096 + 1) * sizeof(uint32_t));
    CG_CUDA_TRY(ctx->hp_ws.ensure(4 * nb + cb + hb));
    char *w = ctx->hp_ws.as<char>();
    uint32_t *keys = reinterpret_cast<uint32_t *>(w), *vals = reinterpret_cast<uint32_t *>(w + nb);
    uint32_t *tk = reinterpret_cast<uint32_t *>(w + 2 * nb), *tv = reinterpret_cast<uint32_t *>(w + 3 * nb);
    uint32_t *counts = reinterpret_cast<uint32_t *>(w + 4 * nb);
    uint32_t *hist = reinterpret_cast<uint32_t *>(w + 4 * nb + cb);
    CG_CUDA_TRY(cudaMemsetAsync(counts, 0, (npix + 1) * sizeof(uint32_t), st));
    if (npoints > 0) {
        k_bin_keys<<<ceil_div(npoints, 256), 256, 0, st>>>(nside, points_dev, npoints, keys, vals, counts, err_dev);
        count_launch();
        CG_CUDA_TRY(cudaGetLastError());
        int bits = 0;
        while ((int64_t(1) << bits) < npix) bits += 8;
        catana_status_t s = radix_sort_pairs(keys, vals, tk, tv, npoints, bits, hist, st);
        if (s != CATANA_OK) return s;
    }
    // exclusive scan of the counts -> pixel offsets (uint32), then widen to int64
    catana_status_t s = scan_u32(counts, npix, st);
    if (s != CATANA_OK) return s;
    const int64_t nthreads = std::max<int64_t>(npoints, npix + 1);
    k_bin_gather<<<ceil_div(nthreads, 256), 256, 0, st>>>(points_dev, vals, npoints, counts, npix, r_sorted_dev,
                                                          offsets_dev);
    count_launch();
    CG_CUDA_TRY(cudaGetLastError());
    return CATANA_OK;
}

catana_status_t healpix_sfb_dev(DeviceContext *ctx, int64_t nside, const int64_t *offsets_dev,
                                const double *r_sorted_dev, int64_t npoints, int lmax, int nmax, bool interpolated,
                                bool conj_fix, const double *kln_dev, const double *kln_host, double r_min,
                                double r_max, double norm, double *f_dev, double *c_ln_dev, int *err_dev,
                                cudaStream_t st) {
    if (lmax == 0 || nmax == 0) return CATANA_OK;
    if (4 * nside > HP_MAXPIX) {
        set_error("HEALPix path supports nside <= 1024");
        return CATANA_ERR_ARG;
    }
    catana_status_t s = ensure_coefs(ctx, lmax + 1, st);
    if (s != CATANA_OK) return s;
    if (interpolated) {
        s = ensure_lerp_tables(ctx, lmax, nmax, st);
        if (s != CATANA_OK) return s;
    }
    s = ensure_rings(nside, st);
    if (s != CATANA_OK) return s;
    RingTables &R = g_rings;
    const int64_t npix = 12 * nside * nside;
    const int nrings = R.nrings;
    char *rb = R.buf.as<char>();
    const int64_t *ring_start = reinterpret_cast<const int64_t *>(rb + R.off_start);
    const int *ring_pix = reinterpret_cast<const int *>(rb + R.off_pix);
    const double *ring_x = reinterpret_cast<const double *>(rb + R.off_x);
    const double *ring_phi = reinterpret_cast<const double *>(rb + R.off_phi);
    const int64_t *tw_off = reinterpret_cast<const int64_t *>(rb + R.off_twoff);
    const double2 *tw = reinterpret_cast<const double2 *>(rb + R.off_tw);
    const int *order = reinterpret_cast<const int *>(rb + R.off_order);
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t mapb = al((size_t)npix * nmax * sizeof(double));
    const size_t ylmb = al((size_t)nrings * lmax * sizeof(double2));
    const size_t partb = al((size_t)nrings * lmax * nmax * sizeof(double2));
    const size_t kdb = al((size_t)lmax * nmax * sizeof(double));
    CG_CUDA_TRY(ctx->partial.ensure(mapb + ylmb + partb + kdb));
    double *map = ctx->partial.as<double>();
    double2 *ylm = reinterpret_cast<double2 *>(ctx->partial.as<char>() + mapb);
    double2 *partial = reinterpret_cast<double2 *>(ctx->partial.as<char>() + mapb + ylmb);
    double *kd_dev = reinterpret_cast<double *>(ctx->partial.as<char>() + mapb + ylmb + partb);
    if (interpolated && kln_host) {  // k_ln / dx per (l, n): the unchecked map levels' table scale
        std::vector<double> kd((size_t)lmax * nmax);
        for (int l = 0; l < lmax; ++l)
            for (int n = 0; n < nmax; ++n) kd[(size_t)l * nmax + n] = kln_host[(size_t)l * nmax + n] * ctx->tab_dxinv[l];
        CG_CUDA_TRY(cudaMemcpyAsync(kd_dev, kd.data(), kd.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        CG_CUDA_TRY(cudaStreamSynchronize(st));
    }
    const int npts_tab = 1000 * nmax;
    const size_t smem = (2 * HP_MAXPIX + 4 * HP_JC * HP_NB) * sizeof(double);
    const size_t smem_fft = (size_t)HF_G * R.max_pow2 * sizeof(double2);
    if (!ctx->attr_healpix) {
        CG_CUDA_TRY(cudaFuncSetAttribute(k_hp_ring, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        CG_CUDA_TRY(cudaFuncSetAttribute(k_hp_fft, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(HF_G * HP_MAXPIX * sizeof(double2))));
        ctx->attr_healpix = true;
    }
    for (int l = 0; l < lmax; ++l) {
        // the level is in the table's range when 0 <= r_min and k_max r_max < zmax (NaN radii fail both)
        const bool in_range = interpolated && kln_host && r_min >= 0.0 &&
                              kln_host[(size_t)l * nmax + nmax - 1] * r_max < ctx->tab_zmax[l];
        auto map_kern = in_range ? k_hp_map<false> : k_hp_map<true>;
        map_kern<<<ceil_div(npix * nmax, 256), 256, 0, st>>>(
            offsets_dev, r_sorted_dev, npix, nmax, kln_dev + (size_t)l * nmax, kd_dev + (size_t)l * nmax,
            interpolated ? ctx->tables.as<double>() + (size_t)l * npts_tab : nullptr, npts_tab,
            interpolated ? ctx->tab_dxinv[l] : 0.0, interpolated ? ctx->tab_zmax[l] : 0.0, l, map, err_dev);
        k_hp_ylm<<<ceil_div(nrings * (l + 1), 128), 128, 0, st>>>(ring_x, ring_phi, nrings, l, ctx->coef.as<double2>(),
                                                                  ylm);
        const int nfft = fft_count(R, l);
        prof_begin(st);
        if (nfft > 0) {
            dim3 gf(nfft, ceil_div(ceil_div(nmax, 2), HF_G));
            k_hp_fft<<<gf, HF_T, smem_fft, st>>>(map, nmax, l, order, ring_start, ring_pix, tw, tw_off, ylm,
                                                 conj_fix ? 1 : 0, partial);
            count_launch();
        }
        if (nfft < nrings) {
            dim3 grid(nrings - nfft, ceil_div(nmax, HP_NB), ceil_div(l + 1, HP_MS * HP_MPT));
            k_hp_ring<<<grid, HP_NB * HP_MS, smem, st>>>(map, nmax, l, order + nfft, ring_start, ring_pix, tw,
                                                         tw_off, ylm, conj_fix ? 1 : 0, partial);
            count_launch();
        }
        prof_end(st, 4.0 * (double)npix * nmax * (l + 1));
        double2 *fl = reinterpret_cast<double2 *>(f_dev) + (size_t)nmax * l * (l + 1) / 2;
        k_hp_reduce<<<dim3(l + 1, ceil_div(nmax, 32)), 32 * HR_W, 0, st>>>(partial, nrings, l, nmax,
                                                                   kln_dev + (size_t)l * nmax, norm, fl);
        k_hp_cln<<<ceil_div(nmax, 64), 64, 0, st>>>(fl, l, nmax, c_ln_dev + (size_t)l * nmax);
        count_launch(4);
        CG_CUDA_TRY(cudaGetLastError());
    }
    return CATANA_OK;
}

}  // namespace catana_gpu
