// sfb_fp64.cu -- the plain FP64 raw SFB path on CUDA cores (the drop-in form).
//
// Reference: _sfb_raw, sfb_raw.cpp:13-108.  The reference loops l outermost and,
// per point, evaluates j_l(k_ln r) for every n (:67-69), P_lm by gsl_sf_legendre_sphPlm
// for every m <= l (:72-74, O(l-m) each) and accumulates k j Y* (:76-78); thread
// partial sums are combined under `omp critical` (:81-84).
//
// GPU form, per multipole l and per chunk of points:
//   * the Legendre values advance by one step of the l-recurrence from two stored
//     rows P_{l-1}^m, P_{l-2}^m (FP64 [m][point] arrays in HBM), so each P_lm costs
//     O(1) instead of O(l-m);
//   * e^{-im phi} comes from one sincospi of the exactly reduced phase frac(m u) per
//     thread and m-run plus complex rotation by e^{i phi} (prepared once per point);
//   * j_l comes from the reference's own linear table (1000*nmax nodes up to
//     z_{l,nmax}, same node placement, same dx_inv, same lerp), in exact mode from
//     the direct evaluation in special.cuh, or (CATANA_JL_POLY, no counterpart in the
//     reference) from piecewise FP64 polynomials of degree 11 on unit intervals of
//     z = k r, within ~1e-14 of j_l's envelope at the cost of a table lookup;
//   * a CTA owns a slab of points and a TILE x TILE block of (m, n); it stages
//     J[n][pt] and Y[m][pt] for 32 points in shared memory and accumulates f(m,n) in
//     FP64 registers (TILE/16 x TILE/16 complex per thread);
//   * slabs write partial tiles; a second kernel sums them in slab order into the
//     f_lmn accumulator (deterministic, no atomics).
// The FP64 pipe bounds this path: 2*nmax*(l+1) FMAs per point per l.
#include <cuda_runtime.h>
#include <type_traits>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "special.cuh"

namespace catana_gpu {

namespace {

constexpr int kTP = 32;        // points per shared-memory step
constexpr int kThreads = 256;  // threads per CTA

// AoS (r, theta, phi) -> SoA r, x = cos(theta), w, (cos, sin)(phi) and the phase
// fraction u = frac(phi / 2 pi) 2^64, from which e^{-i m phi} of any m follows exactly
// (frac(m u) is exact in 64-bit arithmetic).
__global__ void k_prep_points(const double *__restrict__ pts, const double *__restrict__ w, int64_t n,
                              double *__restrict__ r_o, double *__restrict__ x_o, double *__restrict__ w_o,
                              double *__restrict__ c1_o, double *__restrict__ s1_o,
                              unsigned long long *__restrict__ u_o) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    r_o[i] = pts[3 * i];
    x_o[i] = cos(pts[3 * i + 1]);
    w_o[i] = w ? w[i] : 1.0;
    const double ph = pts[3 * i + 2];
    double sn, cs;
    sincos(ph, &sn, &cs);
    c1_o[i] = cs;
    s1_o[i] = sn;
    double f = ph * 0.15915494309189533576888376337251436;  // 1 / (2 pi)
    f -= floor(f);
    if (!(f < 1.0) || !(f >= 0.0)) f = 0.0;  // rounding up to 1, or a non-finite angle
    u_o[i] = (unsigned long long)ldexp(f, 64);
}

// y[l][i] = j_l(0 + i*dx_l): FunctionInterpolator.cpp:12-19 with the node formula
// x_min + i*dx of the reference.
__global__ void k_lerp_tables(double *__restrict__ tab, const double *__restrict__ dx, int lmax, int npts) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)lmax * npts) return;
    int l = (int)(t / npts);
    int i = (int)(t - (int64_t)l * npts);
    tab[t] = sbessel_jl(l, 0.0 + (double)(size_t)i * dx[l]);
}

// ---- piecewise FP64 j_l polynomials (CATANA_JL_POLY) ----
// Interval j covers z in [j - 1/2, j + 1/2]; on it j_l(z) = sum_s a_s t^s, t = 2 (z - j),
// the monomial form of the degree-11 Chebyshev interpolant through 12 Chebyshev
// nodes.  Chebyshev interpolation of an entire function of bounded derivatives on a
// unit interval errs by <= 2 (1/4)^12 / 12! max |j_l^(12)| ~ 1e-16 of the envelope, so
// the FP64 node values (special.cuh, ~1e-14) bound the accuracy.
constexpr int kPolyNC = 12;

__host__ __device__ inline double poly_node(int k) {
    return cos((2.0 * k + 1.0) * kPi / (2.0 * kPolyNC));
}

// vals[node][l] = j_l(z_node) for every l < lmax (node = 12 j + k)
__global__ void k_poly_nodes(int lmax, int nint, double *vals) {
    const int node = blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= nint * kPolyNC) return;
    const int j = node / kPolyNC, k = node - kPolyNC * j;
    const double z = (double)j + 0.5 * poly_node(k);
    double *o = vals + (size_t)node * lmax;
    sbessel_jl_all(lmax, fabs(z), o);
    if (z < 0.0)  // the first interval straddles 0: j_l(-z) = (-1)^l j_l(z)
        for (int l = 1; l < lmax; l += 2) o[l] = -o[l];
}

// Chebyshev coefficients c_r = (2/12) sum_k f_k T_r(t_k) (c_0 halved), then the
// monomial coefficients a_s = sum_r c_r [t^s] T_r(t) (cheb2mono, row-major [s][r]).
// The two steps keep the large entries of the basis change away from the node values:
// they multiply only the small high-order c_r.
__global__ void k_poly_coefs(int lmax, int nint, const double *__restrict__ vals,
                             const double *__restrict__ cheb2mono, double *__restrict__ tab) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= lmax * nint) return;
    const int l = t / nint, j = t - l * nint;
    double f[kPolyNC], c[kPolyNC];
    for (int k = 0; k < kPolyNC; ++k) f[k] = vals[(size_t)(kPolyNC * j + k) * lmax + l];
    for (int r = 0; r < kPolyNC; ++r) {
        double acc = 0.0;
        for (int k = 0; k < kPolyNC; ++k) acc += f[k] * cospi((double)(r * (2 * k + 1)) / (2.0 * kPolyNC));
        c[r] = acc * (r == 0 ? 1.0 : 2.0) / kPolyNC;
    }
    double *o = tab + ((size_t)l * nint + j) * kPolyNC;
    for (int s2 = 0; s2 < kPolyNC; ++s2) {
        double acc = 0.0;
        for (int r = kPolyNC - 1; r >= s2; --r) acc += cheb2mono[s2 * kPolyNC + r] * c[r];
        o[s2] = acc;
    }
}

// max r over the catalog (IEEE bits of a non-negative double) and a flag for a
// negative or non-finite radius
__global__ void k_fp64_maxr(const double *__restrict__ pts, int64_t n, unsigned long long *out) {
    double mr = 0.0;
    bool bad = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double r = pts[3 * i];
        if (!(r >= 0.0) || !isfinite(r)) bad = true;
        else if (r > mr) mr = r;
    }
    for (int o = 16; o > 0; o >>= 1) {
        mr = fmax(mr, __shfl_xor_sync(0xffffffffu, mr, o));
        bad |= __shfl_xor_sync(0xffffffffu, (int)bad, o) != 0;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&out[0], (unsigned long long)__double_as_longlong(mr));
        if (bad) atomicMax(&out[1], 1ull);
    }
}

struct LArgs {
    int l, nmax, nslabs;
    int64_t n;  // points in the chunk
    const double *r, *x, *w, *c1, *s1;
    const unsigned long long *u;  // phase fractions frac(phi / 2 pi) 2^64
    const double *kln;  // k_ln row of l (nmax)
    const double *tab;  // lerp table of l, or null
    const double *poly; // FP64 polynomial table of l ([interval][12]), or null (exact j_l when both are null)
    int poly_nint;
    int npts_tab;
    double dx_inv, zmax;
    const double *st1, *st2;  // P_{l-1}^m, P_{l-2}^m rows: [m][n]
    double *st0;              // P_l^m out
    const double2 *coef;      // recurrence coefficients of l (m = 0..l)
    double2 *partial;         // [slab][m][nmax]
    int *err;
};

template <int TILE>
__global__ void __launch_bounds__(kThreads) k_fp64_raw_l(LArgs a) {
    constexpr int TT = TILE / 16;     // per-thread accumulator tile
    constexpr int LD = TILE + 1;      // padded row of the staged tiles
    constexpr int PER_G = TILE / 8;   // items per generator thread
    extern __shared__ double smem[];
    double *sJ = smem;                // [kTP][LD]
    double *sYr = sJ + kTP * LD;      // [kTP][LD]
    double *sYi = sYr + kTP * LD;     // [kTP][LD]

    const int l = a.l;
    const int slab = blockIdx.x;
    const int m0 = blockIdx.y * TILE, n0 = blockIdx.z * TILE;
    const int mcount = min(TILE, l + 1 - m0), ncount = min(TILE, a.nmax - n0);
    const int64_t per = ((a.n + a.nslabs - 1) / a.nslabs + kTP - 1) / kTP * kTP;
    const int64_t i0 = (int64_t)slab * per, i1 = min(a.n, i0 + per);

    const int tid = threadIdx.x;
    const int q = tid % kTP, g = tid / kTP;   // generator: point q, group g
    const int tx = tid % 16, ty = tid / 16;   // contraction: n = tx+16b, m = ty+16a
    const bool write_state = (blockIdx.z == 0);
    // row sets u whose m = ty + 16 u lie past the block's count for the whole warp (its
    // ty are 2w, 2w+1) skip the contraction: the test is warp-uniform
    const int ty_warp = 2 * (tid / 32);
    int urows = 0;
#pragma unroll
    for (int u = 0; u < TT; ++u)
        if (ty_warp + 16 * u < mcount) urows = u + 1;

    double accR[TT][TT], accI[TT][TT];
#pragma unroll
    for (int u = 0; u < TT; ++u)
#pragma unroll
        for (int v = 0; v < TT; ++v) accR[u][v] = accI[u][v] = 0.0;

    const double inv_sqrt4pi = 0.28209479177387814347403972578038630;  // 1/sqrt(4 pi)

    for (int64_t base = i0; base < i1; base += kTP) {
        const int64_t i = base + q;
        const bool valid = i < i1;
        double r = 0.0, x = 0.0, wi = 0.0, c1 = 1.0, s1 = 0.0;
        unsigned long long uph = 0;
        if (valid) {
            r = a.r[i];
            x = a.x[i];
            wi = a.w[i];
            c1 = a.c1[i];
            s1 = a.s1[i];
            uph = a.u[i];
        }
        // ---- J[pt][n] = k_ln j_l(k_ln r) w ----
#pragma unroll
        for (int k = 0; k < PER_G; ++k) {
            const int nl = g + 8 * k;
            double val = 0.0;
            if (valid && nl < ncount) {
                const double kk = a.kln[n0 + nl];
                const double z = kk * r;
                double j;
                if (a.tab) {
                    if (!(z >= 0.0) || z >= a.zmax) {  // beyond the table (or a negative / NaN radius)
                        *a.err = CATANA_ERR_DOMAIN;
                        j = 0.0;
                    } else {
                        const double ia = z * a.dx_inv;
                        int ii = (int)ia;
                        if (ii > a.npts_tab - 2) ii = a.npts_tab - 2;
                        const double y0 = a.tab[ii], y1 = a.tab[ii + 1];
                        j = y0 + (y1 - y0) * (ia - ii);
                    }
                } else if (a.poly) {
                    const double zr = rint(z);
                    int jj = (int)zr;
                    if (!(z >= 0.0) || jj >= a.poly_nint) {  // the host sized the table from max r
                        *a.err = CATANA_ERR_DOMAIN;
                        jj = 0;
                    }
                    const double t = 2.0 * (z - zr);
                    const double2 *c2 = reinterpret_cast<const double2 *>(a.poly + (size_t)jj * kPolyNC);
                    const double2 c45 = c2[5], c34 = c2[4], c23 = c2[3], c12 = c2[2], c01 = c2[1], c00 = c2[0];
                    double p = fma(c45.y, t, c45.x);
                    p = fma(p, t, c34.y);
                    p = fma(p, t, c34.x);
                    p = fma(p, t, c23.y);
                    p = fma(p, t, c23.x);
                    p = fma(p, t, c12.y);
                    p = fma(p, t, c12.x);
                    p = fma(p, t, c01.y);
                    p = fma(p, t, c01.x);
                    p = fma(p, t, c00.y);
                    j = fma(p, t, c00.x);
                } else {
                    j = sbessel_jl(l, z);
                }
                val = kk * j * wi;
            }
            sJ[q * LD + nl] = val;
        }
        // ---- Y[pt][m] = P_lm(x) e^{-i m phi}, P by one recurrence step ----
        {
            const int ml0 = g * PER_G;
            // e^{-i m phi} of the run's first m: 2 pi frac(m u) reduced exactly, as a
            // fraction in [-1/2, 1/2) of a turn
            const unsigned long long tm = (unsigned long long)(m0 + ml0) * uph;
            double sn, cs;
            sincospi((double)(long long)tm * 1.0842021724855044340074528008699e-19, &sn, &cs);  // 2^-63
            double er = cs, ei = -sn;
#pragma unroll
            for (int k = 0; k < PER_G; ++k) {
                const int ml = ml0 + k;
                const int m = m0 + ml;
                if (ml >= mcount) {  // past this level's m: zero rows, no phase to advance
                    sYr[q * LD + ml] = 0.0;
                    sYi[q * LD + ml] = 0.0;
                    continue;
                }
                double P = 0.0;
                if (valid) {
                    if (l == 0) {
                        P = inv_sqrt4pi;
                    } else {
                        const double2 c = a.coef[m];
                        if (m == l) {
                            const double somx2 = sqrt((1.0 - x) * (1.0 + x));
                            P = c.x * somx2 * a.st1[(int64_t)(l - 1) * a.n + i];
                        } else if (m == l - 1) {
                            P = c.x * (x * a.st1[(int64_t)m * a.n + i]);
                        } else {
                            P = c.x * (x * a.st1[(int64_t)m * a.n + i] - c.y * a.st2[(int64_t)m * a.n + i]);
                        }
                    }
                    if (write_state) a.st0[(int64_t)m * a.n + i] = P;
                }
                sYr[q * LD + ml] = P * er;
                sYi[q * LD + ml] = P * ei;
                const double nr = er * c1 + ei * s1;
                const double ni = ei * c1 - er * s1;
                er = nr;
                ei = ni;
            }
        }
        __syncthreads();
        // ---- f(m, n) += J(n) Y(m), over the warp's live row sets only ----
        auto contract = [&](auto rows_c) {
            constexpr int U = decltype(rows_c)::value;
#pragma unroll 4
            for (int pp = 0; pp < kTP; ++pp) {
                double jv[TT], yr[U > 0 ? U : 1], yi[U > 0 ? U : 1];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    yr[u] = sYr[pp * LD + ty + 16 * u];
                    yi[u] = sYi[pp * LD + ty + 16 * u];
                }
#pragma unroll
                for (int v = 0; v < TT; ++v) jv[v] = sJ[pp * LD + tx + 16 * v];
#pragma unroll
                for (int u = 0; u < U; ++u)
#pragma unroll
                    for (int v = 0; v < TT; ++v) {
                        accR[u][v] = fma(jv[v], yr[u], accR[u][v]);
                        accI[u][v] = fma(jv[v], yi[u], accI[u][v]);
                    }
            }
        };
        if (urows == TT) contract(std::integral_constant<int, TT>());
        else if (urows == 1) contract(std::integral_constant<int, 1>());
        else if (TT == 4 && urows == 2) contract(std::integral_constant<int, (TT == 4 ? 2 : 1)>());
        else if (TT == 4 && urows == 3) contract(std::integral_constant<int, (TT == 4 ? 3 : 1)>());
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < TT; ++u)
#pragma unroll
        for (int v = 0; v < TT; ++v) {
            const int m = m0 + ty + 16 * u, n = n0 + tx + 16 * v;
            if (m < l + 1 && n < a.nmax)
                a.partial[((int64_t)slab * (l + 1) + m) * a.nmax + n] = make_double2(accR[u][v], accI[u][v]);
        }
}

// f_acc[l block][m][n] += sum over slabs, in slab order.
__global__ void k_sum_partials(const double2 *__restrict__ partial, int nslabs, int count, double2 *__restrict__ f) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    double sr = 0.0, si = 0.0;
    for (int s = 0; s < nslabs; ++s) {
        const double2 v = partial[(int64_t)s * count + t];
        sr += v.x;
        si += v.y;
    }
    double2 o = f[t];
    o.x += sr;
    o.y += si;
    f[t] = o;
}

// f *= norm, then C_ln = sum_{m=-l..l} |f_{l|m|n}|^2 / (2l+1) (sfb_raw.cpp:89-96).
__global__ void k_finish(double2 *__restrict__ f, double norm, int lmax, int nmax, double *__restrict__ c_ln) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= lmax * nmax) return;
    const int l = t / nmax, n = t - l * nmax;
    double2 *fl = f + (int64_t)nmax * l * (l + 1) / 2;
    for (int m = 0; m <= l; ++m) {
        double2 v = fl[m * nmax + n];
        v.x *= norm;
        v.y *= norm;
        fl[m * nmax + n] = v;
    }
    double c = 0.0;
    for (int m = -l; m <= l; ++m) {
        const double2 v = fl[(m < 0 ? -m : m) * nmax + n];
        c += v.x * v.x + v.y * v.y;
    }
    c_ln[t] = c / (2 * l + 1);
}

}  // namespace

catana_status_t ensure_coefs(DeviceContext *ctx, int lmax, cudaStream_t st) {
    if (ctx->coef_lmax >= lmax) return CATANA_OK;
    const int L = std::max(lmax, 2);
    std::vector<double> h((size_t)L * (L + 1));  // (a, b) pairs, triangular by l
    for (int l = 0; l < L; ++l) {
        double *row = h.data() + (size_t)l * (l + 1);
        for (int m = 0; m <= l; ++m) {
            double ca = 0.0, cb = 0.0;
            if (l >= 1 && m == l) {
                ca = -sqrt((2.0 * l + 1.0) / (2.0 * l));
            } else if (l >= 1 && m == l - 1) {
                ca = sqrt(2.0 * l + 1.0);
            } else if (l >= 2) {
                const double dl = l, dl1 = l - 1, mm = (double)m * m;
                ca = sqrt((4.0 * dl * dl - 1.0) / (dl * dl - mm));
                cb = sqrt((dl1 * dl1 - mm) / (4.0 * dl1 * dl1 - 1.0));
            }
            row[2 * m] = ca;
            row[2 * m + 1] = cb;
        }
    }
    CG_CUDA_TRY(ctx->coef.ensure(h.size() * sizeof(double)));
    CG_CUDA_TRY(cudaMemcpyAsync(ctx->coef.ptr, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    CG_CUDA_TRY(cudaStreamSynchronize(st));
    ctx->coef_lmax = L;
    return CATANA_OK;
}

catana_status_t ensure_lerp_tables(DeviceContext *ctx, int lmax, int nmax, cudaStream_t st) {
    if (ctx->tab_lmax >= lmax && ctx->tab_nmax == nmax) return CATANA_OK;
    const int npts = 1000 * nmax;  // BESSELINTERPOLATIONPOINTS_PER_ZERO * nmax
    std::vector<double> dx(lmax);
    ctx->tab_dxinv.assign(lmax, 0.0);
    ctx->tab_zmax.assign(lmax, 0.0);
    for (int l = 0; l < lmax; ++l) {
        const double zmax = zeros_for((unsigned)l, nmax + 1)[nmax];  // SBZ(l)[nmax]
        dx[l] = (zmax - 0.0) / (npts - 1);
        ctx->tab_dxinv[l] = 1. / dx[l];
        ctx->tab_zmax[l] = zmax;
    }
    CG_CUDA_TRY(ctx->tables.ensure((size_t)lmax * npts * sizeof(double) + 256 + lmax * sizeof(double)));
    double *tab = ctx->tables.as<double>();
    double *dxd = tab + (size_t)lmax * npts;
    CG_CUDA_TRY(cudaMemcpyAsync(dxd, dx.data(), lmax * sizeof(double), cudaMemcpyHostToDevice, st));
    const int64_t total = (int64_t)lmax * npts;
    k_lerp_tables<<<ceil_div(total, 256), 256, 0, st>>>(tab, dxd, lmax, npts);
    count_launch();
    CG_CUDA_TRY(cudaGetLastError());
    CG_CUDA_TRY(cudaStreamSynchronize(st));
    ctx->tab_lmax = lmax;
    ctx->tab_nmax = nmax;
    return CATANA_OK;
}

// FP64 j_l polynomials for l < lmax over nint unit intervals (cached per device; a
// larger cached table serves, with its own interval count as the row stride)
catana_status_t ensure_poly_tables(DeviceContext *ctx, int lmax, int nint, cudaStream_t st) {
    if (ctx->poly_lmax >= lmax && ctx->poly_nint >= nint) return CATANA_OK;
    lmax = std::max(lmax, ctx->poly_lmax);
    nint = std::max(nint, ctx->poly_nint);
    // [t^s] T_r(t) by T_{r+1} = 2 t T_r - T_{r-1} (exact small integers)
    std::vector<double> T((size_t)kPolyNC * kPolyNC, 0.0), m2((size_t)kPolyNC * kPolyNC, 0.0);
    T[0] = 1.0;                 // T_0 = 1   (row r, column s)
    T[kPolyNC + 1] = 1.0;       // T_1 = t
    for (int r = 1; r + 1 < kPolyNC; ++r)
        for (int s2 = 0; s2 < kPolyNC; ++s2) {
            const double up = s2 > 0 ? 2.0 * T[(size_t)r * kPolyNC + s2 - 1] : 0.0;
            T[(size_t)(r + 1) * kPolyNC + s2] = up - T[(size_t)(r - 1) * kPolyNC + s2];
        }
    for (int s2 = 0; s2 < kPolyNC; ++s2)
        for (int r = 0; r < kPolyNC; ++r) m2[(size_t)s2 * kPolyNC + r] = T[(size_t)r * kPolyNC + s2];
    const size_t tab_bytes = (size_t)lmax * nint * kPolyNC * sizeof(double);
    CG_CUDA_TRY(ctx->poly.ensure(tab_bytes));
    DevBuf tmp;
    const size_t vbytes = (size_t)nint * kPolyNC * lmax * sizeof(double);
    CG_CUDA_TRY(tmp.ensure(vbytes + m2.size() * sizeof(double)));
    double *vals = tmp.as<double>();
    double *m2d = vals + (size_t)nint * kPolyNC * lmax;
    CG_CUDA_TRY(cudaMemcpyAsync(m2d, m2.data(), m2.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    k_poly_nodes<<<ceil_div((int64_t)nint * kPolyNC, 64), 64, 0, st>>>(lmax, nint, vals);
    count_launch();
    CG_CUDA_TRY(cudaGetLastError());
    k_poly_coefs<<<ceil_div((int64_t)lmax * nint, 128), 128, 0, st>>>(lmax, nint, vals, m2d, ctx->poly.as<double>());
    count_launch();
    CG_CUDA_TRY(cudaGetLastError());
    CG_CUDA_TRY(cudaStreamSynchronize(st));
    tmp.release();
    ctx->poly_lmax = lmax;
    ctx->poly_nint = nint;
    return CATANA_OK;
}

catana_status_t fp64_raw_accumulate(DeviceContext *ctx, const double *points_dev, const double *weights_dev,
                                    int64_t npoints, int lmax, int nmax, JlMode jl, const double *kln_dev,
                                    double *f_acc_dev, int *err_dev, cudaStream_t st) {
    const bool interpolated = (jl == JL_MODE_LERP);
    catana_status_t s = ensure_coefs(ctx, lmax, st);
    if (s != CATANA_OK) return s;
    if (interpolated) {
        s = ensure_lerp_tables(ctx, lmax, nmax, st);
        if (s != CATANA_OK) return s;
    }
    if (npoints == 0 || lmax == 0 || nmax == 0) return CATANA_OK;
    if (jl == JL_MODE_POLY) {
        // the table must reach max_l k_{l,nmax-1} * max r: one read-back of max r
        CG_CUDA_TRY(ctx->cat_scratch.ensure(16));
        unsigned long long *mx = ctx->cat_scratch.as<unsigned long long>();
        CG_CUDA_TRY(cudaMemsetAsync(mx, 0, 16, st));
        k_fp64_maxr<<<std::min<int64_t>(4 * ctx->sm_count, ceil_div(npoints, 256)), 256, 0, st>>>(points_dev, npoints,
                                                                                                  mx);
        count_launch();
        CG_CUDA_TRY(cudaGetLastError());
        unsigned long long mh[2] = {0ull, 0ull};
        std::vector<double> kh((size_t)lmax * nmax);
        CG_CUDA_TRY(cudaMemcpyAsync(mh, mx, 16, cudaMemcpyDeviceToHost, st));
        CG_CUDA_TRY(cudaMemcpyAsync(kh.data(), kln_dev, kh.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
        CG_CUDA_TRY(cudaStreamSynchronize(st));
        double max_r;
        memcpy(&max_r, &mh[0], 8);
        if (mh[1]) {
            set_error("argument (z) outside of defined range: a radius is negative or not finite");
            return CATANA_ERR_DOMAIN;
        }
        double kmax = 0.0;
        for (double k : kh) kmax = std::max(kmax, k);
        const double zmax = kmax * max_r;
        if (!(zmax < 1e6)) {
            set_error("poly j_l: k_ln * max(r) beyond 1e6");
            return CATANA_ERR_DOMAIN;
        }
        s = ensure_poly_tables(ctx, lmax, (int)std::floor(zmax + 0.5) + 2, st);
        if (s != CATANA_OK) return s;
    }
    // Chunk so that the three Legendre rows stay under ~1.5 GB.
    int64_t chunk = (int64_t)(1.5e9 / (3.0 * 8.0 * std::max(lmax, 1)));
    chunk = std::max<int64_t>(1024, std::min<int64_t>(chunk, npoints));
    CG_CUDA_TRY(ctx->soa.ensure((size_t)chunk * 6 * sizeof(double)));
    CG_CUDA_TRY(ctx->state.ensure((size_t)chunk * 3 * std::max(lmax, 1) * sizeof(double)));
    double *soa = ctx->soa.as<double>();
    double *rows[3];
    for (int k = 0; k < 3; ++k) rows[k] = ctx->state.as<double>() + (size_t)k * chunk * std::max(lmax, 1);
    const int npts_tab = 1000 * nmax;
    const double2 *coef = ctx->coef.as<double2>();
    // size the partial buffer once for the largest multipole of this call
    {
        size_t pmax = 0;
        for (int l = 0; l < lmax; ++l) {
            const int TILE = ((l + 1 > 32) || (nmax > 32)) ? 64 : 32;
            const int mb = ceil_div(l + 1, TILE), nb = ceil_div(nmax, TILE);
            int nslabs = std::min(std::max(1, (4 * ctx->sm_count) / (mb * nb)), ceil_div(chunk, kTP));
            pmax = std::max(pmax, (size_t)nslabs * (l + 1) * nmax * sizeof(double2));
        }
        CG_CUDA_TRY(ctx->partial.ensure(pmax));
    }
    if (!ctx->attr_fp64) {
        CG_CUDA_TRY(cudaFuncSetAttribute(k_fp64_raw_l<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(3 * kTP * (64 + 1) * sizeof(double))));
        ctx->attr_fp64 = true;
    }

    for (int64_t c0 = 0; c0 < npoints; c0 += chunk) {
        const int64_t nc = std::min(chunk, npoints - c0);
        double *r = soa, *x = soa + chunk, *w = soa + 2 * chunk, *c1 = soa + 3 * chunk, *s1 = soa + 4 * chunk;
        unsigned long long *uph = reinterpret_cast<unsigned long long *>(soa + 5 * chunk);
        k_prep_points<<<ceil_div(nc, 256), 256, 0, st>>>(points_dev + 3 * c0, weights_dev ? weights_dev + c0 : nullptr,
                                                         nc, r, x, w, c1, s1, uph);
        count_launch();
        double *st0 = rows[0], *st1 = rows[1], *st2 = rows[2];
        for (int l = 0; l < lmax; ++l) {
            const bool big = (l + 1 > 32) || (nmax > 32);
            const int TILE = big ? 64 : 32;
            const int mb = ceil_div(l + 1, TILE), nb = ceil_div(nmax, TILE);
            const int tiles = ceil_div(nc, kTP);
            int nslabs = std::max(1, (4 * ctx->sm_count) / (mb * nb));
            nslabs = std::min(nslabs, tiles);
            LArgs a;
            a.l = l;
            a.nmax = nmax;
            a.nslabs = nslabs;
            a.n = nc;
            a.r = r;
            a.x = x;
            a.w = w;
            a.c1 = c1;
            a.s1 = s1;
            a.u = uph;
            a.kln = kln_dev + (size_t)l * nmax;
            a.tab = interpolated ? ctx->tables.as<double>() + (size_t)l * npts_tab : nullptr;
            a.poly = jl == JL_MODE_POLY ? ctx->poly.as<double>() + (size_t)l * ctx->poly_nint * kPolyNC : nullptr;
            a.poly_nint = ctx->poly_nint;
            a.npts_tab = npts_tab;
            a.dx_inv = interpolated ? ctx->tab_dxinv[l] : 0.0;
            a.zmax = interpolated ? ctx->tab_zmax[l] : 0.0;
            a.st1 = st1;
            a.st2 = st2;
            a.st0 = st0;
            a.coef = coef + (size_t)l * (l + 1) / 2 * 1;  // (a,b) pairs: row l starts at l(l+1)/2 pairs
            a.partial = ctx->partial.as<double2>();
            a.err = err_dev;
            dim3 grid(nslabs, mb, nb);
            prof_begin(st);
            if (big) {
                const size_t sm = 3 * kTP * (64 + 1) * sizeof(double);
                k_fp64_raw_l<64><<<grid, kThreads, sm, st>>>(a);
            } else {
                const size_t sm = 3 * kTP * (32 + 1) * sizeof(double);
                k_fp64_raw_l<32><<<grid, kThreads, sm, st>>>(a);
            }
            prof_end(st, 4.0 * (double)nc * nmax * (l + 1));
            count_launch();
            CG_CUDA_TRY(cudaGetLastError());
            const int cnt = (l + 1) * nmax;
            double2 *fl = reinterpret_cast<double2 *>(f_acc_dev) + (size_t)nmax * l * (l + 1) / 2;
            k_sum_partials<<<ceil_div(cnt, 256), 256, 0, st>>>(ctx->partial.as<double2>(), nslabs, cnt, fl);
            count_launch();
            CG_CUDA_TRY(cudaGetLastError());
            // rotate rows: new l-1 <- st0, new l-2 <- st1
            double *t = st2;
            st2 = st1;
            st1 = st0;
            st0 = t;
        }
    }
    return CATANA_OK;
}

catana_status_t finish_flmn_cln(double *f_dev, double norm, int lmax, int nmax, double *c_ln_dev, cudaStream_t st) {
    const int cnt = lmax * nmax;
    if (cnt == 0) return CATANA_OK;
    k_finish<<<ceil_div(cnt, 128), 128, 0, st>>>(reinterpret_cast<double2 *>(f_dev), norm, lmax, nmax, c_ln_dev);
    count_launch();
    CG_CUDA_TRY(cudaGetLastError());
    return CATANA_OK;
}


// ---------------------------------------------------------------------------
// Allocation-free entry point: catana_gpu_sfb_raw_noalloc.
//
// For callers that cannot allocate device memory themselves or let a library do
// it (code running under a caller-owned memory pool or a fixed memory budget, or
// work that must not trigger cudaMalloc's implicit device synchronisation), this
// runs the plain FP64 raw path with all of its scratch -- point SoA, Legendre rows,
// slab partial sums, recurrence coefficients, interpolation tables, the error and
// weight-sum words -- carved out of one fixed static device array, kNoAllocBytes per
// device, held for the life of the process.  The first call on each device resolves
// the array's device address with cudaGetSymbolAddress (make that first call before
// any stream capture).  Every call shares the array: overlapping calls on the GPU
// (two host threads, or several streams) race on it.
// ---------------------------------------------------------------------------
constexpr size_t kNoAllocBytes = size_t(32) << 20;  // 32 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {

std::mutex g_noalloc_mu;
constexpr int kNoAllocMaxDevices = 64;
unsigned char *g_noalloc_base[kNoAllocMaxDevices] = {nullptr};
constexpr int kNoAllocMaxSlabs = 256;

__global__ void k_noalloc_wsum(const double *w, int64_t n, double *out) {
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

}  // namespace

}  // namespace catana_gpu

using namespace catana_gpu;

extern "C" catana_status_t catana_gpu_sfb_raw_noalloc(const double *points_dev, const double *weights_dev,
                                                     int64_t npoints, uint16_t lmax, uint16_t nmax, double rmax,
                                                     uint32_t flags, double *k_ln_dev, double *c_ln_dev,
                                                     double *f_lmn_dev, catana_gpu_stream_t stream) {
    if (npoints < 0 || !(rmax > 0.0) || !std::isfinite(rmax)) {
        set_error("sfb_raw_noalloc: npoints must be >= 0 and rmax positive and finite");
        return CATANA_ERR_ARG;
    }
    if ((flags & CATANA_FORM_MASK) != CATANA_FORM_PLAIN) {
        set_error("sfb_raw_noalloc: only the plain FP64 form runs allocation-free");
        return CATANA_ERR_ARG;
    }
    const size_t lm = (size_t)lmax * nmax;
    if (lm && (!k_ln_dev || !c_ln_dev || !f_lmn_dev)) {
        set_error("sfb_raw_noalloc: k_ln, c_ln and f_lmn device buffers are required");
        return CATANA_ERR_ARG;
    }
    if (npoints > 0 && !points_dev) {
        set_error("sfb_raw_noalloc: null points");
        return CATANA_ERR_ARG;
    }
    const uint32_t jl = flags & CATANA_JL_MASK;
    if (jl == CATANA_JL_POLY) {
        set_error("sfb_raw_noalloc: the polynomial j_l tables (CATANA_JL_POLY) are not available allocation-free");
        return CATANA_ERR_ARG;
    }
    const bool interpolated = jl == CATANA_JL_INTERP || (jl == CATANA_JL_AUTO && npoints > 1000);
    // scratch plan: [words 256 B][coefficients][tables + dx][SoA][3 Legendre rows][partials]
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    const int L = std::max<int>(lmax, 2);
    const int npts_tab = 1000 * nmax;
    const size_t b_words = 256;
    const size_t b_coef = al((size_t)L * (L + 1) * sizeof(double));
    const size_t b_tab = interpolated ? al(((size_t)lmax * npts_tab + lmax) * sizeof(double)) : 0;
    const size_t b_part = al((size_t)kNoAllocMaxSlabs * lmax * nmax * sizeof(double2));
    const size_t fixed = b_words + b_coef + b_tab + b_part;
    const size_t per_point = (6 + 3 * (size_t)std::max<int>(lmax, 1)) * sizeof(double);
    const int64_t min_chunk = std::min<int64_t>(std::max<int64_t>(npoints, 1), 1024);
    if (fixed + (size_t)min_chunk * per_point + 256 > kNoAllocBytes) {
        set_error("sfb_raw_noalloc: lmax=" + std::to_string(lmax) + ", nmax=" + std::to_string(nmax) +
                  " needs more than the " + std::to_string(kNoAllocBytes >> 20) +
                  " MiB allocation-free scratch (the tables and partial sums grow with lmax * nmax)");
        return CATANA_ERR_ARG;
    }
    int dev = 0;
    CG_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) {
        set_error("sfb_raw_noalloc: device index out of range");
        return CATANA_ERR_ARG;
    }
    int cs;
    DeviceContext *ctx = get_context(&cs);  // device properties only; its buffers are not used
    if (!ctx) return (catana_status_t)cs;
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_noalloc_base[dev]) {
        void *p = nullptr;
        CG_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_base[dev] = static_cast<unsigned char *>(p);
    }
    unsigned char *base = g_noalloc_base[dev];
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    int *err_d = reinterpret_cast<int *>(base);
    double *wsum_d = reinterpret_cast<double *>(base + 64);
    double2 *coef_d = reinterpret_cast<double2 *>(base + b_words);
    double *tab_d = reinterpret_cast<double *>(base + b_words + b_coef);
    double2 *part_d = reinterpret_cast<double2 *>(base + b_words + b_coef + b_tab);
    unsigned char *var = base + fixed;
    const size_t var_bytes = kNoAllocBytes - fixed;
    int64_t chunk = (int64_t)(var_bytes / per_point);
    chunk = std::max<int64_t>(1, std::min<int64_t>(chunk, std::max<int64_t>(npoints, 1)));
    double *soa = reinterpret_cast<double *>(var);
    double *rows0 = soa + 6 * chunk;

    CG_CUDA_TRY(cudaMemsetAsync(err_d, 0, sizeof(int), st));
    // k_ln on the host (cached zeros of the reference's zero finder)
    std::vector<double> kh(lm);
    kln_table(lmax, nmax, rmax, kh.data());
    if (lm) CG_CUDA_TRY(cudaMemcpyAsync(k_ln_dev, kh.data(), lm * sizeof(double), cudaMemcpyHostToDevice, st));
    const size_t fbytes = catana_gpu_flmn_size(lmax, nmax) * 2 * sizeof(double);
    if (fbytes) CG_CUDA_TRY(cudaMemsetAsync(f_lmn_dev, 0, fbytes, st));
    if (lm == 0) return CATANA_OK;
    // recurrence coefficients (same values as the cached table of the plain path)
    std::vector<double> ch((size_t)L * (L + 1));
    for (int l = 0; l < L; ++l) {
        double *row = ch.data() + (size_t)l * (l + 1);
        for (int m = 0; m <= l; ++m) {
            double ca = 0.0, cb = 0.0;
            if (l >= 1 && m == l) {
                ca = -sqrt((2.0 * l + 1.0) / (2.0 * l));
            } else if (l >= 1 && m == l - 1) {
                ca = sqrt(2.0 * l + 1.0);
            } else if (l >= 2) {
                const double dl = l, dl1 = l - 1, mm = (double)m * m;
                ca = sqrt((4.0 * dl * dl - 1.0) / (dl * dl - mm));
                cb = sqrt((dl1 * dl1 - mm) / (4.0 * dl1 * dl1 - 1.0));
            }
            row[2 * m] = ca;
            row[2 * m + 1] = cb;
        }
    }
    CG_CUDA_TRY(cudaMemcpyAsync(coef_d, ch.data(), ch.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    // interpolation tables, rebuilt each call (the array keeps whatever the last call left)
    std::vector<double> dx(lmax), dxinv(lmax), zmx(lmax);
    if (interpolated) {
        for (int l = 0; l < lmax; ++l) {
            zmx[l] = zeros_for((unsigned)l, nmax + 1)[nmax];
            dx[l] = (zmx[l] - 0.0) / (npts_tab - 1);
            dxinv[l] = 1. / dx[l];
        }
        double *dx_d = tab_d + (size_t)lmax * npts_tab;
        CG_CUDA_TRY(cudaMemcpyAsync(dx_d, dx.data(), lmax * sizeof(double), cudaMemcpyHostToDevice, st));
        const int64_t total = (int64_t)lmax * npts_tab;
        k_lerp_tables<<<ceil_div(total, 256), 256, 0, st>>>(tab_d, dx_d, lmax, npts_tab);
        count_launch();
        CG_CUDA_TRY(cudaGetLastError());
    }
    CG_CUDA_TRY(cudaFuncSetAttribute(k_fp64_raw_l<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(3 * kTP * (64 + 1) * sizeof(double))));
    double *rows[3];
    for (int k = 0; k < 3; ++k) rows[k] = rows0 + (size_t)k * chunk * std::max<int>(lmax, 1);
    for (int64_t c0 = 0; c0 < npoints; c0 += chunk) {
        const int64_t nc = std::min(chunk, npoints - c0);
        double *r = soa, *x = soa + chunk, *w = soa + 2 * chunk, *c1 = soa + 3 * chunk, *s1 = soa + 4 * chunk;
        unsigned long long *uph = reinterpret_cast<unsigned long long *>(soa + 5 * chunk);
        k_prep_points<<<ceil_div(nc, 256), 256, 0, st>>>(points_dev + 3 * c0, weights_dev ? weights_dev + c0 : nullptr,
                                                         nc, r, x, w, c1, s1, uph);
        count_launch();
        double *st0 = rows[0], *st1 = rows[1], *st2 = rows[2];
        for (int l = 0; l < lmax; ++l) {
            const bool big = (l + 1 > 32) || (nmax > 32);
            const int TILE = big ? 64 : 32;
            const int mb = ceil_div(l + 1, TILE), nb = ceil_div(nmax, TILE);
            int nslabs = std::max(1, (4 * ctx->sm_count) / (mb * nb));
            nslabs = std::min(std::min(nslabs, ceil_div(nc, kTP)), kNoAllocMaxSlabs);
            LArgs a;
            a.l = l;
            a.nmax = nmax;
            a.nslabs = nslabs;
            a.n = nc;
            a.r = r;
            a.x = x;
            a.w = w;
            a.c1 = c1;
            a.s1 = s1;
            a.u = uph;
            a.tab = interpolated ? tab_d + (size_t)l * npts_tab : nullptr;
            a.poly = nullptr;
            a.poly_nint = 0;
            a.npts_tab = npts_tab;
            a.dx_inv = interpolated ? dxinv[l] : 0.0;
            a.zmax = interpolated ? zmx[l] : 0.0;
            a.st1 = st1;
            a.st2 = st2;
            a.st0 = st0;
            a.coef = coef_d + (size_t)l * (l + 1) / 2;
            a.partial = part_d;
            a.err = err_d;
            a.kln = k_ln_dev + (size_t)l * nmax;
            dim3 grid(nslabs, mb, nb);
            if (big)
                k_fp64_raw_l<64><<<grid, kThreads, 3 * kTP * (64 + 1) * sizeof(double), st>>>(a);
            else
                k_fp64_raw_l<32><<<grid, kThreads, 3 * kTP * (32 + 1) * sizeof(double), st>>>(a);
            count_launch();
            CG_CUDA_TRY(cudaGetLastError());
            const int cnt = (l + 1) * nmax;
            double2 *fl = reinterpret_cast<double2 *>(f_lmn_dev) + (size_t)nmax * l * (l + 1) / 2;
            k_sum_partials<<<ceil_div(cnt, 256), 256, 0, st>>>(part_d, nslabs, cnt, fl);
            count_launch();
            CG_CUDA_TRY(cudaGetLastError());
            double *t = st2;
            st2 = st1;
            st1 = st0;
            st0 = t;
        }
    }
    double wsum = (double)npoints;
    if (weights_dev && npoints > 0) {
        k_noalloc_wsum<<<1, 1024, 0, st>>>(weights_dev, npoints, wsum_d);
        count_launch();
        CG_CUDA_TRY(cudaGetLastError());
        CG_CUDA_TRY(cudaMemcpyAsync(&wsum, wsum_d, sizeof(double), cudaMemcpyDeviceToHost, st));
        CG_CUDA_TRY(cudaStreamSynchronize(st));
    }
    double nf = std::sqrt(2. / kPi) * (4. / 3.) * kPi;  // sfb_raw.cpp:29-30
    nf *= (double)rmax * rmax * rmax / wsum;
    catana_status_t s = finish_flmn_cln(f_lmn_dev, nf, lmax, nmax, c_ln_dev, st);
    if (s != CATANA_OK) return s;
    int err_h = 0;
    CG_CUDA_TRY(cudaMemcpyAsync(&err_h, err_d, sizeof(int), cudaMemcpyDeviceToHost, st));
    CG_CUDA_TRY(cudaStreamSynchronize(st));
    if (err_h == CATANA_ERR_DOMAIN) {
        set_error("argument (z) outside of defined range.");
        return CATANA_ERR_DOMAIN;
    }
    return CATANA_OK;
}

namespace catana_gpu {
}  // namespace catana_gpu
