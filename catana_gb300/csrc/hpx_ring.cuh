// hpx_ring.cuh -- HEALPix RING ang2pix / pix2ang on the device (Gorski et al. 2005,
// ApJ 622:759, sec. 4), every product and sum rounded separately in the operation
// order of the CPU restatement, so both give the same pixel.  Shared by the binning,
// the pixelized SFB and the on-device ingest (angular masks).
// Source of the operation order: the reference bins with HEALPix C++
// (Healpix_Base::loc2pix / pix2loc in Healpix_cxx/healpix_base.cc, GPL-2), and a
// bit-exact pixel needs that implementation's branches -- the sin(theta) path for
// theta within 0.01 of a pole, the za < 0.99 polar test, and the integer
// kshift / (t1 >> 1) & (4 nside - 1) arithmetic of the equatorial belt -- which the
// paper does not spell out.  They are restated here, not copied.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "special.cuh"

namespace catana_gpu {
namespace {

constexpr double kInvHalfPi = 0.63661977236758134308;  // 2/pi

__device__ __forceinline__ double fmodulo_d(double v1, double v2) {
    if (v1 >= 0) return (v1 < v2) ? v1 : fmod(v1, v2);
    const double tmp = __dadd_rn(fmod(v1, v2), v2);
    return (tmp == v2) ? 0. : tmp;
}

// RING ang2pix, theta in [0, pi]; -1 outside.
__device__ int64_t ang2pix_ring_dev(int64_t nside, double theta, double phi) {
    if (!(theta >= 0.0 && theta <= kPi)) return -1;
    const int64_t npix = 12 * nside * nside, ncap = 2 * nside * (nside - 1);
    const bool have_sth = (theta < 0.01) || (theta > 3.14159 - 0.01);
    const double z = cos(theta), sth = have_sth ? sin(theta) : 0.0;
    const double za = fabs(z);
    const double tt = fmodulo_d(__dmul_rn(phi, kInvHalfPi), 4.0);
    const double dn = (double)nside;
    if (za <= 2. / 3.) {
        const int64_t nl4 = 4 * nside;
        const double temp1 = __dmul_rn(dn, __dadd_rn(0.5, tt));
        const double temp2 = __dmul_rn(__dmul_rn(dn, z), 0.75);
        const int64_t jp = (int64_t)__dsub_rn(temp1, temp2);
        const int64_t jm = (int64_t)__dadd_rn(temp1, temp2);
        const int64_t ir = nside + 1 + jp - jm;
        const int64_t kshift = 1 - (ir & 1);
        const int64_t t1 = jp + jm - nside + kshift + 1 + nl4 + nl4;
        const int64_t ip = (t1 >> 1) & (nl4 - 1);
        return ncap + (ir - 1) * nl4 + ip;
    }
    const double tp = __dsub_rn(tt, (double)(int64_t)tt);
    const double tmp = ((za < 0.99) || !have_sth)
                           ? __dmul_rn(dn, sqrt(__dmul_rn(3.0, __dsub_rn(1.0, za))))
                           : __ddiv_rn(__dmul_rn(dn, sth), sqrt(__ddiv_rn(__dadd_rn(1., za), 3.)));
    const int64_t jp = (int64_t)__dmul_rn(tp, tmp);
    const int64_t jm = (int64_t)__dmul_rn(__dsub_rn(1.0, tp), tmp);
    const int64_t ir = jp + jm + 1;
    int64_t ip = (int64_t)__dmul_rn(tt, (double)ir);
    if (ip >= 4 * ir) ip -= 4 * ir;
    return (z > 0) ? 2 * ir * (ir - 1) + ip : npix - 2 * ir * (ir + 1) + ip;
}

__device__ int64_t isqrt_dev(int64_t v) {
    int64_t r = (int64_t)sqrt((double)v + 0.5);
    while (r * r > v) --r;
    while ((r + 1) * (r + 1) <= v) ++r;
    return r;
}

__device__ void pix2ang_ring_dev(int64_t nside, int64_t pix, double *theta, double *phi) {
    const int64_t npix = 12 * nside * nside, ncap = 2 * nside * (nside - 1);
    const double fact2 = __ddiv_rn(4., (double)npix), fact1 = __dmul_rn((double)(nside << 1), fact2);
    double z, ph, sth = 0.0;
    bool have_sth = false;
    if (pix < ncap) {
        const int64_t iring = (1 + isqrt_dev(1 + 2 * pix)) >> 1;
        const int64_t iphi = (pix + 1) - 2 * iring * (iring - 1);
        const double tmp = __dmul_rn((double)(iring * iring), fact2);
        z = __dsub_rn(1.0, tmp);
        if (z > 0.99) {
            sth = sqrt(__dmul_rn(tmp, __dsub_rn(2.0, tmp)));
            have_sth = true;
        }
        ph = __ddiv_rn(__dmul_rn(__dsub_rn((double)iphi, 0.5), 0.5 * kPi), (double)iring);
    } else if (pix < (npix - ncap)) {
        const int64_t nl4 = 4 * nside, ip = pix - ncap;
        const int64_t tmp = ip / nl4;
        const int64_t iring = tmp + nside, iphi = ip - nl4 * tmp + 1;
        const double fodd = ((iring + nside) & 1) ? 1 : 0.5;
        z = __dmul_rn((double)(2 * nside - iring), fact1);
        ph = __dmul_rn(__dmul_rn(__dmul_rn(__dsub_rn((double)iphi, fodd), kPi), 0.75), fact1);
    } else {
        const int64_t ip = npix - pix;
        const int64_t iring = (1 + isqrt_dev(2 * ip - 1)) >> 1;
        const int64_t iphi = 4 * iring + 1 - (ip - 2 * iring * (iring - 1));
        const double tmp = __dmul_rn((double)(iring * iring), fact2);
        z = __dsub_rn(tmp, 1.0);
        if (z < -0.99) {
            sth = sqrt(__dmul_rn(tmp, __dsub_rn(2.0, tmp)));
            have_sth = true;
        }
        ph = __ddiv_rn(__dmul_rn(__dsub_rn((double)iphi, 0.5), 0.5 * kPi), (double)iring);
    }
    *theta = have_sth ? atan2(sth, z) : acos(z);
    *phi = ph;
}


}  // namespace
}  // namespace catana_gpu
