// C entry points over the reference's own SphericalBesselZeros / SBesselInterpolator
// classes (compiled from the reference tree by `make -C oracle ref`).  Test
// infrastructure only: used to pin the oracle's zero finder and interpolation table
// against the reference code bit for bit.
#include <catana/besseltools/SphericalBesselZeros.hpp>
#include <catana/besseltools/SBesselInterpolator.hpp>
#include <stdexcept>

extern "C" double co_sbessel_jl(int l, double x);

double gsl_sf_bessel_jl(const int l, const double x) { return co_sbessel_jl(l, x); }

extern "C" {

// zeros 0..count-1 of j_l through SphericalBesselZeros::operator[]
void ref_sbessel_zeros(unsigned int l, int count, double *out) {
  catana::besseltools::SphericalBesselZeros sbz(l);
  for(int n = 0; n < count; ++n) out[n] = sbz[n];
}

// the interpolation table the raw path builds for multipole l:
// SBesselInterpolator_uptozero(l, nmax, npts); y[i] = table[i] via operator[]
void ref_interp_table(unsigned short l, unsigned short nmax, unsigned int npts, double *y, double *zmax) {
  auto ip = catana::besseltools::SBesselInterpolator_uptozero(l, nmax, npts);
  for(unsigned int i = 0; i < npts; ++i) y[i] = ip[i];
  *zmax = ip.get_zmax();
}

// evaluate that interpolator at z[0..n); returns 1 if any call threw domain_error
int ref_interp_eval(unsigned short l, unsigned short nmax, unsigned int npts, const double *z, int n, double *out) {
  auto ip = catana::besseltools::SBesselInterpolator_uptozero(l, nmax, npts);
  int err = 0;
  for(int i = 0; i < n; ++i) {
    try {
      out[i] = ip(z[i]);
    } catch(const std::domain_error&) {
      out[i] = 0.0;
      err = 1;
    }
  }
  return err;
}
}
