/* Stand-in for the one GSL declaration the reference's besseltools sources use.
 * Test infrastructure only: the definition (ref_driver.cpp) forwards to the
 * oracle's spherical Bessel function. */
#ifndef ORACLE_REF_SHIM_GSL_SF_BESSEL_H
#define ORACLE_REF_SHIM_GSL_SF_BESSEL_H
double gsl_sf_bessel_jl(const int l, const double x);
#endif
