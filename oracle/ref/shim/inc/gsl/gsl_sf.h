/* Stand-in for <gsl/gsl_sf.h>: special functions used only by harmonic-mode
 * code outside the membrane-surface path. Calls abort. */
#ifndef UMCP_SHIM_GSL_SF_H
#define UMCP_SHIM_GSL_SF_H
#ifdef __cplusplus
extern "C" {
#endif
double gsl_sf_legendre_sphPlm(int l, int m, double x);
double gsl_sf_legendre_Pl(int l, double x);
double gsl_sf_bessel_J0(double x);
double gsl_sf_bessel_J1(double x);
double gsl_sf_bessel_Jn(int n, double x);
double gsl_sf_erf(double x);
double gsl_sf_erfc(double x);
double gsl_sf_gamma(double x);
#ifdef __cplusplus
}
#endif
#endif
