/* Stand-in for <gsl/gsl_randist.h>: distributions the reference names. */
#ifndef UMCP_SHIM_GSL_RANDIST_H
#define UMCP_SHIM_GSL_RANDIST_H
#include "gsl_rng.h"
#ifdef __cplusplus
extern "C" {
#endif
double gsl_ran_gaussian(const gsl_rng *r, double sigma);
double gsl_ran_chisq(const gsl_rng *r, double nu);
double gsl_ran_exponential(const gsl_rng *r, double mu);
void gsl_ran_dir_3d(const gsl_rng *r, double *x, double *y, double *z);
void gsl_ran_dir_2d(const gsl_rng *r, double *x, double *y);
unsigned int gsl_ran_poisson(const gsl_rng *r, double mu);
double gsl_ran_flat(const gsl_rng *r, double a, double b);
#ifdef __cplusplus
}
#endif
#endif
