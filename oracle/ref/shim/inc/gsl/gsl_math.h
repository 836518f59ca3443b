/* Stand-in for <gsl/gsl_math.h>: declarations used by the reference's gauss.C. */
#ifndef UMCP_SHIM_GSL_MATH_H
#define UMCP_SHIM_GSL_MATH_H
#include <math.h>
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
typedef struct {
  double (*function)(double x, void *params);
  void *params;
} gsl_function;
#define GSL_FN_EVAL(F, x) (*((F)->function))(x, (F)->params)
#endif
