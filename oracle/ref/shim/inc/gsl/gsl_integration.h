/* Stand-in for <gsl/gsl_integration.h>: the subset the reference's gauss.C
 * calls (qags). The implementation in gsl_shim.c integrates to ~1e-15
 * relative, tighter than the 1e-9 absolute tolerance the reference asks for. */
#ifndef UMCP_SHIM_GSL_INTEGRATION_H
#define UMCP_SHIM_GSL_INTEGRATION_H
#include <stddef.h>
#include "gsl_math.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { size_t limit; } gsl_integration_workspace;
gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace *w);
int gsl_integration_qags(const gsl_function *f, double a, double b, double epsabs,
                         double epsrel, size_t limit, gsl_integration_workspace *workspace,
                         double *result, double *abserr);
#ifdef __cplusplus
}
#endif
#endif
