/* Type-only stand-in for <fftw3.h>: the reference's interp.h declares FFTW
 * members unconditionally (local_config.h forces FFTW), but the
 * energy/gradient path never calls FFTW. Any call aborts. */
#ifndef UMCP_SHIM_FFTW3_H
#define UMCP_SHIM_FFTW3_H
#include <stdlib.h>
typedef double fftw_complex[2];
typedef struct umcp_fftw_plan_s *fftw_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_MEASURE (0U)
#ifdef __cplusplus
extern "C" {
#endif
void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
fftw_plan fftw_plan_dft_1d(int n0, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
#ifdef __cplusplus
}
#endif
#endif
