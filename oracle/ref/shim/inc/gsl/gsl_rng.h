/* Stand-in for <gsl/gsl_rng.h>: a seeded generator handle. The energy and
 * gradient path draws no random numbers; dynamics noise is compared
 * statistically, never draw by draw. */
#ifndef UMCP_SHIM_GSL_RNG_H
#define UMCP_SHIM_GSL_RNG_H
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { const char *name; } gsl_rng_type;
typedef struct { unsigned long long state; } gsl_rng;
extern const gsl_rng_type *gsl_rng_default;
extern const gsl_rng_type *gsl_rng_taus;
extern const gsl_rng_type *gsl_rng_mt19937;
extern unsigned long gsl_rng_default_seed;
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_free(gsl_rng *r);
void gsl_rng_set(const gsl_rng *r, unsigned long seed);
const gsl_rng_type *gsl_rng_env_setup(void);
double gsl_rng_uniform(const gsl_rng *r);
double gsl_rng_uniform_pos(const gsl_rng *r);
unsigned long gsl_rng_get(const gsl_rng *r);
unsigned long gsl_rng_uniform_int(const gsl_rng *r, unsigned long n);
#ifdef __cplusplus
}
#endif
#endif
