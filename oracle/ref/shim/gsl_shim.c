/*
 * Project-written stand-ins for the GSL and FFTW calls that the reference's
 * membrane-surface sources link against. This file is test infrastructure:
 * it lets the reference's own interpLib.C / grad.C / gauss.C be compiled
 * here as the pinned oracle (oracle/_ref). Nothing in the product links it.
 *
 * gsl_integration_qags: the reference (gauss.C:96-306) asks for 1e-9
 * absolute accuracy on integrals of polynomial x (u+v)^p weights with an
 * endpoint singularity. This stand-in returns the integral to ~1e-15
 * relative: composite Gauss-Legendre (20 nodes, computed by Newton
 * iteration on P_20) on pieces graded geometrically toward both endpoints.
 *
 * Random numbers: splitmix64 + Box-Muller. The energy/gradient path draws
 * none; dynamics noise is only ever compared statistically.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "gsl/gsl_integration.h"
#include "gsl/gsl_rng.h"
#include "gsl/gsl_randist.h"
#include "gsl/gsl_sf.h"
#include "fftw3.h"

/* ---------------- quadrature ---------------- */

#define GL_N 20
static double gl_x[GL_N], gl_w[GL_N];
static int gl_ready = 0;

static void gl_init(void)
{
	/* Newton iteration on the Legendre polynomial P_n, three-term recurrence. */
	for (int i = 0; i < GL_N; i++) {
		double x = cos(M_PI * (i + 0.75) / (GL_N + 0.5));
		for (int it = 0; it < 100; it++) {
			double p0 = 1.0, p1 = x;
			for (int k = 2; k <= GL_N; k++) {
				double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
				p0 = p1;
				p1 = p2;
			}
			double dp = GL_N * (x * p1 - p0) / (x * x - 1.0);
			double dx = p1 / dp;
			x -= dx;
			if (fabs(dx) < 1e-17) break;
		}
		double p0 = 1.0, p1 = x;
		for (int k = 2; k <= GL_N; k++) {
			double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
			p0 = p1;
			p1 = p2;
		}
		double dp = GL_N * (x * p1 - p0) / (x * x - 1.0);
		gl_x[i] = x;
		gl_w[i] = 2.0 / ((1.0 - x * x) * dp * dp);
	}
	gl_ready = 1;
}

static double gl_piece(const gsl_function *f, double a, double b)
{
	double h = 0.5 * (b - a), c = 0.5 * (a + b), s = 0.0;
	for (int i = 0; i < GL_N; i++) s += gl_w[i] * GSL_FN_EVAL(f, c + h * gl_x[i]);
	return s * h;
}

int gsl_integration_qags(const gsl_function *f, double a, double b, double epsabs,
                         double epsrel, size_t limit, gsl_integration_workspace *workspace,
                         double *result, double *abserr)
{
	(void)epsabs; (void)epsrel; (void)limit; (void)workspace;
	if (!gl_ready) gl_init();
	double m = 0.5 * (a + b), half = m - a, coarse = 0.0, fine = 0.0;
	/* Pieces [a + half*2^-(k+1), a + half*2^-k] toward a, mirrored toward b;
	 * each piece once whole (coarse) and once as two halves (fine). On
	 * pieces graded toward an endpoint singularity of (u+v)^p type, 20-point
	 * Gauss-Legendre is exact to rounding; the two sums give the error. */
	const int NG = 120;
	for (int k = 0; k < NG; k++) {
		double lo = a + half * ldexp(1.0, -(k + 1)), hi = a + half * ldexp(1.0, -k);
		double lo2 = b - half * ldexp(1.0, -k), hi2 = b - half * ldexp(1.0, -(k + 1));
		coarse += gl_piece(f, lo, hi) + gl_piece(f, lo2, hi2);
		fine += gl_piece(f, lo, 0.5 * (lo + hi)) + gl_piece(f, 0.5 * (lo + hi), hi);
		fine += gl_piece(f, lo2, 0.5 * (lo2 + hi2)) + gl_piece(f, 0.5 * (lo2 + hi2), hi2);
	}
	double ea = a + half * ldexp(1.0, -NG), eb = b - half * ldexp(1.0, -NG);
	double tail = gl_piece(f, a, ea) + gl_piece(f, eb, b);
	*result = fine + tail;
	if (abserr) *abserr = fabs(fine - coarse);
	return 0;
}

gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n)
{
	gsl_integration_workspace *w = (gsl_integration_workspace *)malloc(sizeof(*w));
	w->limit = n;
	return w;
}

void gsl_integration_workspace_free(gsl_integration_workspace *w) { free(w); }

/* ---------------- random numbers ---------------- */

static const gsl_rng_type shim_taus = {"taus"};
static const gsl_rng_type shim_mt = {"mt19937"};
const gsl_rng_type *gsl_rng_default = &shim_mt;
const gsl_rng_type *gsl_rng_taus = &shim_taus;
const gsl_rng_type *gsl_rng_mt19937 = &shim_mt;
unsigned long gsl_rng_default_seed = 0;

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T)
{
	(void)T;
	gsl_rng *r = (gsl_rng *)malloc(sizeof(gsl_rng));
	r->state = 0x9E3779B97F4A7C15ULL;
	return r;
}
void gsl_rng_free(gsl_rng *r) { free(r); }
void gsl_rng_set(const gsl_rng *r, unsigned long seed)
{
	((gsl_rng *)r)->state = 0x9E3779B97F4A7C15ULL ^ (unsigned long long)seed;
}
const gsl_rng_type *gsl_rng_env_setup(void) { return gsl_rng_default; }
unsigned long gsl_rng_get(const gsl_rng *r)
{
	gsl_rng *g = (gsl_rng *)r;
	unsigned long long z = (g->state += 0x9E3779B97F4A7C15ULL);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
	return (unsigned long)((z ^ (z >> 31)) >> 11);
}
double gsl_rng_uniform(const gsl_rng *r) { return (double)gsl_rng_get(r) * ldexp(1.0, -53); }
double gsl_rng_uniform_pos(const gsl_rng *r)
{
	double u;
	do u = gsl_rng_uniform(r); while (u == 0.0);
	return u;
}
unsigned long gsl_rng_uniform_int(const gsl_rng *r, unsigned long n)
{
	return (unsigned long)(gsl_rng_uniform(r) * n);
}
double gsl_ran_gaussian(const gsl_rng *r, double sigma)
{
	double u1 = gsl_rng_uniform_pos(r), u2 = gsl_rng_uniform(r);
	return sigma * sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
}
double gsl_ran_flat(const gsl_rng *r, double a, double b) { return a + (b - a) * gsl_rng_uniform(r); }
double gsl_ran_exponential(const gsl_rng *r, double mu) { return -mu * log(gsl_rng_uniform_pos(r)); }
double gsl_ran_chisq(const gsl_rng *r, double nu)
{
	double s = 0.0;
	int n = (int)nu;
	for (int i = 0; i < n; i++) {
		double g = gsl_ran_gaussian(r, 1.0);
		s += g * g;
	}
	return s;
}
void gsl_ran_dir_3d(const gsl_rng *r, double *x, double *y, double *z)
{
	double a = gsl_ran_gaussian(r, 1.0), b = gsl_ran_gaussian(r, 1.0), c = gsl_ran_gaussian(r, 1.0);
	double n = sqrt(a * a + b * b + c * c);
	*x = a / n; *y = b / n; *z = c / n;
}
void gsl_ran_dir_2d(const gsl_rng *r, double *x, double *y)
{
	double t = 2.0 * M_PI * gsl_rng_uniform(r);
	*x = cos(t); *y = sin(t);
}
unsigned int gsl_ran_poisson(const gsl_rng *r, double mu)
{
	double L = exp(-mu), p = 1.0;
	unsigned int k = 0;
	do { k++; p *= gsl_rng_uniform(r); } while (p > L);
	return k - 1;
}

/* ---------------- functions off the surface path: abort if reached -------- */

#define SHIM_ABORT(name) do { fprintf(stderr, "oracle shim: %s is not available\n", name); abort(); } while (0)
double gsl_sf_legendre_sphPlm(int l, int m, double x) { (void)l; (void)m; (void)x; SHIM_ABORT("gsl_sf_legendre_sphPlm"); }
double gsl_sf_legendre_Pl(int l, double x) { (void)l; (void)x; SHIM_ABORT("gsl_sf_legendre_Pl"); }
double gsl_sf_bessel_J0(double x) { (void)x; SHIM_ABORT("gsl_sf_bessel_J0"); }
double gsl_sf_bessel_J1(double x) { (void)x; SHIM_ABORT("gsl_sf_bessel_J1"); }
double gsl_sf_bessel_Jn(int n, double x) { (void)n; (void)x; SHIM_ABORT("gsl_sf_bessel_Jn"); }
double gsl_sf_erf(double x) { return erf(x); }
double gsl_sf_erfc(double x) { return erfc(x); }
double gsl_sf_gamma(double x) { return tgamma(x); }
void *fftw_malloc(size_t n) { return malloc(n); }
void fftw_free(void *p) { free(p); }
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out, int sign, unsigned flags)
{ (void)n0; (void)n1; (void)in; (void)out; (void)sign; (void)flags; SHIM_ABORT("fftw_plan_dft_2d"); }
fftw_plan fftw_plan_dft_1d(int n0, fftw_complex *in, fftw_complex *out, int sign, unsigned flags)
{ (void)n0; (void)in; (void)out; (void)sign; (void)flags; SHIM_ABORT("fftw_plan_dft_1d"); }
void fftw_execute(const fftw_plan p) { (void)p; SHIM_ABORT("fftw_execute"); }
void fftw_destroy_plan(fftw_plan p) { (void)p; }
