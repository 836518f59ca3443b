/*
 * ORACLE - test infrastructure, not product code.
 *
 * CPU restatement of the reference's membrane-surface hot path (see
 * umcp_oracle.h). Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline leg load this file's library, always as the checker.
 *
 * Energy per quadrature point follows surface::fenergy / ifenergy
 * (src/interpLib.C:3641-3881, 3426-3639) with the reference's compile-time
 * model: FIXED_A, LOCAL_LIPID_ENERGY, GLOBAL_AREA and MICRO_KA off
 * (src/local_config.h:14-24). The gradient follows surface::grad / igrad
 * (src/grad.C:65-942, 6445-7457): the same intermediate variables (c1, c2
 * from the shape operator entries a,b,c,d; g; the normal), chained backward
 * in reverse order instead of the reference's forward-expanded products.
 */
#include "umcp_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define SAFETY 1e-12                       /* src/interp.h:14 */
#define ORACLE_PI 3.14159265358979323846
#define AKMA_TIME (1.0 / (0.04888 * 1e-12)) /* src/units.h:5 */

static void cross3(const double *a, const double *b, double *c)
{
	c[0] = a[1] * b[2] - a[2] * b[1];
	c[1] = a[2] * b[0] - a[0] * b[2];
	c[2] = a[0] * b[1] - a[1] * b[0];
}
static double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

typedef struct {
	int ncp, npt, irregular;
	const int *cp;
	const signed char *img;
	const double *rows; /* [6][npt][ncp] */
	const double *w;
	const double *g0, *rr0;
	const double *outer, *inner;
	double dudv;
} face_view;

static face_view face_at(const oracle_surface *s, int f)
{
	face_view v;
	if (f < s->nreg) {
		v.ncp = 12; v.npt = 15; v.irregular = 0;
		v.cp = s->reg_cp + 12 * f;
		v.img = s->reg_img + 36 * f;
		v.rows = s->reg_rows;
		v.w = s->reg_w;
		v.g0 = s->reg_g0 + 15 * f;
		v.rr0 = s->reg_rr0 + 15 * f;
		v.outer = s->reg_outer + s->ntypes * f;
		v.inner = s->reg_inner + s->ntypes * f;
		v.dudv = 0.5; /* src/interpLib.C:3808 */
	} else {
		int q = f - s->nreg, val = s->irr_val[q];
		v.ncp = val + 6; v.npt = 16; v.irregular = 1;
		v.cp = s->irr_cp + 13 * q;
		v.img = s->irr_img + 39 * q;
		v.rows = (val == 5) ? s->irr_rows5 : s->irr_rows7;
		v.w = (val == 5) ? s->irr_w5 : s->irr_w7;
		v.g0 = s->irr_g0 + 16 * q;
		v.rr0 = s->irr_rr0 + 16 * q;
		v.outer = s->irr_outer + s->ntypes * q;
		v.inner = s->irr_inner + s->ntypes * q;
		v.dudv = 1.0; /* src/interpLib.C:3575 */
	}
	return v;
}

/* Unscaled image position r[cp] + lattice shift, and its alpha-scaled form. */
static void control_points(const oracle_surface *s, const double *r, const face_view *F, double X[][3], double Xs[][3])
{
	const double *al = r + 3 * s->nv;
	for (int x = 0; x < F->ncp; x++)
		for (int c = 0; c < 3; c++) {
			double p = r[3 * F->cp[x] + c];
			for (int d = 0; d < 3; d++) p += F->img[3 * x + d] * s->box[d][c];
			X[x][c] = p;
			Xs[x][c] = al[c] * p;
		}
}

/* Contractions R_u, R_v, S_uu, S_uv, S_vv at point pt (src/interpLib.C:3680-3706). */
static void contract(const face_view *F, double Xs[][3], int pt, double K[5][3])
{
	for (int k = 0; k < 5; k++) {
		K[k][0] = K[k][1] = K[k][2] = 0.0;
		const double *row = F->rows + ((size_t)(k + 1) * F->npt + pt) * F->ncp;
		for (int x = 0; x < F->ncp; x++)
			for (int c = 0; c < 3; c++) K[k][c] += row[x] * Xs[x][c];
	}
}

static double energy_range(const oracle_surface *s, const double *r, double *terms, double *face_e, int f0, int f1)
{
	double VA = 0, VC = 0, VR = 0, E = 0;
	for (int f = f0; f < f1; f++) {
		face_view F = face_at(s, f);
		double X[13][3], Xs[13][3];
		control_points(s, r, &F, X, Xs);
		double ef = 0.0;
		for (int p = 0; p < F.npt; p++) {
			double K[5][3];
			contract(&F, Xs, p, K);
			double *Ru = K[0], *Rv = K[1], *Suu = K[2], *Suv = K[3], *Svv = K[4];
			double nrm[3];
			cross3(Ru, Rv, nrm);
			double nl = sqrt(dot3(nrm, nrm));
			nrm[0] /= nl; nrm[1] /= nl; nrm[2] /= nl;
			double RuRu = dot3(Ru, Ru), RuRv = dot3(Ru, Rv), RvRv = dot3(Rv, Rv);
			double g = sqrt(RuRu * RvRv - RuRv * RuRv);
			double nsuu = dot3(Suu, nrm), nsuv = dot3(Suv, nrm), nsvv = dot3(Svv, nrm);
			double ig2 = 1.0 / (g * g);
			double a = ig2 * (nsuu * RvRv - nsuv * RuRv), b = ig2 * (nsuv * RvRv - nsvv * RuRv);
			double c = ig2 * (nsuv * RuRu - nsuu * RuRv), d = ig2 * (nsvv * RuRu - nsuv * RuRv);
			double sq = sqrt(SAFETY + a * a + 4 * b * c - 2 * a * d + d * d);
			double c1 = -0.5 * (a + d - sq), c2 = -0.5 * (a + d + sq);
			double w = F.w[p], g0 = F.g0[p];
			double en = s->kg * c1 * c2; /* LOCAL_LIPID_ENERGY: kg term only (:3834) */
			double dAf = g0 * w;          /* FIXED_A (:3843) */
			double A = F.dudv * g * w, A0 = F.dudv * g0 * w;
			double val = RuRv / sqrt(RuRu * RvRv);
			double er = s->k_reg * (val - F.rr0[p]) * (val - F.rr0[p]);
			double lec = 0.0; /* lipid-area bending, no dudv (src/interpLib.C:3832-3834) */
			for (int x = 0; x < s->ntypes; x++) {
				double dco = (c1 + c2 - s->lipid_c0[x]), dci = (-c1 - c2 - s->lipid_c0[x]);
				lec += 0.5 * s->kc * dco * dco * F.outer[x] * 0.5 * w;
				lec += 0.5 * s->kc * dci * dci * F.inner[x] * 0.5 * w;
			}
			double ea = 2 * 0.5 * A0 * s->KA * ((A - A0) / A0) * ((A - A0) / A0);
			double eb = lec + F.dudv * dAf * en;
			VR += er; VC += eb; VA += ea;
			ef += er + eb + ea;
		}
		if (face_e) face_e[f - f0] = ef;
		E += ef;
	}
	if (terms) { terms[0] = VA; terms[1] = VC; terms[2] = VR; }
	return E;
}

double oracle_energy(const oracle_surface *s, const double *r, double *terms, double *face_e)
{
	return energy_range(s, r, terms, face_e, 0, s->nreg + s->nirr);
}

double oracle_energy_faces(const oracle_surface *s, const double *r, int f0, int f1)
{
	return energy_range(s, r, NULL, NULL, f0, f1);
}

static void grad_range(const oracle_surface *s, const double *r, double *gr, int f0, int f1)
{
	const int nv = s->nv;
	const double *al = r + 3 * nv;
	for (int f = f0; f < f1; f++) {
		face_view F = face_at(s, f);
		double X[13][3], Xs[13][3];
		control_points(s, r, &F, X, Xs);
		for (int p = 0; p < F.npt; p++) {
			double K[5][3];
			contract(&F, Xs, p, K);
			double *Ru = K[0], *Rv = K[1], *Suu = K[2], *Suv = K[3], *Svv = K[4];
			double m[3];
			cross3(Ru, Rv, m);
			double ml = sqrt(dot3(m, m));
			double nrm[3] = {m[0] / ml, m[1] / ml, m[2] / ml};
			double RuRu = dot3(Ru, Ru), RuRv = dot3(Ru, Rv), RvRv = dot3(Rv, Rv);
			double g = sqrt(RuRu * RvRv - RuRv * RuRv);
			double nsuu = dot3(Suu, nrm), nsuv = dot3(Suv, nrm), nsvv = dot3(Svv, nrm);
			double g2 = g * g, ig2 = 1.0 / g2;
			double a = ig2 * (nsuu * RvRv - nsuv * RuRv), b = ig2 * (nsuv * RvRv - nsvv * RuRv);
			double c = ig2 * (nsuv * RuRu - nsuu * RuRv), d = ig2 * (nsvv * RuRu - nsuv * RuRv);
			double sq = sqrt(SAFETY + a * a + 4 * b * c - 2 * a * d + d * d);
			double e1 = -0.5 * (a + d - sq), e2 = -0.5 * (a + d + sq);
			double w = F.w[p], g0 = F.g0[p];
			double dAf = g0 * w;
			double A = F.dudv * g * w, A0 = F.dudv * g0 * w;

			/* Energy partials (src/grad.C:401-466). */
			double de_dc1 = 0, de_dc2 = 0, de_dg = 0;
			for (int x = 0; x < s->ntypes; x++) {
				double dco = (e1 + e2 - s->lipid_c0[x]), dci = (-e1 - e2 - s->lipid_c0[x]);
				double t = s->kc * dco * 0.5 * F.outer[x] * w - s->kc * dci * 0.5 * F.inner[x] * w;
				de_dc1 += t;
				de_dc2 += t;
			}
			de_dc1 += s->kg * e2 * F.dudv * dAf;
			de_dc2 += s->kg * e1 * F.dudv * dAf;
			de_dg += 2 * s->KA * ((A - A0) / A0) * w * F.dudv;

			/* c1, c2 -> a,b,c,d (src/grad.C:383-400). */
			double ad = (a - d) / sq;
			double dc1_da = -0.5 * (1 - ad), dc1_db = c / sq, dc1_dc = b / sq, dc1_dd = -0.5 * (1 + ad);
			double dc2_da = -0.5 * (1 + ad), dc2_db = -c / sq, dc2_dc = -b / sq, dc2_dd = -0.5 * (1 - ad);
			double abar = de_dc1 * dc1_da + de_dc2 * dc2_da, bbar = de_dc1 * dc1_db + de_dc2 * dc2_db;
			double cbar = de_dc1 * dc1_dc + de_dc2 * dc2_dc, dbar = de_dc1 * dc1_dd + de_dc2 * dc2_dd;

			/* a,b,c,d -> g, n.S, first fundamental form (src/grad.C:361-381). */
			double gbar = de_dg - 2.0 / g * (abar * a + bbar * b + cbar * c + dbar * d);
			double nuu_bar = ig2 * (abar * RvRv - cbar * RuRv);
			double nuv_bar = ig2 * (-abar * RuRv + bbar * RvRv + cbar * RuRu - dbar * RuRv);
			double nvv_bar = ig2 * (-bbar * RuRv + dbar * RuRu);
			double EE_bar = ig2 * (cbar * nsuv + dbar * nsvv);                              /* RuRu */
			double EF_bar = ig2 * (-abar * nsuv - bbar * nsvv - cbar * nsuu - dbar * nsuv); /* RuRv */
			double GG_bar = ig2 * (abar * nsuu + bbar * nsuv);                              /* RvRv */
			/* g = sqrt(RuRu RvRv - RuRv^2) (src/grad.C:352-354). */
			EE_bar += gbar * RvRv / (2 * g);
			EF_bar += -gbar * RuRv / g;
			GG_bar += gbar * RuRu / (2 * g);
			/* k_reg angle term (src/grad.C:560-568), kept apart for igrad's alpha quirk. */
			double val = RuRv / sqrt(RuRu * RvRv);
			double vbar = 2 * s->k_reg * (val - F.rr0[p]);
			double rEE = -vbar * val / (2 * RuRu), rEF = vbar / sqrt(RuRu * RvRv), rGG = -vbar * val / (2 * RvRv);

			double Kb[5][3], Kreg[2][3];
			for (int q = 0; q < 3; q++) {
				Kb[0][q] = 2 * EE_bar * Ru[q] + EF_bar * Rv[q];
				Kb[1][q] = 2 * GG_bar * Rv[q] + EF_bar * Ru[q];
				Kreg[0][q] = 2 * rEE * Ru[q] + rEF * Rv[q];
				Kreg[1][q] = 2 * rGG * Rv[q] + rEF * Ru[q];
				Kb[2][q] = nuu_bar * nrm[q];
				Kb[3][q] = nuv_bar * nrm[q];
				Kb[4][q] = nvv_bar * nrm[q];
			}
			/* normal n = m/|m|, m = Ru x Rv (src/grad.C:470-494). */
			double nbar[3], mbar[3], t[3];
			for (int q = 0; q < 3; q++) nbar[q] = nuu_bar * Suu[q] + nuv_bar * Suv[q] + nvv_bar * Svv[q];
			double nn = dot3(nbar, nrm);
			for (int q = 0; q < 3; q++) mbar[q] = (nbar[q] - nn * nrm[q]) / ml;
			cross3(Rv, mbar, t);
			for (int q = 0; q < 3; q++) Kb[0][q] += t[q];
			cross3(mbar, Ru, t);
			for (int q = 0; q < 3; q++) Kb[1][q] += t[q];

			/* Scatter (src/grad.C:863-930; igrad :7390-7450). */
			for (int x = 0; x < F.ncp; x++) {
				double dedr[3] = {0, 0, 0}, dreg[3] = {0, 0, 0};
				for (int k = 0; k < 5; k++) {
					double bk = F.rows[((size_t)(k + 1) * F.npt + p) * F.ncp + x];
					for (int q = 0; q < 3; q++) dedr[q] += bk * Kb[k][q];
				}
				for (int k = 0; k < 2; k++) {
					double bk = F.rows[((size_t)(k + 1) * F.npt + p) * F.ncp + x];
					for (int q = 0; q < 3; q++) dreg[q] += bk * Kreg[k][q];
				}
				for (int q = 0; q < 3; q++) {
					gr[3 * F.cp[x] + q] += (dedr[q] + dreg[q]) * al[q];
					/* igrad adds the k_reg part to the box-scale derivative with an
					 * extra alpha factor (src/grad.C:7414-7421). */
					double dreg_alpha = F.irregular ? dreg[q] * al[q] : dreg[q];
					gr[3 * nv + q] += (dedr[q] + dreg_alpha) * X[x][q];
				}
			}
		}
	}
}

void oracle_grad(const oracle_surface *s, const double *r, double *gr)
{
	grad_range(s, r, gr, 0, s->nreg + s->nirr);
}

void oracle_grad_faces(const oracle_surface *s, const double *r, double *gr, int f0, int f1)
{
	grad_range(s, r, gr, f0, f1);
}

void oracle_sparse_apply(int nrow, const int *row_ptr, const int *col, const double *val,
                         const double *scalev, double scale, const double *alphas,
                         const double *in, double *out)
{
	/* SparseMatrix::mult per component (src/sparse.C:941-953), then the
	 * scale / alpha_c^2 (and optional per-row factor) of src/parallel.C:1053-1065. */
	for (int c = 0; c < 3; c++)
		for (int i = 0; i < nrow; i++) {
			double acc = 0.0;
			for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++) acc += val[k] * in[3 * col[k] + c];
			double f = scale / (alphas[c] * alphas[c]);
			if (scalev) f = scalev[c * nrow + i] * scale / (alphas[c] * alphas[c]);
			out[3 * i + c] += acc * f;
		}
}

static void minv_apply(const oracle_step_params *p, int nv, const double *in, double *out)
{
	const double one[3] = {1, 1, 1};
	if (p->row_ptr) oracle_sparse_apply(p->nrow, p->row_ptr, p->col, p->val, NULL, 1.0, one, in, out);
	else
		for (int i = 0; i < 3 * nv; i++) out[i] += in[i];
}

void oracle_step(const oracle_step_params *p, int nv, double *r, double *pmom, const double *g, const double *noise)
{
	if (p->mode == 0) {
		/* Overdamped BD: r += -(D/kT) g dt + sqrt(2 D dt) xi (mode-space form of src/bd.C:1028-1038). */
		double mob = p->D * p->dt / p->kT, sig = sqrt(2.0 * p->D * p->dt);
		for (int i = 0; i < 3 * nv; i++) r[i] += -mob * g[i] + sig * noise[i];
		return;
	}
	/* Leapfrog of src/hd.C:1540-1720 (no particles: qdot_temp = 0). */
	const double AK = AKMA_TIME * p->dt;
	const double sig = sqrt(2.0 * p->gamma * p->kT * AK);
	for (int i = 0; i < 3 * nv; i++) {
		double pp = pmom[i];
		if (p->mode == 2) pp -= p->gamma * AK * pp;             /* friction (:1555-1556) */
		pp += -g[i] * AK / 2;                                     /* half kick (:1600-1605) */
		if (p->mode == 1) pp += (1.0 / p->gamma) * sig * noise[i] / AK; /* BD noise (:1653-1660) */
		else pp += sig * noise[i];                                /* LD noise (:1669-1673) */
		pp += -g[i] * AK / 2;                                     /* half kick (:1686-1693) */
		pmom[i] = pp;
	}
	/* qdot = M^-1 p, r += qdot AK (:1700-1720) */
	double *qdot = (double *)calloc((size_t)3 * nv, sizeof(double));
	minv_apply(p, nv, pmom, qdot);
	for (int i = 0; i < 3 * nv; i++) r[i] += qdot[i] * AK;
	free(qdot);
	if (p->mode == 1) memset(pmom, 0, sizeof(double) * 3 * (size_t)nv); /* BD reset (:1943-1947) */
}

/* Philox4x32-10 (Salmon et al., SC'11) and the normal draws of the GPU integrator. */
static void philox(uint32_t c[4], uint32_t k0, uint32_t k1)
{
	for (int round = 0; round < 10; round++) {
		uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
		uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
		uint32_t n0 = hi1 ^ c[1] ^ k0, n1 = lo1, n2 = hi0 ^ c[3] ^ k1, n3 = lo0;
		c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
		k0 += 0x9E3779B9u;
		k1 += 0xBB67AE85u;
	}
}
static double u53(uint32_t a, uint32_t b)
{
	uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
	return ((double)m + 0.5) * (1.0 / 9007199254740992.0);
}

void oracle_noise(unsigned long long seed, unsigned int stream, unsigned long long step, int nv, double *out)
{
	for (int v = 0; v < nv; v++) {
		for (int half = 0; half < 2; half++) {
			uint32_t c[4] = {(uint32_t)v, (uint32_t)step, (uint32_t)(step >> 32), stream | (half ? 0x80000000u : 0u)};
			philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
			double u1 = u53(c[0], c[1]), u2 = u53(c[2], c[3]);
			double rad = sqrt(-2.0 * log(u1));
			if (half == 0) {
				out[3 * v + 0] = rad * cos(2.0 * ORACLE_PI * u2);
				out[3 * v + 1] = rad * sin(2.0 * ORACLE_PI * u2);
			} else {
				out[3 * v + 2] = rad * cos(2.0 * ORACLE_PI * u2);
			}
		}
	}
}
