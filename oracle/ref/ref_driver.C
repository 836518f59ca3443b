/*
 * Oracle driver (test infrastructure, never shipped): runs the REFERENCE's own
 * membrane-surface code, compiled from its sources by oracle/ref/Makefile, and
 * dumps what it computes so the CPU restatement (oracle/umcp_oracle.c) and
 * the GPU path can be pinned against it.
 *
 * It follows the setup order of the reference's hd.C (src/hd.C:158-270):
 *   surface::loadLattice -> surface::generatePlan -> readLipidComposition
 *   -> r = vertex positions, alpha = 1 -> setg0(r)
 * then fills the serial face partition that setupParallel would build
 * (src/parallel.C:137) and calls surface::energy(r, NULL) and
 * surface::grad(r, g) as hd.C does in its dynamics loop (src/hd.C:1128,1240).
 *
 * Usage:
 *   ref_driver dump <mesh> <params> <positions.bin|-> <out_prefix>
 *   ref_driver time <mesh> <params> <positions.bin|-> <n_calls>
 *   ref_driver mass <mesh> <params> - <out_prefix>
 *   ref_driver sub6 - - - <out_prefix>
 *   ref_driver rnrm <mesh> <params> <positions.bin|-> <out_prefix>
 *     surface::evaluateRNRM at 7 fixed (u,v) on every face: face, u, v, R, N
 *   ref_driver min <mesh> <params> <positions.bin|-> <out_prefix>
 *     the reference's L-BFGS (src/l-bfgs.C) driven as Simulation::minimize
 *     drives it for one surface without particles (src/minimize.C:26-140,
 *     489-560): parameters {alpha, r, alpha}, alpha's gradient zeroed,
 *     100 iterations, 100 back vectors, max move 1.0; writes the energy
 *     before and after every iteration and the final positions
 *
 * "mass" sets up the mass points as hd.C does before a dynamics run
 * (src/hd.C:417-481: a 66-point grid per triangle, mass per point from
 * surface::area's area0), calls load_least_squares_fitting and
 * getSparseEffectiveMass (src/hd.C:740-751), and dumps the inverse effective
 * mass densely, the mass per point and the coefficients of every point.
 *
 * <params> holds "kc X", "KA X", "kg X", "k_reg X" lines and any
 * "lipid ..." lines (read by the reference's readLipidComposition).
 * <positions.bin> holds 3*nv+3 doubles (xyz per vertex, then alpha_x,y,z);
 * "-" keeps the mesh-file positions. setg0 always uses the mesh-file
 * positions (as hd.C does), so a positions file evaluates a deformed state.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>
#include <sys/time.h>
#include "interp.h"
#include "parallel.h"
#include "lagrange.h"
#include "sparse.h"
#include "units.h"
#include "l-bfgs.h"

extern double kc, KA, kg, k_reg;
extern double VA, VC, VR, AVC;
extern int setup_for_parallel;

static void read_params(const char *path)
{
	FILE *f = fopen(path, "r");
	if (!f) { fprintf(stderr, "cannot open params %s\n", path); exit(2); }
	char line[4096], key[256];
	double val;
	while (fgets(line, sizeof line, f)) {
		if (sscanf(line, "%255s %lf", key, &val) != 2) continue;
		if (!strcasecmp(key, "kc")) kc = val;
		else if (!strcasecmp(key, "KA")) KA = val;
		else if (!strcasecmp(key, "kg")) kg = val;
		else if (!strcasecmp(key, "k_reg")) k_reg = val;
	}
	fclose(f);
}

static surface *setup(const char *mesh, const char *params, double **r_out)
{
	read_params(params);
	surface *s = (surface *)calloc(1, sizeof(surface));
	s->surface_id = 0;
	s->loadLattice(mesh, 0.);
	fprintf(stderr, "ref_driver: loaded %d vertices\n", s->nv);
	s->generatePlan();
	fprintf(stderr, "ref_driver: plan %d regular, %d irregular faces\n", s->nf_faces, s->nf_irr_faces);
	FILE *pf = fopen(params, "r");
	s->readLipidComposition(pf);
	if (pf) fclose(pf);
	int nv = s->nv;
	double *r = (double *)calloc(3 * nv + 3, sizeof(double));
	s->get(r);
	r[3 * nv + 0] = r[3 * nv + 1] = r[3 * nv + 2] = 1.0;
	s->setg0(r);
	fprintf(stderr, "ref_driver: reference state set\n");

	/* Serial face partition: every face on rank 0 (what setupParallel's
	 * balanced partition reduces to for one process). */
	setup_for_parallel = 1;
	par_info.nSurfaces = 1;
	par_info.my_id = 0;
	par_info.nprocs = 1;
	par_info.faces = (int **)malloc(sizeof(int *));
	par_info.nf = (int *)malloc(sizeof(int));
	int nfaces = s->nf_faces + s->nf_irr_faces;
	par_info.faces[0] = (int *)malloc(sizeof(int) * nfaces);
	for (int f = 0; f < nfaces; f++) par_info.faces[0][f] = f;
	par_info.nf[0] = nfaces;
	par_info.nc = 0;
	*r_out = r;
	return s;
}

static void load_positions(const char *path, double *r, int nv)
{
	if (!strcmp(path, "-")) return;
	FILE *f = fopen(path, "rb");
	if (!f) { fprintf(stderr, "cannot open positions %s\n", path); exit(2); }
	size_t n = fread(r, sizeof(double), 3 * nv + 3, f);
	fclose(f);
	if (n != (size_t)(3 * nv + 3)) { fprintf(stderr, "positions file too short\n"); exit(2); }
}

static FILE *open_out(const char *prefix, const char *suffix, const char *mode)
{
	char name[4096];
	snprintf(name, sizeof name, "%s.%s", prefix, suffix);
	FILE *f = fopen(name, mode);
	if (!f) { fprintf(stderr, "cannot write %s\n", name); exit(2); }
	return f;
}

static void dump_formulas(FILE *f, formula *frm, int n)
{
	/* Per point: ncoor, tri, cp[ncoor], then doubles: weight, g0, RuRv0,
	 * r_pbc[3*ncoor], r_w, r_u, r_v, r_uu, r_uv, r_vv [ncoor each]. */
	for (int i = 0; i < n; i++) {
		int hdr[2] = {frm[i].ncoor, frm[i].tri};
		fwrite(hdr, sizeof(int), 2, f);
		fwrite(frm[i].cp, sizeof(int), frm[i].ncoor, f);
		double d[3] = {frm[i].weight, frm[i].g0, frm[i].RuRv0};
		fwrite(d, sizeof(double), 3, f);
		fwrite(frm[i].r_pbc, sizeof(double), 3 * frm[i].ncoor, f);
		fwrite(frm[i].r_w, sizeof(double), frm[i].ncoor, f);
		fwrite(frm[i].r_u, sizeof(double), frm[i].ncoor, f);
		fwrite(frm[i].r_v, sizeof(double), frm[i].ncoor, f);
		fwrite(frm[i].r_uu, sizeof(double), frm[i].ncoor, f);
		fwrite(frm[i].r_uv, sizeof(double), frm[i].ncoor, f);
		fwrite(frm[i].r_vv, sizeof(double), frm[i].ncoor, f);
	}
}

void fast_sub6_0(double *r_in, double *r_out);
void fast_sub6_1(double *r_in, double *r_out);
void fast_sub6_2(double *r_in, double *r_out);
void fast_sub6_3(double *r_in, double *r_out);

/* Simulation::minimize's objective for one surface without particles
 * (src/minimize.C:26-140): p = {alpha_x,y,z, r[3 nv], alpha copy}. */
static surface *min_surface = NULL;
static int min_nv = 0;

static double min_f(double *p)
{
	int nv = min_nv;
	p[3 + 3 * nv + 0] = p[0];
	p[3 + 3 * nv + 1] = p[1];
	p[3 + 3 * nv + 2] = p[2];
	return min_surface->energy(p + 3, NULL);
}

static double min_fdf(double *p, double *g)
{
	int nv = min_nv, n = 3 * nv + 6;
	memset(g, 0, sizeof(double) * n);
	p[3 + 3 * nv + 0] = p[0];
	p[3 + 3 * nv + 1] = p[1];
	p[3 + 3 * nv + 2] = p[2];
	min_surface->grad(p + 3, g + 3);
	g[0] = g[1] = g[2] = 0;
	g[3 + 3 * nv + 0] = g[3 + 3 * nv + 1] = g[3 + 3 * nv + 2] = 0;
	return min_surface->energy(p + 3, NULL);
}

int main(int argc, char **argv)
{
	if (argc >= 6 && !strcmp(argv[1], "sub6")) {
		/* The reference's four child stencils (src/fast_mm.C) as 36 x 36
		 * matrices: column j is the image of unit vector j. */
		void (*fn[4])(double *, double *) = {fast_sub6_0, fast_sub6_1, fast_sub6_2, fast_sub6_3};
		FILE *f = open_out(argv[5], "sub6.bin", "wb");
		for (int k = 0; k < 4; k++)
			for (int j = 0; j < 36; j++) {
				double in[36] = {0}, out[36] = {0};
				in[j] = 1.0;
				fn[k](in, out);
				fwrite(out, sizeof(double), 36, f);
			}
		fclose(f);
		return 0;
	}
	if (argc < 6) {
		fprintf(stderr, "usage: %s dump|time <mesh> <params> <positions|-> <out_prefix|n_calls>\n", argv[0]);
		return 2;
	}
	double *r = NULL;
	surface *s = setup(argv[2], argv[3], &r);
	int nv = s->nv;
	load_positions(argv[4], r, nv);
	double *g = (double *)calloc(3 * nv + 3, sizeof(double));

	if (!strcmp(argv[1], "rnrm")) {
		const double uvs[7][2] = {{1.0 / 3, 1.0 / 3}, {0.1, 0.2}, {0.7, 0.1}, {0.05, 0.05}, {0.0, 0.5}, {0.25, 0.0}, {0.45, 0.45}};
		FILE *f = open_out(argv[5], "rnrm.bin", "wb");
		for (int fc = 0; fc < s->nf_faces + s->nf_irr_faces; fc++)
			for (int q = 0; q < 7; q++) {
				double rp[3], nrm[3], rec[9];
				s->evaluateRNRM(fc, uvs[q][0], uvs[q][1], rp, nrm, r);
				rec[0] = fc; rec[1] = uvs[q][0]; rec[2] = uvs[q][1];
				for (int c = 0; c < 3; c++) { rec[3 + c] = rp[c]; rec[6 + c] = nrm[c]; }
				fwrite(rec, sizeof(double), 9, f);
			}
		fclose(f);
		return 0;
	}

	if (!strcmp(argv[1], "mass")) {
		const int plim = 10, ppf = (plim + 1) * (plim + 2) / 2;
		force_set fs;
		memset(&fs, 0, sizeof fs);
		fs.npts = ppf * s->nt;
		fs.face_set = (int *)malloc(sizeof(int) * fs.npts);
		fs.uv_set = (double *)malloc(sizeof(double) * 2 * fs.npts);
		fs.mass = (double *)malloc(sizeof(double) * fs.npts);
		double cur_area = 0, area0 = 0;
		s->area(r, -1, &cur_area, &area0);
		const double mass_per_lipid = 5 * 1000 * 760.09 / 6.022e23 / 1000;
		const double mass_per_pt = AMU_PER_KG * 2 * area0 / (s->nf_faces + s->nf_irr_faces) / ppf * mass_per_lipid / 65.35;
		int p = 0;
		for (int t = 0; t < s->nt; t++)
			for (int fi = 0; fi <= plim; fi++)
				for (int fj = 0; fj <= plim - fi; fj++, p++) {
					fs.face_set[p] = s->theTriangles[t].f;
					fs.uv_set[2 * p] = fi / (double)plim;
					fs.uv_set[2 * p + 1] = fj / (double)plim;
					fs.mass[p] = mass_per_pt;
				}
		s->load_least_squares_fitting(&fs);
		/* serial vertex partition (what setupParallel gives one process) */
		par_info.nv = (int *)malloc(sizeof(int));
		par_info.verts = (int **)malloc(sizeof(int *));
		par_info.nv[0] = nv;
		par_info.verts[0] = (int *)malloc(sizeof(int) * nv);
		for (int v = 0; v < nv; v++) par_info.verts[0][v] = v;
		int *use = (int *)malloc(sizeof(int) * nv), nuse = 0;
		SparseMatrix *M = NULL;
		s->getSparseEffectiveMass(&fs, use, &nuse, &M, NULL, nv, NULL);
		double *dense = (double *)calloc((size_t)nv * nv, sizeof(double));
		for (int a = 0; a < M->nneed; a++)
			for (int x = 0; x < M->nnz[a]; x++)
				dense[(size_t)M->need_list[a] * nv + M->source_list[M->nzl[a][x]]] = M->nzv[a][x];
		FILE *f = open_out(argv[5], "mass.txt", "w");
		fprintf(f, "area0 %.17e\nmass_per_pt %.17e\nnpts %d\nnuse %d\nnt %d\n", area0, mass_per_pt, fs.npts, nuse, s->nt);
		fclose(f);
		f = open_out(argv[5], "minv.bin", "wb");
		fwrite(dense, sizeof(double), (size_t)nv * nv, f);
		fclose(f);
		/* per point: face, u, v, ncoef, then 13 vertex ids and 13 coefficients (zero padded) */
		f = open_out(argv[5], "coef.bin", "wb");
		for (int q = 0; q < fs.npts; q++) {
			int hdr[2] = {fs.face_set[q], fs.frc_ncoef[q]};
			fwrite(hdr, sizeof(int), 2, f);
			fwrite(&fs.uv_set[2 * q], sizeof(double), 2, f);
			int ids[13] = {0};
			double cf[13] = {0};
			for (int c = 0; c < fs.frc_ncoef[q]; c++) {
				ids[c] = fs.frc_coef_list[q * 13 + c];
				cf[c] = fs.frc_coef[q * 13 + c];
			}
			fwrite(ids, sizeof(int), 13, f);
			fwrite(cf, sizeof(double), 13, f);
		}
		fclose(f);
		printf("mass_per_pt %.17e nuse %d\n", mass_per_pt, nuse);
		return 0;
	}

	if (!strcmp(argv[1], "min")) {
		const int nsteps = 100, n = 3 * nv + 6;
		min_surface = s;
		min_nv = nv;
		double *p = (double *)calloc(n, sizeof(double));
		double *gp = (double *)calloc(n, sizeof(double));
		p[0] = r[3 * nv]; p[1] = r[3 * nv + 1]; p[2] = r[3 * nv + 2];
		memcpy(p + 3, r, sizeof(double) * 3 * nv);
		min_fdf(p, gp);
		double mag = 0;
		for (int i = 0; i < n; i++) mag += gp[i] * gp[i];
		int use_m = nsteps < n ? nsteps : n;
		FILE *f = open_out(argv[5], "min_energy.bin", "wb");
		double e = min_f(p);
		fwrite(&e, sizeof(double), 1, f);
		l_bfgs_setup(use_m, n, p, 1.0, min_f, min_fdf);
		int done = 0;
		if (mag > 1e-20)
			for (int x = 0; x < nsteps; x++) {
				if (!l_bfgs_iteration(p)) break;
				e = min_f(p);
				fwrite(&e, sizeof(double), 1, f);
				done++;
			}
		l_bfgs_clear();
		fclose(f);
		memcpy(r, p + 3, sizeof(double) * 3 * nv);
		f = open_out(argv[5], "min_positions.bin", "wb");
		fwrite(r, sizeof(double), 3 * nv + 3, f);
		fclose(f);
		printf("iterations %d E %.17e\n", done, e);
		return 0;
	}

	if (!strcmp(argv[1], "time")) {
		int ncalls = atoi(argv[5]);
		struct timeval t0, t1;
		gettimeofday(&t0, NULL);
		double esum = 0;
		for (int c = 0; c < ncalls; c++) {
			esum += s->energy(r, NULL);
			memset(g, 0, sizeof(double) * (3 * nv + 3));
			s->grad(r, g);
		}
		gettimeofday(&t1, NULL);
		double dt = (t1.tv_sec - t0.tv_sec) + 1e-6 * (t1.tv_usec - t0.tv_usec);
		printf("{\"nv\": %d, \"calls\": %d, \"seconds\": %.6f, \"energy\": %.17e}\n", nv, ncalls, dt, esum / ncalls);
		return 0;
	}

	double E = s->energy(r, NULL);
	double va = VA, vc = VC, vr = VR;
	s->grad(r, g);

	const char *pre = argv[5];
	FILE *f = open_out(pre, "energy.txt", "w");
	fprintf(f, "E %.17e\nVA %.17e\nVC %.17e\nVR %.17e\nnv %d\nnf_faces %d\nnf_irr_faces %d\nnf_g_q_p %d\nnf_irr_pts %d\nnt %d\n",
	        E, va, vc, vr, nv, s->nf_faces, s->nf_irr_faces, s->nf_g_q_p, s->nf_irr_pts, s->nt);
	fclose(f);

	f = open_out(pre, "grad.bin", "wb");
	fwrite(g, sizeof(double), 3 * nv + 3, f);
	fclose(f);

	f = open_out(pre, "positions.bin", "wb");
	fwrite(r, sizeof(double), 3 * nv + 3, f);
	fclose(f);

	/* Per-face energy, in the reference's face numbering. */
	f = open_out(pre, "face_energy.bin", "wb");
	for (int fx = 0; fx < s->nf_faces + s->nf_irr_faces; fx++) {
		double e = s->faceEnergy(fx, r, NULL, 0);
		fwrite(&e, sizeof(double), 1, f);
	}
	fclose(f);

	f = open_out(pre, "plan_reg.bin", "wb");
	dump_formulas(f, s->theFormulas, s->nf_faces * s->nf_g_q_p);
	fclose(f);
	f = open_out(pre, "plan_irr.bin", "wb");
	dump_formulas(f, s->theIrregularFormulas, s->nf_irr_faces * s->nf_irr_pts);
	fclose(f);

	/* Triangle compositions (outer, inner leaflet areas per lipid type). */
	f = open_out(pre, "composition.txt", "w");
	fprintf(f, "ntypes %d\n", s->bilayerComp.nlipidTypes);
	for (int x = 0; x < s->bilayerComp.nlipidTypes; x++)
		fprintf(f, "type %d %s c0 %.17e APL %.17e\n", x, s->bilayerComp.names[x], s->bilayerComp.c0[x], s->bilayerComp.APL[x]);
	for (int t = 0; t < s->nt; t++) {
		fprintf(f, "tri %d %d %d %d", t, s->theTriangles[t].ids[0], s->theTriangles[t].ids[1], s->theTriangles[t].ids[2]);
		for (int x = 0; x < s->bilayerComp.nlipidTypes; x++)
			fprintf(f, " %.17e %.17e", s->theTriangles[t].composition.outerLeaflet[x], s->theTriangles[t].composition.innerLeaflet[x]);
		fprintf(f, "\n");
	}
	fclose(f);

	/* Final (oriented) neighbour order of every vertex. */
	f = open_out(pre, "edges.txt", "w");
	for (int i = 0; i < nv; i++) {
		fprintf(f, "%d %d", i, s->theVertices[i].valence);
		for (int e = 0; e < s->theVertices[i].valence; e++) fprintf(f, " %d", s->theVertices[i].edges[e]);
		fprintf(f, "\n");
	}
	fclose(f);
	printf("E %.17e\n", E);
	return 0;
}
