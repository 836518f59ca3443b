/*
 * ORACLE - test infrastructure, not product code.
 *
 * CPU restatement (plain C) of the reference's membrane-surface hot path,
 * used only by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline
 * leg as the checker. Each function cites the reference file:line it follows.
 * Pinned against the reference's own code compiled here (oracle/ref, output
 * oracle/_ref) through the committed fixtures under tests/golden/.
 */
#ifndef UMCP_ORACLE_H
#define UMCP_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* One surface as the reference's formula arrays describe it, flattened:
 * per face the control points cp[ncp] and their lattice images img[ncp][3],
 * per point g0/RuRv0, per face the leaflet composition areas per lipid type,
 * and shared basis rows per patch type rows[kind=0..5][pt][ncp] + weights. */
typedef struct {
  int nv;
  double box[3][3];
  double kc, KA, kg, k_reg;
  int ntypes;
  const double *lipid_c0;      /* [ntypes] */
  /* regular faces (valence-6 corner, 12 control points, 15 points, dudv 0.5) */
  int nreg;
  const int *reg_cp;           /* [nreg*12] */
  const signed char *reg_img;  /* [nreg*12*3] */
  const double *reg_rows;      /* [6*15*12] */
  const double *reg_w;         /* [15] */
  const double *reg_g0, *reg_rr0;       /* [nreg*15] */
  const double *reg_outer, *reg_inner;  /* [nreg*ntypes] */
  /* irregular faces (valence 5 or 7 corner, val+6 control points, 16 points, dudv 1) */
  int nirr;
  const int *irr_val;          /* [nirr] */
  const int *irr_cp;           /* [nirr*13], first val+6 used */
  const signed char *irr_img;  /* [nirr*13*3] */
  const double *irr_rows5, *irr_rows7;  /* [6*16*11], [6*16*13] */
  const double *irr_w5, *irr_w7;        /* [16] */
  const double *irr_g0, *irr_rr0;       /* [nirr*16] */
  const double *irr_outer, *irr_inner;  /* [nirr*ntypes] */
} oracle_surface;

/* surface::energy(r, NULL) (src/interpLib.C:4180-4352): r has 3*nv+3 entries
 * (xyz per vertex, then the box scales alpha_x,y,z). terms (may be NULL)
 * receives {VA, VC, VR}. face_e (may be NULL) receives per-face energies,
 * regular faces first. */
double oracle_energy(const oracle_surface *s, const double *r, double *terms, double *face_e);

/* surface::grad(r, g) (src/grad.C:65-942 + igrad :6445-7457): ADDS dE/dr
 * into g (3*nv+3 entries, last three the box-scale derivatives). */
void oracle_grad(const oracle_surface *s, const double *r, double *g);

/* The same two passes restricted to faces [f0, f1) (regular faces first,
 * then irregular), for a face-partitioned run over several processes as the
 * reference's MPI face partition does (src/parallel.C:137-387). */
double oracle_energy_faces(const oracle_surface *s, const double *r, int f0, int f1);
void oracle_grad_faces(const oracle_surface *s, const double *r, double *g, int f0, int f1);

/* AltSparseCartMatVecIncrScale (src/parallel.C:1028-1075) over a row-list
 * matrix in CSR form: out[3*row+c] += scale/alpha_c^2 * (scalev ? scalev[c*nrow+row] : 1)
 *                                     * sum_k val[k] * in[3*col[k]+c]. */
void oracle_sparse_apply(int nrow, const int *row_ptr, const int *col, const double *val,
                         const double *scalev, double scale, const double *alphas,
                         const double *in, double *out);

/* One step of the reference's membrane integrators (src/hd.C:1520-1720,
 * 1943-1947) with the mass matrix replaced by its action (Minv_apply) and
 * the Gaussian draws supplied (noise: 3*nv unit normals).
 * mode 0: overdamped BD  r += -(D/kT) g dt + sqrt(2 D dt) xi
 * mode 1: do_bd_membrane (p reset to 0 after the step)
 * mode 2: do_ld (Langevin leapfrog with friction gamma)
 * For modes 1/2 the matrix is the CSR effective inverse mass (NULL = identity). */
typedef struct {
  int mode;
  double dt;           /* time_step in the reference's units (ps); AKMA scaling applied inside */
  double gamma;        /* gamma_langevin */
  double kT;           /* kcal/mol */
  double D;            /* mode 0: diffusion coefficient (A^2 per dt unit) */
  int nrow; const int *row_ptr; const int *col; const double *val;
} oracle_step_params;

void oracle_step(const oracle_step_params *p, int nv, double *r, double *pmom, const double *g,
                 const double *noise);

/* Philox4x32-10 normal draws exactly as the GPU integrator makes them:
 * out[3*v+c] for vertices [0,nv) of stream `stream` at step `step`. */
void oracle_noise(unsigned long long seed, unsigned int stream, unsigned long long step, int nv, double *out);

#ifdef __cplusplus
}
#endif
#endif
