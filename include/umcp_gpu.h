/*
 * umcp_gpu.h - C ABI of the GB300 membrane-surface engine.
 *
 * Drop-in replacement for the hot path of UMCP's `struct surface`
 * (src/interp.h:210-552): the Loop limit-surface Helfrich energy and its
 * gradient, the effective-mass apply and the membrane integrators. Plain C
 * types only; every call returns a umcp_status and never exits the process
 * (the reference prints and calls exit(1), e.g. src/grad.C:67-72).
 *
 * Threading: a umcp_ctx owns one CUDA stream on one device; calls on a ctx
 * (and on meshes made from it) are serialised on that stream. Use one ctx
 * per host thread. Host-pointer calls copy in and out; *_device calls take
 * device pointers that live on the ctx's device.
 */
#ifndef UMCP_GPU_H
#define UMCP_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  UMCP_OK = 0,
  UMCP_ERR_INVALID = 1,     /* bad argument, malformed mesh or plan */
  UMCP_ERR_IO = 2,          /* file could not be read or written */
  UMCP_ERR_CUDA = 3,        /* CUDA runtime error (umcp_last_error has the text) */
  UMCP_ERR_NONFINITE = 4,   /* NaN/Inf in the energy ("nan en.", src/interpLib.C:3770-3774) */
  UMCP_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
  UMCP_ERR_NOMEM = 6,       /* device memory exhausted or over the admission budget */
  UMCP_ERR_UNSUPPORTED = 7, /* option the engine does not implement */
  UMCP_ERR_DIVERGED = 8     /* energy jump above the divergence threshold (src/hd.C:1280-1305) */
} umcp_status;

typedef enum { UMCP_FP64 = 0, UMCP_FP32_CENTRED = 1 } umcp_precision;

typedef struct umcp_ctx umcp_ctx;
typedef struct umcp_plan umcp_plan;   /* host-side plan: topology, basis rows, reference state */
typedef struct umcp_mesh umcp_mesh;   /* device-resident surface built from a plan */

/* Physical parameters, as the reference's input keywords (src/input.C:16-310). */
typedef struct {
  double kc;          /* bending modulus, kcal/mol ("kc", default 14) */
  double KA;          /* per-point area modulus ("KA", default -1 -> 0.215) */
  double kg;          /* Gaussian modulus ("kg", default 0) */
  double k_reg;       /* angle regulariser (global k_reg, default 0) */
  double temperature; /* K ("T", default 298) */
  int precision;      /* umcp_precision */
  const char *lipid_directives; /* text holding "lipid library|inner|outer ..." lines, or NULL */
  int face_kernel;    /* precision form, regular faces: 0 FP32 SIMT kernel (default, faster here),
                         1 tcgen05 tensor-core kernel (kind::f16 MMAs on fp16 hi/lo splits) */
} umcp_params;

/* Sizes of a plan. */
typedef struct {
  int nv;            /* vertices; state vectors have 3*nv+3 doubles (xyz..., alpha_x,y,z) */
  int n_regular;     /* faces whose lowest-index corner has valence 6 (12 control points, 15 points) */
  int n_irregular;   /* faces at a valence 5/7 corner (valence+6 control points, 16 points) */
  int n_lipid_types;
  double box[9];     /* periodic box vectors PBC_vec, row-major */
} umcp_plan_info;

/* ---- errors ---------------------------------------------------------- */
const char *umcp_last_error(void);           /* text of the last failure on this host thread */
const char *umcp_status_string(umcp_status s);

/* ---- parameters and synthetic meshes (host only) ---------------------- */
umcp_status umcp_params_default(umcp_params *p);
/* Replaces src/input.C keyword parsing for the hot-path keys: "kc", "KA",
 * "kg", "T", "k_reg", "lipid ..." lines; unknown keys are ignored. */
umcp_status umcp_params_from_input(const char *input_text, umcp_params *p, char *lipid_buf, size_t lipid_buf_len);

/* Icosahedron Loop-subdivided `level` times (original vertices first, so every
 * valence-5 vertex is its faces' lowest index), radius R, radial N(0,sigma)
 * noise from Philox(seed, vertex), box 3R; written in the .mesh format
 * (src/write_structures.C:473-530). */
umcp_status umcp_mesh_generate_icosphere(int level, double R, double sigma, uint64_t seed, const char *mesh_path);
/* nx*ny triangular lattice (ny even), spacing a, periodic box, height field
 * with a q^-4 spectrum of variance kT/(kc*Lx*Ly*q^4) for kc = kc_kT kT. */
umcp_status umcp_mesh_generate_planar(int nx, int ny, double a, double kc_kT, uint64_t seed, const char *mesh_path);

/* ---- plans (host only) ------------------------------------------------ */
/* surface::loadLattice + generatePlan + readLipidComposition + setg0 at the
 * mesh-file positions (src/interpLib.C:1144, 4998; src/lipid_composition.C:47;
 * src/interpLib.C:2969; order of src/hd.C:158-270). */
umcp_status umcp_plan_from_file(const char *mesh_path, const umcp_params *p, umcp_plan **out);
/* surface::setg0(r) (src/interpLib.C:2969-3390): r has 3*nv+3 doubles; the
 * box scales are ignored, as the reference ignores them there. */
umcp_status umcp_plan_set_reference(umcp_plan *plan, const double *r);
umcp_status umcp_plan_info_get(const umcp_plan *plan, umcp_plan_info *info);
/* Copies the positions the plan was built from (3*nv+3, alpha = 1). */
umcp_status umcp_plan_positions(const umcp_plan *plan, double *r);
/* Oriented neighbour rings (after the reference's orientation pass):
 * valence[nv], ring[sum valence]. */
umcp_status umcp_plan_rings(const umcp_plan *plan, int *valence, int *ring);
/* Face tables. kind: 0 regular, 1 irregular. Arrays may be NULL to skip.
 *   cp[nf*13], img[nf*13*3] (lattice image of each control point),
 *   valence[nf], g0[nf*npt], rr0[nf*npt], outer[nf*ntypes], inner[nf*ntypes] */
umcp_status umcp_plan_faces(const umcp_plan *plan, int kind, int *cp, int8_t *img, int *valence, double *g0,
                            double *rr0, double *outer, double *inner);
/* Basis rows of a patch type: valence 6 (15 points x 12) or 5/7 (16 points x
 * valence+6): rows[kind(w,u,v,uu,uv,vv)][pt][cp], weight[pt], u[pt], v[pt]. */
umcp_status umcp_plan_basis(const umcp_plan *plan, int valence, double *rows, double *weight, double *u, double *v);
/* Lipid types of the plan: c0[ntypes], apl[ntypes]. */
umcp_status umcp_plan_lipids(const umcp_plan *plan, double *c0, double *apl);
/* Limit-surface point at (u,v) of face `face` (regular faces first, then
 * irregular, the reference's face numbering) as weights coef[n] of vertices
 * ids[n] (surface::get_pt_coeffs, src/uv_map.C:14-195); n <= 13. */
umcp_status umcp_plan_point_coeffs(const umcp_plan *plan, int face, double u, double v, int *ids, double *coef,
                                   int *n);
/* Limit-surface points and unit normals (surface::evaluateRNRM,
 * src/interpLib.C:7936-8100) of state r (3*nv+3, box scales applied) at n
 * queries (faces[q], uv[2q], uv[2q+1]): R[3n], N[3n] (N may be NULL; the
 * normal of the surface before the box scaling, as the reference forms it). At an
 * extraordinary vertex itself the normal is NaN, as the reference leaves it;
 * the position there follows r, where the reference reads its stored vertex
 * positions. Host only. */
umcp_status umcp_plan_evaluate(const umcp_plan *plan, const double *r, int n, const int *faces, const double *uv,
                               double *R, double *N);
/* The same evaluation on the device, from a mesh's resident state, at every
 * face's lattice points (u, v) = (i/plim, j/plim), i + j <= plim (i outer):
 * R and N (host, 3 doubles per point, N may be NULL) hold the points of face
 * 0 first, then face 1, ... in the plan's face order. */
umcp_status umcp_limit_points(umcp_mesh *mesh, int plim, double *R, double *N);
/* surface::writeLimitingSurface (src/write_structures.C:660-715) of the
 * resident state: the xyz text the reference writes (a count line, a title
 * line, "C x y z" per point at %lf) with each face's three corners
 * (plim = 1), evaluated by umcp_limit_points. */
umcp_status umcp_write_limiting_surface(umcp_mesh *mesh, const char *path);
void umcp_plan_destroy(umcp_plan *plan);

/* ---- device context and meshes --------------------------------------- */
umcp_status umcp_ctx_create(int device, umcp_ctx **out);
/* Drops the caller's reference: the context (and its stream) lives on until
 * the last mesh or batch created on it is destroyed. */
void umcp_ctx_destroy(umcp_ctx *ctx);
umcp_status umcp_ctx_synchronize(umcp_ctx *ctx);
/* The cudaStream_t (as void*) every call on this ctx is queued on, so a
 * caller can order its own work (timing events, copies) with the engine's. */
umcp_status umcp_ctx_stream(umcp_ctx *ctx, void **stream);
/* Free and total device memory of the context's device (cudaMemGetInfo). */
umcp_status umcp_ctx_mem_info(umcp_ctx *ctx, size_t *free_bytes, size_t *total_bytes);

/* Upload a plan; the mesh keeps its own state buffers on the device. */
umcp_status umcp_mesh_create(umcp_ctx *ctx, const umcp_plan *plan, const umcp_params *p, umcp_mesh **out);
void umcp_mesh_destroy(umcp_mesh *mesh);
umcp_status umcp_mesh_set_params(umcp_mesh *mesh, const umcp_params *p);

/* surface::energy(r, NULL) (src/interpLib.C:4180-4352). terms (may be NULL)
 * receives {VA, VC, VR}: area, curvature (bending + Gaussian) and angle parts. */
umcp_status umcp_energy(umcp_mesh *mesh, const double *r, double *E, double *terms);
/* surface::grad(r, g) (src/grad.C:65): ADDS dE/dr into g (3*nv+3). */
umcp_status umcp_grad(umcp_mesh *mesh, const double *r, double *g);
/* Both in one pass: E and g (g accumulated). */
umcp_status umcp_energy_grad(umcp_mesh *mesh, const double *r, double *E, double *g);
/* Device-pointer form: d_r, d_g hold 3*nv+3 doubles; d_E one double; g accumulated. */
umcp_status umcp_energy_grad_device(umcp_mesh *mesh, const double *d_r, double *d_E, double *d_g);
/* Energy and gradient with NO device allocation at call time. This entry
 * point has no counterpart in the reference: it exists for callers that
 * cannot call cudaMalloc when they need the energy (inside another
 * framework's CUDA-graph capture, or under a device-memory budget owned by
 * another runtime). Same inputs and outputs as umcp_energy_grad_device (the
 * mesh's plan tables, made at set-up, plus the caller's d_r, d_E, d_g; g is
 * accumulated; d_E may be NULL, the energy then goes to the mesh's own
 * slot); every scratch buffer lives in one 32 MiB file-scope device array
 * that each GPU loading the library holds until exit. Meshes whose scratch
 * exceeds 32 MiB (about 110,000 faces in FP64, 190,000 in the FP32 form) are
 * rejected with UMCP_ERR_NOMEM. The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress), so make that first call
 * before any stream capture. All calls on one device share that device's
 * array and it keeps the last call's contents: calls whose work overlaps on
 * the GPU (e.g. from two streams) race. Queued on the mesh's ctx stream;
 * returns without waiting: a non-finite energy (or a tensor-core wait that
 * gave up) is recorded in the mesh's status word, which
 * umcp_mesh_check_status reports. */
umcp_status umcp_energy_grad_static(umcp_mesh *mesh, const double *d_r, double *d_E, double *d_g);
/* Waits for the mesh's queued work and reports what its kernels recorded
 * since the last check: UMCP_ERR_NONFINITE (the reference's "nan en." stop,
 * src/interpLib.C:3770-3774), UMCP_ERR_DIVERGED (src/hd.C:1280-1305),
 * UMCP_ERR_TIMEOUT, or UMCP_OK; then clears the record. The status of the
 * asynchronous device-pointer calls (umcp_energy_grad_device,
 * umcp_energy_grad_static, umcp_run_async). */
umcp_status umcp_mesh_check_status(umcp_mesh *mesh);
/* Queues only the per-face pass (quadrature, pointwise energy and adjoint,
 * per-face gradient partials) on the mesh's resident state, without the
 * per-vertex gather or the sums: the unit a roofline measurement times. */
umcp_status umcp_face_pass(umcp_mesh *mesh);

/* Work sizes of a mesh: faces, quadrature points, gradient partial slots,
 * and kernels queued per integrator step (with and without a mass matrix). */
typedef struct {
  int nv, n_faces, n_points, n_slots;
  int kernels_per_step, kernels_per_step_mass;
  int precision;
  long long device_bytes;  /* device memory held by the mesh's buffers */
  long long h2d_bytes;     /* host-to-device bytes umcp_mesh_create copied (tables, bases, positions) */
  int mass_form;           /* installed M^-1: 0 none, 1 dense, 2 CSR */
} umcp_mesh_info;
umcp_status umcp_mesh_info_get(const umcp_mesh *mesh, umcp_mesh_info *info);
/* Device bytes umcp_mesh_create would allocate for this plan at this
 * precision, plus the energy record of an n_energies-step run: the
 * footprint a server admits jobs by. */
umcp_status umcp_plan_device_bytes(const umcp_plan *plan, umcp_ctx *ctx, int precision, int64_t n_energies,
                                   size_t *bytes);

/* ---- global area and volume restraints ----------------------------------
 * New global terms (the reference has no restraint energy on the total area
 * or enclosed volume; its surface::area and volume.C only measure them):
 *   A = sum over points of dudv w |Ru x Rv|   (the limit surface's area)
 *   V = 1/3 sum of dudv w R.(Ru x Rv)         (its enclosed volume, signed by orientation)
 *   E_r = 1/2 K_area (A - area0)^2 / area0 + 1/2 K_volume (V - volume0)^2
 * added to every energy, gradient and step of the mesh (kcal/mol; K_area in
 * kcal/mol/A^2, K_volume in kcal/mol/A^6). area0 or volume0 < 0 takes the
 * resident state's value at the call. A volume restraint needs a closed
 * surface. NULL or both constants 0 turns them off. Not available in batches
 * or through umcp_energy_grad_static. */
typedef struct {
  double K_area, area0, K_volume, volume0;
} umcp_restraints;
umcp_status umcp_restraints_set(umcp_mesh *mesh, const umcp_restraints *rs);
/* A, V and E_r of the latest evaluation (energy, gradient or step). */
umcp_status umcp_restraints_get(umcp_mesh *mesh, double *area, double *volume, double *energy);

/* ---- effective mass ---------------------------------------------------- */
/* Install M^-1 as a CSR matrix over vertices (SparseMatrix nzl/nzv rows,
 * src/sparse.h:4-53). */
umcp_status umcp_mass_set(umcp_mesh *mesh, int nrow, const int *row_ptr, const int *col, const double *val);
/* Build and install M^-1 from the limit surface (getSparseEffectiveMass,
 * src/modes.C:1719-1990, with the mass points of src/hd.C:417-481): per face
 * the (p+1)(p+2)/2 points (u,v) = (i/p, j/p), each carrying the mass per
 * point of src/hd.C:442-452 (mass_scale x 760.09 g/mol per 65.35 A^2 of
 * lipid, two leaflets, over surface::area's area0); M = sum_k m_k c_k c_k^T
 * with c_k the limit-point weights of the control points (umcp_plan_point_coeffs);
 * then the Cholesky inverse on the device (dense FP64, cuSOLVER potrf/potri
 * as the reference's LAPACK dpotrf/dpotri), symmetrised, and entries with
 * |M^-1_ij| <= rel_tol sqrt(|M^-1_ii M^-1_jj|) dropped (src/modes.C:1893).
 * The plan must be the one the mesh was created from. */
typedef struct {
  double mass_scale;    /* MSCALE of src/hd.C:445 (5) */
  int points_per_edge;  /* plim of src/hd.C:418 (10: 66 points per face) */
  double rel_tol;       /* truncation tolerance (1e-20, src/modes.C:16) */
} umcp_mass_opts;
typedef struct {
  double area0;         /* surface::area's area0 (src/interpLib.C:4413-4601) */
  double mass_per_point;
  long long points, nnz_mass, nnz_inverse;
  int dense;            /* 1: M^-1 kept dense (fill >= 30%), 0: CSR */
  double assembly_s;    /* wall time of the build: M assembled on the device, */
  double inverse_s;     /* its Cholesky inverse (potrf + potri), */
  double truncation_s;  /* symmetrising, truncation and the stored form */
  long long column_bytes; /* bytes of the stored columns: CSR 4 per nonzero (2 in the precision form up to
                          * 65,536 rows); 0 when dense */
} umcp_mass_info;
umcp_status umcp_mass_build(umcp_mesh *mesh, const umcp_plan *plan, const umcp_mass_opts *opts, umcp_mass_info *info);
/* The installed M^-1 as a dense nv x nv row-major array. Meshes of the
 * precision form (UMCP_FP32_CENTRED) store and apply M^-1 in FP32 (rounded
 * once from the FP64 inverse; sums compensated, scaling in FP64); their
 * values come back FP32-rounded. */
umcp_status umcp_mass_get(umcp_mesh *mesh, double *dense);
/* AltSparseCartMatVecIncrScale (src/parallel.C:1028-1075):
 * out[3i+c] += scale/alpha_c^2 * (scalev ? scalev[c*nrow+i] : 1) * sum_k val[k] in[3 col[k]+c]. */
umcp_status umcp_mass_apply(umcp_mesh *mesh, const double *in, double *out, const double *scalev, double scale,
                            const double *alphas);
umcp_status umcp_mass_apply_device(umcp_mesh *mesh, const double *d_in, double *d_out, const double *d_scalev,
                                   double scale, const double *alphas);

/* ---- dynamics ---------------------------------------------------------- */
typedef enum {
  UMCP_OVERDAMPED_BD = 0, /* r += -(D/kT) g dt + sqrt(2 D dt) xi */
  UMCP_BD_MEMBRANE = 1,   /* "do_bd_membrane" leapfrog with p reset (src/hd.C:1520-1720,1943) */
  UMCP_LANGEVIN = 2       /* "do_ld" leapfrog with friction (src/hd.C:1546-1720) */
} umcp_integrator_kind;

typedef struct {
  int kind;           /* umcp_integrator_kind */
  double time_step;   /* "time_step" (s); AKMA_TIME scaling applied inside for kinds 1,2 */
  double gamma;       /* "gamma_langevin" */
  double D;           /* kind 0: diffusion coefficient, A^2 per time_step unit */
  uint64_t seed;      /* Philox key */
  uint32_t stream;    /* Philox stream id (distinguishes meshes / replicas) */
  double divergence_threshold; /* energy jump that stops the run (hd.C uses 1e5); <= 0 disables */
  int use_mass;       /* 1: apply the installed M^-1; 0: identity */
} umcp_integrator;

/* Run n_steps steps starting at step index `step0` on the mesh's resident
 * state (set with umcp_state_set). Energies of each step may be returned in
 * energies[n_steps] (may be NULL). The loop is captured into a CUDA graph
 * after its first use with the same mesh and n_steps. */
umcp_status umcp_state_set(umcp_mesh *mesh, const double *r, const double *p);
umcp_status umcp_state_get(umcp_mesh *mesh, double *r, double *p);
umcp_status umcp_run(umcp_mesh *mesh, const umcp_integrator *it, uint64_t step0, int n_steps, double *energies);
/* Same as umcp_run without waiting: queues the steps on the ctx stream and
 * returns; umcp_ctx_synchronize or a later blocking call observes errors. */
umcp_status umcp_run_async(umcp_mesh *mesh, const umcp_integrator *it, uint64_t step0, int n_steps);

/* ---- energy minimization ---------------------------------------------------
 * Replaces Simulation::minimize (src/minimize.C:489-560) for a membrane
 * without particles, with the reference's L-BFGS (l_bfgs_iteration and
 * do_linesearch, src/l-bfgs.C:97-404): the vertex positions move, the box
 * scales alpha stay fixed (the reference zeroes their gradient,
 * src/minimize.C:321-333). The energy is the mesh's (umcp_energy, with any
 * restraints set). Starts from and replaces the resident state's positions;
 * momenta are kept. */
typedef struct {
  int max_iterations; /* the reference's nsteps: 100 */
  int history;        /* stored curvature pairs; 0: min(max_iterations, 3 nv + 6) as the reference */
  double max_move;    /* the line search's first step moves no coordinate further than this: 1.0 */
} umcp_minimize_opts;
typedef struct {
  int iterations;         /* done (fewer when the newest curvature pair vanishes, as the reference stops) */
  int evaluations;        /* energy (+gradient) evaluations */
  double energy_initial, energy_final;
  double grad_rms;        /* rms of the final gradient over the 3 nv position coordinates */
} umcp_minimize_info;
/* opts NULL: the reference's settings. energies (may be NULL, else room for
 * max_iterations + 1 values): the energy before the first iteration and
 * after each; only the first info->iterations + 1 are written. */
umcp_status umcp_minimize(umcp_mesh *mesh, const umcp_minimize_opts *opts, double *energies,
                          umcp_minimize_info *info);
/* One step of the integrator on HOST state: copies r (3*nv+3) and p (3*nv,
 * may be NULL for zero momenta) in, steps once at step index `step`, copies
 * the new r (and p) back and returns the energy of the pre-step state in *E.
 * This is the drop-in for one pass of the reference's dynamics loop body
 * (src/hd.C:1102-1720): energy, gradient, update. */
umcp_status umcp_step_host(umcp_mesh *mesh, const umcp_integrator *it, uint64_t step, double *r, double *p, double *E);
/* ---- Loop subdivision of regular patches (fast_sub6_0..3, src/fast_mm.C) --
 * d_in: n patches of 12 control points (xyz each, 36 doubles, the regular
 * patch's point order); d_out: n x 4 child patches of 36 doubles, children in
 * the reference's order. Device pointers, queued on the context's stream. */
umcp_status umcp_subdivide_patches(umcp_ctx *ctx, const double *d_in, double *d_out, long long n);
/* The stencils themselves: S[child][out point][in point], 4 x 12 x 12 (host). */
umcp_status umcp_subdivision_stencils(double *S);

/* Restart files in the reference's save format (src/restart.C:7-168): the
 * box scales, one "x y z px py pz" line per vertex and one for the box
 * scales, "seed N". Reading accepts lines without momenta and ignores the
 * particle records a reference save may hold after the surface. */
umcp_status umcp_restart_write(umcp_mesh *mesh, const char *path, int seed);
/* Sets the resident state (r and p) from the file; *seed gets its seed (-1 if none). */
umcp_status umcp_restart_read(umcp_mesh *mesh, const char *path, int *seed);
/* Energies recorded by the mesh's latest run (umcp_run, umcp_run_async or a
 * batch job): the first n of them. Synchronizes the context stream. */
umcp_status umcp_mesh_energies(umcp_mesh *mesh, double *energies, int64_t n);

/* ---- Batches: many meshes of one context advanced together.
 * No counterpart in the reference, which runs one surface per process
 * (src/hd.C:1102-1720 is the loop each job replaces). A job is a mesh with an
 * integrator, a first step index and a step count; it behaves as
 * umcp_run(mesh, it, step0, n_steps) would, on the mesh's resident state,
 * and its trajectory does not depend on the other jobs. Each step launches
 * one face kernel per patch type over all jobs, one per-job energy sum and
 * one fused gather + update. */
typedef struct umcp_batch umcp_batch;
/* The face launches' layout: the regular faces' tile size (one block's unit of
 * work), the irregular faces' tile size and the regular launch's blocks per
 * SM. With tile_faces 0 the three are chosen by timing the face launches at
 * the first run (again when the batch has grown fourfold): tile_faces over
 * multiples of the face kernel's faces per block pass, irregular tiles of 1 to
 * 8 faces per half-warp, and the occupancy limit or one block fewer. The
 * choice is keyed by (device, precision, patch types present, log2 of the
 * face count) and, with tune_cache set, read from and written to that JSON
 * file, so a later batch of the same kind takes it without timing. The
 * choice changes how the energy sums are grouped (their last bits), never the
 * per-vertex gradient sums, so trajectories do not depend on it. */
typedef struct {
  int tile_faces;     /* faces per regular tile; 0: tuned as above */
  int blocks_per_sm;  /* cap on the persistent face grids; 0: the occupancy limit (or the tuned value) */
  int irr_tile_faces; /* faces per irregular tile; 0: 4 per half-warp of the kernel's block (or the tuned value) */
  const char *tune_cache; /* JSON file of tuned choices, or NULL */
} umcp_batch_opts;
typedef struct {
  int n_jobs;
  long long n_vertices, n_faces;   /* summed over the jobs */
  int n_tiles[3];                  /* face tiles: regular, irregular valence 5, valence 7 */
  int face_grid[3];                /* blocks of each face launch */
  int n_vertex_tiles;
  int tile_faces;
  int kernels_per_step;
  double tuned_face_ms;            /* the best face-pass time of the tuning (ms), 0 when not tuned */
  int irr_tile_faces;
  int tune_source;                 /* 0 given by the options, 1 timed, 2 read from the tune cache */
} umcp_batch_info;
/* precision: umcp_precision of every job's mesh. opts may be NULL. */
umcp_status umcp_batch_create(umcp_ctx *ctx, int precision, const umcp_batch_opts *opts, umcp_batch **out);
/* Waits for the batch's work; its meshes stay valid and leave the batch. */
void umcp_batch_destroy(umcp_batch *batch);
/* Adds a job. The mesh must belong to the batch's context, have the batch's
 * precision and be in no other batch; it->use_mass must be 0. The job's run
 * starts (counters, status) at the next umcp_batch_run. Destroying the mesh
 * removes the job. */
umcp_status umcp_batch_add(umcp_batch *batch, umcp_mesh *mesh, const umcp_integrator *it, uint64_t step0,
                           int64_t n_steps);
/* Removes the job of mesh (waits for the batch's queued work first). */
umcp_status umcp_batch_remove(umcp_batch *batch, umcp_mesh *mesh);
/* Queues n_steps steps on the context stream. A job that has done its step
 * count, or stopped on a non-finite or diverging energy, takes no more steps. */
umcp_status umcp_batch_run(umcp_batch *batch, int n_steps);
/* Steps done and status (umcp_status: OK, NONFINITE or DIVERGED) of every
 * job, in the order they were added (removed jobs leave no gap). Waits for
 * the batch's queued work. Either array may be NULL. */
umcp_status umcp_batch_poll(umcp_batch *batch, int64_t *steps_done, int *job_status);
umcp_status umcp_batch_job(umcp_batch *batch, const umcp_mesh *mesh, int64_t *steps_done, int *job_status);
umcp_status umcp_batch_info_get(const umcp_batch *batch, umcp_batch_info *info);
/* The host-driven form of a batch run, for callers that keep the states on
 * the host as the reference's dynamics loop does (src/hd.C:1102-1720, one
 * surface per process there): r_in holds every job's state (3*nv+3 doubles:
 * positions, then the box scales) packed in job order (the order of
 * umcp_batch_add; umcp_batch_poll reports the same order). They are copied
 * in (one copy; pinned host memory makes it a direct DMA), n_steps steps are
 * run as umcp_batch_run runs them, and the new states and each job's latest
 * energy are copied out to r_out (packed the same way; may equal r_in) and
 * E (one double per job). Either output may be NULL, and r_in may be NULL
 * to step the resident states. Momenta stay on the device. Waits for the
 * copies; per-job status as umcp_batch_poll reports it. */
umcp_status umcp_batch_step_host(umcp_batch *batch, const double *r_in, double *r_out, double *E, int n_steps);
/* Queues only the face launches of one step over the batch's current jobs
 * (tables as of the latest run): the unit a roofline measurement times. The
 * jobs' states and counters do not change; jobs that have done their step
 * count or stopped are skipped, as in a step. */
umcp_status umcp_batch_face_pass(umcp_batch *batch);

/* ---- Serving: a request loop over one batch.
 * No counterpart in the reference. Jobs (a .mesh file, parameters, an
 * integrator, a step count) are submitted from any host thread. Host worker
 * threads build their plans; the server thread admits ready jobs in arrival
 * order while their device footprint (umcp_plan_device_bytes) fits the HBM
 * budget, adds them to its batch (their state stays resident until they
 * finish), runs the batch in chunks of steps, and at each chunk boundary
 * copies out the results of finished jobs and frees their memory. Jobs
 * admitted while a chunk runs are built and uploaded during it and join at
 * the next chunk. Each job's trajectory is the one umcp_run gives its mesh
 * alone. Times are seconds on the server's steady clock. */
typedef struct umcp_server umcp_server;
typedef struct {
  int precision;               /* of every job (a job's params.precision is overridden) */
  double hbm_budget_bytes;     /* footprint limit of resident jobs; 0: 80% of the free memory at creation */
  int max_jobs;                /* resident job cap; 0: none */
  double chunk_ms;             /* target wall time of one chunk; 0: 25 ms */
  int builder_threads;         /* plan-building threads; 0: hardware threads, at most 16 */
  int tile_faces;              /* as umcp_batch_opts.tile_faces */
} umcp_server_opts;
typedef struct {
  const char *mesh_path;       /* read by a worker thread; must exist until the job is built */
  umcp_params params;          /* lipid_directives text is copied at submit */
  umcp_integrator it;          /* use_mass must be 0 */
  uint64_t step0;
  int64_t n_steps;
  int keep_energies;           /* keep the per-step energies for umcp_server_fetch */
} umcp_job_desc;
typedef enum { UMCP_JOB_QUEUED = 0, UMCP_JOB_BUILDING = 1, UMCP_JOB_READY = 2, UMCP_JOB_RUNNING = 3,
               UMCP_JOB_DONE = 4 } umcp_job_state;
typedef struct {
  int state;                   /* umcp_job_state */
  int status;                  /* umcp_status of a done job */
  int nv;
  int64_t steps_done;
  double t_submit, t_admit, t_done;  /* -1 until reached */
  double device_bytes;
  double h2d_bytes, d2h_bytes; /* copied in at admission; copied out at the end */
  char message[160];           /* error text of a failed job */
} umcp_job_info;
typedef struct {
  long long submitted, completed, failed, queued, running, chunks;
  double p50_latency_s, p99_latency_s, mean_latency_s, max_latency_s;  /* submit to done, completed jobs */
  double vertex_steps;         /* performed by all jobs so far */
  double busy_s;               /* wall time spent in chunks (launch to results) */
  double vertex_steps_per_s;   /* vertex_steps / busy_s */
  double hbm_budget_bytes, hbm_in_use_bytes, hbm_peak_bytes;
  int chunk_steps;             /* size of the latest chunk */
} umcp_server_stats;
umcp_status umcp_server_create(umcp_ctx *ctx, const umcp_server_opts *opts, umcp_server **out);
/* Stops the loop after the chunk in flight; unfinished jobs are dropped. */
void umcp_server_destroy(umcp_server *server);
umcp_status umcp_server_submit(umcp_server *server, const umcp_job_desc *job, uint64_t *job_id);
/* Waits until the job is done (UMCP_OK) or timeout_s passes (UMCP_ERR_TIMEOUT);
 * timeout_s < 0 waits without limit. The job's own status is in its info. */
umcp_status umcp_server_wait(umcp_server *server, uint64_t job_id, double timeout_s);
umcp_status umcp_server_wait_all(umcp_server *server, double timeout_s);
umcp_status umcp_server_job(umcp_server *server, uint64_t job_id, umcp_job_info *info);
/* Copies a done job's final state r (3*nv+3) and, if kept, its energies
 * (steps_done of them); either may be NULL. */
umcp_status umcp_server_fetch(umcp_server *server, uint64_t job_id, double *r, double *energies);
/* Forgets a done job and its results. */
umcp_status umcp_server_release(umcp_server *server, uint64_t job_id);
umcp_status umcp_server_stats_get(umcp_server *server, umcp_server_stats *stats);
/* Seconds on the server's clock (the clock of the job times). */
double umcp_server_now(const umcp_server *server);

#ifdef __cplusplus
}
#endif
#endif /* UMCP_GPU_H */
