// Launch wrappers of the device kernels (surface_kernels.cu). Plain pointers;
// all work is queued on the given stream.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.cuh"

namespace umcp {

// Status bits written by kernels into the mesh's device status word.
enum : int { kStatusNonFinite = 1, kStatusDiverged = 2, kStatusTimeout = 4 };

// Where and how the block partials of a face pass are summed (see
// launch_finish). done: device counter of finished blocks, zero between
// launches; when non-null, the last block of that face launch does the sum.
struct FinishArgs {
  int nblk;            // block-partial rows to sum: every block of every face launch of the pass, each of
                       // which counts on `done`; the block that brings it to nblk sums the rows
  double *E, *parts, *galpha;
  double *energies;    // run only: energies[cnt[1]] = E, cnt[1] += 1
  uint64_t *cnt;
  double threshold;    // energy rise that flags divergence (<= 0: off)
  int *status;
  unsigned *done;
  const double *gterm; // global restraint terms to add (NULL: none), see GeoArgs
};

// Global area and volume of the limit surface and their restraint (one
// half-warp per face over every patch type; V in FP64, see geo_sums_kernel):
//   A = sum dudv w |Ru x Rv|,  V = 1/3 sum dudv w R.(Ru x Rv)
//   E_r = 1/2 K_A (A-A0)^2/A0 + 1/2 K_V (V-V0)^2
// gterm receives {A, V, E_r, dE_r/dA, dE_r/dV, dE_r/dalpha_xyz}.
struct GeoGroup {
  const uint32_t *cp;      // [nfaces][ncp] packed control points
  const int *dest;         // [nfaces][ncp] gradient-partial slots
  const double *basis;     // [npt][5][ncpp] rows u,v,uu,uv,vv
  const double *basis_w;   // [npt][ncp] value rows
  const double *weight;    // [npt]
  // FP32 tables of the precision form: rows w,u,v as hi [npt][3][ncp] then
  // lo [npt][3][ncp] (row = hi + lo), then cw = dudv w [npt], then
  // c3 = dudv w / 3 as hi [npt] and lo [npt]
  const float *tab;
  int ncp, npt, ncpp, nfaces, face_base;
  double dudv;
};
// Floats of GeoGroup::tab for a patch type.
inline size_t geo_tab_floats(int ncp, int npt) { return (size_t)6 * npt * ncp + 3 * (size_t)npt; }
enum : int { kGeoA = 0, kGeoV, kGeoE, kGeoCA, kGeoCV, kGeoDAlpha, kGeoWords = 8 };
struct GeoArgs {
  GeoGroup g[3];
  int ngroups, nfaces, nv;
  const double *r;
  const float *rhi, *rlo;  // r = hi + lo (precision form; read by the FP32 gradient pass)
  double box[3][3];
  float box_hi[3][3], box_lo[3][3];
  double KA, A0, KV, V0;
  double *block;           // [blocks][8] partial sums
  double *gterm;           // kGeoWords
  unsigned *done;          // finished-block counter (zero between launches)
};
constexpr int kGeoThreads = 128;
// Fixed grid (a function of the face count only, so every sum has a fixed order).
inline int geo_blocks(int nfaces) {
  const int b = nfaces > 0 ? (nfaces + 4 * (kGeoThreads / 16) - 1) / (4 * (kGeoThreads / 16)) : 1;  // >= 4 faces per half-warp
  return b < 152 * 8 ? b : 152 * 8;
}
// Sums A, V and their alpha derivatives; the last block writes gterm.
// alpha64: the area and the box-scale derivatives in FP64 as well (plain path).
cudaError_t launch_geo_sums(const GeoArgs &G, bool alpha64, cudaStream_t s);
// partial[slot] += alpha * (dE_r/dA dA/dX + dE_r/dV dV/dX) for every (face, control point).
template <typename T>
cudaError_t launch_geo_grad(const GeoArgs &G, T *partial, cudaStream_t s);

// The precision form's FP32 copies of the positions (all NULL in the plain
// path): r = hi + lo to about 2^-48 relative, and dsp = r - r0, the
// displacement from the reference state r0 (setg0's state), rounded once.
// The face kernels form the area strain from dsp (see point_adjoint).
struct F32Pos {
  float *hi = nullptr, *lo = nullptr;
  const double *r0 = nullptr;
  float *dsp = nullptr;
};

// Persistent grid of the face pass for one patch type (fixed per device and
// face count, so the order of every sum is fixed).
template <typename T>
int face_blocks(int nfaces, int ncp, int npt);

// Face pass for one patch type (ncp 12/npt 15 regular; ncp 11 or 13, npt 16
// irregular). T selects the arithmetic: double (plain path) or float
// (face-centred precision form). partial[dest[f*ncp+x]] receives the
// alpha-scaled gradient of control point x of face f; blockpart[L.block_base
// + b] receives block b's sums {E_area, E_curvature, E_angle, dE/dalpha_xyz}.
// f: the FP32 positions and displacements (read by the float instantiation only).
template <typename T>
cudaError_t launch_faces(const dev::FaceLaunch &L, const int *dest, int ncp, int npt, const dev::SurfaceParams &P,
                         const double *r, const F32Pos &f, T *partial, double *blockpart, int *status, int grid,
                         const FinishArgs &fin, cudaStream_t s);

// The regular faces of the precision form on the tensor cores (face_tc_kernel):
// the same outputs as launch_faces<float> for ncp 12 / npt 15, in 128-face
// tiles; grid from face_blocks_tc.
int face_blocks_tc(int nfaces);
cudaError_t launch_faces_tc(const dev::FaceLaunch &L, const int *dest, const dev::SurfaceParams &P, const double *r,
                            const float *rhi, const float *rlo, const float *dsp, float *partial, double *blockpart,
                            int *status, int grid, const FinishArgs &fin, cudaStream_t s);

// The precision form's FP32 positions of r: f.hi[i] + f.lo[i] = r[i] to about
// 2^-48 relative, f.dsp[i] = r[i] - f.r0[i].
cudaError_t launch_split_positions(int n, const double *r, const F32Pos &f, cudaStream_t s);

// *dst |= *src on the device (one thread).
cudaError_t launch_status_merge(const int *src, int *dst, cudaStream_t s);

// Fixed-order sum of F.nblk block partials: E, parts (3), galpha (+= 3). With
// energies/cnt given (a run): energies[cnt[1]] = E, divergence and non-finite
// flags (src/hd.C:1280-1305), cnt[1] += 1.
cudaError_t launch_finish(const FinishArgs &F, const double *blockpart, cudaStream_t s);

// Per vertex: g[3v+c] += sum of its partial slots off[2v] + 32 k, k < off[2v+1]
// (32 vertices interleaved per group, see interleave_slots).
template <typename T>
cudaError_t launch_gather(int nv, const T *partial, const int *off, double *g, cudaStream_t s);

// Integrator kernels. r, p: 3*nv doubles. Noise from Philox4x32-10 keyed by
// seed, counter (vertex, step, stream) with step = cnt[0] + cnt[1] - 1.
struct StepArgs {
  int kind;            // 0 overdamped BD, 1 BD membrane, 2 Langevin
  double mob_dt;       // kind 0: D dt / kT
  double sigma;        // kind 0: sqrt(2 D dt); kinds 1,2: sqrt(2 gamma kT AK)
  double AK;           // AKMA_TIME * time_step
  double gamma;
  uint64_t seed;
  uint32_t stream;
  float mob_dt_f, sigma_f;  // kind 0: mob_dt and sigma rounded to FP32 (the precision form's increment)
};
// Gather fused with the vertex-local update (kind 0; kinds 1/2 with identity mass).
// f (all NULL in the plain path) receives the FP32 positions of the new state.
template <typename T>
cudaError_t launch_gather_step(int nv, const T *partial, const int *off, const StepArgs &a, const uint64_t *cnt,
                               double *r, double *p, const F32Pos &f, const int *status, cudaStream_t s);
// Kinds 1/2 with a mass matrix: kick p (friction, kicks, noise); then
// qdot = M^-1 p by launch_spmv; then r += qdot AK (and p reset for BD).
cudaError_t launch_kick(int nv, const StepArgs &a, const uint64_t *cnt, double *p, const double *g, const int *status,
                        cudaStream_t s);
cudaError_t launch_drift(int nv, const StepArgs &a, double *r, double *p, const double *qdot, const F32Pos &f,
                         const int *status, cudaStream_t s);

// One mesh of a batch (device pointers into the mesh's own buffers). The
// face kernel stages the leading part, BatchFaceJob, in shared memory.
struct BatchFaceJob {
  dev::FaceSrc src[3];     // patch types: regular, irregular valence 5, irregular valence 7
  dev::SurfaceParams P;
  void *partial;           // the mesh's gradient-partial slots
  uint64_t *cnt;           // {first step of the run, steps done}
  uint64_t limit;          // steps in the run
  int *status;
  int pad;
};
struct BatchJob {
  BatchFaceJob f;
  const int *off;          // vertex slot locations {first slot, count} (interleaved numbering)
  double *r, *p;           // state
  float *rhi, *rlo;        // FP32 hi/lo pairs of r (precision form), else NULL
  const double *r0;        // reference state (precision form)
  float *dsp;              // r - r0 in FP32 (precision form)
  double *E, *parts;       // energy (and parts) of the latest step
  double *energies;        // the run's recorded energies, indexed by steps done
  double threshold;        // energy rise that flags divergence (<= 0: off)
  StepArgs a;              // the job's integrator
};
// Faces [first, first+count) of one patch type of one job, or vertices
// [first, first+count) of one job.
struct BatchTile {
  int job, first, count;
};
// Layout of the batch's device count array.
enum : int { kCountTiles = 0, kCountTileBase = 3, kCountJobs = 6, kCountVertexTiles = 7, kCountWords = 8 };
constexpr int kVertexTile = 256;  // vertices per vertex tile (one thread each)

// Face launch of patch type `group` over its tiles (counts[group] of them,
// from counts[3 + group] in tiles); tile_sums[3 * global tile] receives each
// tile's energy terms. Persistent grid; tiles of stopped or finished jobs are
// skipped.
template <typename T>
// next_tile: a device int the regular FP32 launch hands tiles out from (zeroed
// by the launch wrapper, on s, before the kernel).
cudaError_t launch_batch_faces(const BatchJob *jobs, int group, const BatchTile *tiles, const int *counts,
                               const double *basis, const double *weight, int ncp, int npt, double dudv,
                               int irregular, double *tile_sums, int grid, int *next_tile, cudaStream_t s);
// Per job: tile sums in listed order (tile_idx[tile_off[j] .. tile_off[j+1])),
// energy record, flags, steps done; live[j] and prog[j] = {done, status}.
cudaError_t launch_batch_reduce(const BatchJob *jobs, const int *counts, int max_jobs, const int *tile_off,
                                const int *tile_idx, const double *tile_sums, int *live, unsigned long long *prog,
                                cudaStream_t s);
// Gather fused with the update, for live jobs (kinds 0, and 1/2 with identity mass).
template <typename T>
cudaError_t launch_batch_gather_step(const BatchJob *jobs, const BatchTile *vtiles, const int *counts,
                                     const int *live, int grid, cudaStream_t s);
// Run start of the jobs with start[j] != 0: counters {step0[j], 0}, status 0, hi/lo split.
cudaError_t launch_batch_start(const BatchJob *jobs, const BatchTile *vtiles, const int *counts, const int *start,
                               const unsigned long long *step0, int grid, cudaStream_t s);
// Host-driven steps: jobs' states packed in job order at pack + off[j] (3 nv + 3
// doubles each). unpack: into the jobs' resident states (and FP32 copies);
// pack: back out, with each job's latest energy in E[j].
cudaError_t launch_batch_unpack(const BatchJob *jobs, const BatchTile *vtiles, const int *counts,
                                const long long *off, const double *pack, int grid, cudaStream_t s);
cudaError_t launch_batch_pack(const BatchJob *jobs, const BatchTile *vtiles, const int *counts, const long long *off,
                              double *pack, double *E, int grid, cudaStream_t s);
// Device-filling grid of a batch face launch for a patch type.
template <typename T>
int batch_face_blocks(int ncp, int npt);

// out[3i+c] (+)= scale/alpha_c^2 * (scalev ? scalev[c*nrow+i] : 1) * sum_k val[k] in[3 col[k]+c].
// accumulate=0 overwrites out. alphas: device pointer to 3 doubles (or NULL = 1).
// launch_spmv on FP32 values and an FP32 input packed as float4 {x, y, z, 0}
// per row (spmv32_kernel).
cudaError_t launch_spmv32(int nrow, const int *row_ptr, const void *col, bool col16, const float *val, const double *scalev,
                          double scale, const double *alphas, const float4 *in, double *out, int accumulate,
                          cudaStream_t s);
// out[i] = {(float)in[3i], (float)in[3i+1], (float)in[3i+2], 0}, i < n.
cudaError_t launch_to_f32x4(int n, const double *in, float4 *out, cudaStream_t s);
cudaError_t launch_spmv(int nrow, const int *row_ptr, const int *col, const double *val, const double *scalev,
                        double scale, const double *alphas, const double *in, double *out, int accumulate,
                        cudaStream_t s);

}  // namespace umcp
