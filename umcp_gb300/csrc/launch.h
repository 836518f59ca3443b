// Launch wrappers of the device kernels (surface_kernels.cu). Plain pointers;
// all work is queued on the given stream.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.cuh"

namespace umcp {

// Status bits written by kernels into the mesh's device status word.
enum : int { kStatusNonFinite = 1, kStatusDiverged = 2 };

// Face pass for one patch type (ncp 12/npt 15 regular; ncp 11 or 13, npt 16
// irregular). T selects the arithmetic: double (plain path) or float
// (face-centred precision form). partial[dest[f*ncp+x]] receives the
// alpha-scaled gradient of control point x of face f; terms[(face_base+f)*6]
// receives {E_area, E_curvature, E_angle, dE/dalpha_x,y,z}.
template <typename T>
cudaError_t launch_faces(const dev::FaceLaunch &L, const int *dest, int ncp, int npt, const dev::SurfaceParams &P,
                         const double *r, T *partial, double *terms, int *status, int grid, cudaStream_t s);

// Per vertex: g[3v+c] += sum of its partial slots [off[v], off[v+1]).
template <typename T>
cudaError_t launch_gather(int nv, const T *partial, const int *off, double *g, cudaStream_t s);

// Per mesh segment [seg[m], seg[m+1]) of faces: E[m] = sum of the three energy
// terms, parts[3m..] = the terms, and g_alpha[m*? ] += dE/dalpha added into
// galpha (3 doubles per mesh). Fixed-order tree sum.
cudaError_t launch_reduce_terms(int nmesh, const int *seg, const double *terms, double *E, double *parts,
                                double *galpha, cudaStream_t s);

// Integrator kernels. r, p, g: 3*nv (+3) doubles. noise drawn from
// Philox4x32-10 keyed by (seed), counter (vertex, step, stream).
struct StepArgs {
  int kind;            // 0 overdamped BD, 1 BD membrane, 2 Langevin
  double mob_dt;       // kind 0: D dt / kT
  double sigma;        // kind 0: sqrt(2 D dt); kinds 1,2: sqrt(2 gamma kT AK)
  double AK;           // AKMA_TIME * time_step
  double gamma;
  uint64_t seed;
  uint32_t stream;
};
// Kind 0, and kinds 1/2 with identity mass: one fused vertex update.
cudaError_t launch_step_local(int nv, const StepArgs &a, const uint64_t *step, double *r, double *p, const double *g,
                              const int *status, cudaStream_t s);
// Kinds 1/2 with a mass matrix: kick p (friction, kicks, noise); then
// qdot = M^-1 p by launch_spmv; then r += qdot AK (and p reset for BD).
cudaError_t launch_kick(int nv, const StepArgs &a, const uint64_t *step, double *p, const double *g, const int *status,
                        cudaStream_t s);
cudaError_t launch_drift(int nv, const StepArgs &a, double *r, double *p, const double *qdot, const int *status,
                         cudaStream_t s);

// out[3i+c] (+)= scale/alpha_c^2 * (scalev ? scalev[c*nrow+i] : 1) * sum_k val[k] in[3 col[k]+c].
// accumulate=0 overwrites out. alphas: device pointer to 3 doubles (or NULL = 1).
cudaError_t launch_spmv(int nrow, const int *row_ptr, const int *col, const double *val, const double *scalev,
                        double scale, const double *alphas, const double *in, double *out, int accumulate,
                        cudaStream_t s);

// Energy bookkeeping for runs: energies[runidx] = E; flags non-finite
// energies and a rise above threshold since the previous step (src/hd.C:1280).
cudaError_t launch_record_energy(const double *E, double *energies, const uint64_t *runidx, double threshold,
                                 int *status, cudaStream_t s);
cudaError_t launch_advance_step(uint64_t *step, uint64_t *runidx, cudaStream_t s);

}  // namespace umcp
