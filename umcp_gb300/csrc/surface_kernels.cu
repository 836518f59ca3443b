// Kernels of the membrane-surface hot path. See kernels.cuh for the model
// and launch.h for the contracts.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "kernels.cuh"
#include "launch.h"
#include "philox.h"

namespace umcp {
namespace dev {

constexpr int kThreads = 128;
constexpr int kHalfWarps = kThreads / 16;
constexpr int kAdjKinds = 7;  // Ru, Rv, Suu, Suv, Svv adjoints + angle-term part of Ru, Rv

// One half-warp (16 lanes) per face. Shared memory per block: the patch's
// basis rows [kind][cp][pt] (pt fastest, so lanes that differ in pt or in cp
// hit distinct banks), and per half-warp the face's control points and the
// adjoints [kind][xyz][pt].
template <typename T, int NCP, int NPT>
__global__ void __launch_bounds__(kThreads) face_kernel(FaceLaunch L, const int *__restrict__ dest, SurfaceParams P,
                                                        const double *__restrict__ r, T *__restrict__ partial,
                                                        double *__restrict__ terms, int *__restrict__ status) {
  __shared__ T sB[5 * NCP * NPT];
  __shared__ T sX[kHalfWarps][NCP][3];
  __shared__ T sK[kHalfWarps][kAdjKinds][3][16];
  __shared__ T sW[NPT];

  for (int i = threadIdx.x; i < 5 * NCP * NPT; i += kThreads) sB[i] = (T)L.basis[i];
  for (int i = threadIdx.x; i < NPT; i += kThreads) sW[i] = (T)L.weight[i];
  __syncthreads();

  const int hw = threadIdx.x >> 4, lane = threadIdx.x & 15;
  const unsigned hmask = (threadIdx.x & 16) ? 0xFFFF0000u : 0x0000FFFFu;
  const double alpha[3] = {r[3 * P.nv], r[3 * P.nv + 1], r[3 * P.nv + 2]};
  const T kc = (T)P.kc, KA = (T)P.KA, kg = (T)P.kg, k_reg = (T)P.k_reg, dudv = (T)L.dudv;

  for (int f = blockIdx.x * kHalfWarps + hw; f < L.nfaces; f += gridDim.x * kHalfWarps) {
    // ---- control points: alpha*(r + lattice image), centred on the patch centroid
    double X[3] = {0, 0, 0}, Xs[3] = {0, 0, 0};
    if (lane < NCP) {
      uint32_t packed = L.cp[(size_t)f * NCP + lane];
      int v = (int)(packed & kVertexMask);
      int code = (int)(packed >> kVertexBits);
      int ix = code % 3 - 1, iy = (code / 3) % 3 - 1, iz = code / 9 - 1;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        X[c] = r[3 * v + c] + ix * P.box[0][c] + iy * P.box[1][c] + iz * P.box[2][c];
        Xs[c] = alpha[c] * X[c];
      }
    }
    double cen[3] = {Xs[0], Xs[1], Xs[2]}, ucen[3] = {X[0], X[1], X[2]};
#pragma unroll
    for (int off = 8; off >= 1; off >>= 1)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        cen[c] += __shfl_xor_sync(hmask, cen[c], off, 16);
        ucen[c] += __shfl_xor_sync(hmask, ucen[c], off, 16);
      }
#pragma unroll
    for (int c = 0; c < 3; ++c) { cen[c] *= (1.0 / NCP); ucen[c] *= (1.0 / NCP); }
    if (lane < NCP)
#pragma unroll
      for (int c = 0; c < 3; ++c) sX[hw][lane][c] = (T)(Xs[c] - cen[c]);
    __syncwarp(hmask);

    // ---- lanes as quadrature points: contractions, energy, adjoint
    T ea = 0, ec = 0, er = 0;
    if (lane < NPT) {
      Vec3<T> K[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) K[k] = {0, 0, 0};
#pragma unroll
      for (int x = 0; x < NCP; ++x) {
        const T px = sX[hw][x][0], py = sX[hw][x][1], pz = sX[hw][x][2];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          const T b = sB[(k * NCP + x) * NPT + lane];
          K[k].x += b * px;
          K[k].y += b * py;
          K[k].z += b * pz;
        }
      }
      const size_t pi = (size_t)f * NPT + lane;
      const T g0 = (T)L.g0[pi], rr0 = (T)L.rr0[pi];
      const T P2 = (T)L.comp[3 * (size_t)f], Hbar = (T)L.comp[3 * (size_t)f + 1], Pres = (T)L.comp[3 * (size_t)f + 2];
      Vec3<T> Kb[5], Kreg[2];
      point_adjoint<T>(K, sW[lane], g0, rr0, dudv, P2, Hbar, Pres, kc, KA, kg, k_reg, &ea, &ec, &er, Kb, Kreg);
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        sK[hw][k][0][lane] = Kb[k].x;
        sK[hw][k][1][lane] = Kb[k].y;
        sK[hw][k][2][lane] = Kb[k].z;
      }
      if (L.irregular)
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          sK[hw][5 + k][0][lane] = Kreg[k].x;
          sK[hw][5 + k][1][lane] = Kreg[k].y;
          sK[hw][5 + k][2][lane] = Kreg[k].z;
        }
    }
    __syncwarp(hmask);

    // ---- lanes as control points: contract the adjoint back onto the one-ring
    double da[3] = {0, 0, 0};
    if (lane < NCP) {
      T G[3] = {0, 0, 0};
#pragma unroll 5
      for (int p = 0; p < NPT; ++p)
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          const T b = sB[(k * NCP + lane) * NPT + p];
          G[0] += b * sK[hw][k][0][p];
          G[1] += b * sK[hw][k][1][p];
          G[2] += b * sK[hw][k][2][p];
        }
      const int d = dest[(size_t)f * NCP + lane];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        partial[3 * (size_t)d + c] = (T)(alpha[c] * (double)G[c]);
        da[c] = (double)G[c] * (X[c] - ucen[c]);
      }
      if (L.irregular && P.k_reg != 0.0) {
        // igrad adds the angle-term adjoint to dE/dalpha with one more alpha
        // factor (src/grad.C:7414-7421): add (alpha-1) times that part.
        T Gr[3] = {0, 0, 0};
        for (int p = 0; p < NPT; ++p)
#pragma unroll
          for (int k = 0; k < 2; ++k) {
            const T b = sB[(k * NCP + lane) * NPT + p];
            Gr[0] += b * sK[hw][5 + k][0][p];
            Gr[1] += b * sK[hw][5 + k][1][p];
            Gr[2] += b * sK[hw][5 + k][2][p];
          }
#pragma unroll
        for (int c = 0; c < 3; ++c) da[c] += (alpha[c] - 1.0) * (double)Gr[c] * (X[c] - ucen[c]);
      }
    }
    // ---- per-face sums (fixed butterfly order)
    double e3[3] = {(double)ea, (double)ec, (double)er};
#pragma unroll
    for (int off = 8; off >= 1; off >>= 1) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        e3[c] += __shfl_xor_sync(hmask, e3[c], off, 16);
        da[c] += __shfl_xor_sync(hmask, da[c], off, 16);
      }
    }
    if (lane == 0) {
      double *t = terms + 6 * (size_t)(L.face_base + f);
      t[0] = e3[0]; t[1] = e3[1]; t[2] = e3[2];
      t[3] = da[0]; t[4] = da[1]; t[5] = da[2];
      if (!isfinite(e3[0] + e3[1] + e3[2])) atomicOr(status, kStatusNonFinite);
    }
    __syncwarp(hmask);
  }
}

template <typename T>
__global__ void gather_kernel(int nv, const T *__restrict__ partial, const int *__restrict__ off,
                              double *__restrict__ g) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
    double a0 = 0, a1 = 0, a2 = 0;
    for (int s = off[v]; s < off[v + 1]; ++s) {
      a0 += (double)partial[3 * (size_t)s];
      a1 += (double)partial[3 * (size_t)s + 1];
      a2 += (double)partial[3 * (size_t)s + 2];
    }
    g[3 * (size_t)v] += a0;
    g[3 * (size_t)v + 1] += a1;
    g[3 * (size_t)v + 2] += a2;
  }
}

// One block per mesh; each thread sums a strided subset, then a fixed tree.
__global__ void reduce_terms_kernel(const int *__restrict__ seg, const double *__restrict__ terms, double *E,
                                    double *parts, double *galpha) {
  __shared__ double red[6][256];
  const int m = blockIdx.x;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int f = seg[m] + threadIdx.x; f < seg[m + 1]; f += blockDim.x)
#pragma unroll
    for (int q = 0; q < 6; ++q) acc[q] += terms[6 * (size_t)f + q];
#pragma unroll
  for (int q = 0; q < 6; ++q) red[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int width = blockDim.x / 2; width > 0; width >>= 1) {
    if ((int)threadIdx.x < width)
#pragma unroll
      for (int q = 0; q < 6; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + width];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (E) E[m] = red[0][0] + red[1][0] + red[2][0];
    if (parts) { parts[3 * m] = red[0][0]; parts[3 * m + 1] = red[1][0]; parts[3 * m + 2] = red[2][0]; }
    if (galpha) { galpha[3 * m] += red[3][0]; galpha[3 * m + 1] += red[4][0]; galpha[3 * m + 2] += red[5][0]; }
  }
}

__device__ __forceinline__ void normals3(uint64_t seed, uint32_t stream, uint64_t step, int v, double n[3]) {
  philox_out o = philox4x32_10((uint32_t)v, (uint32_t)step, (uint32_t)(step >> 32), stream, (uint32_t)seed,
                               (uint32_t)(seed >> 32));
  double u1 = philox_u53(o.v[0], o.v[1]), u2 = philox_u53(o.v[2], o.v[3]);
  double rad = sqrt(-2.0 * log(u1)), sn, cs;
  sincospi(2.0 * u2, &sn, &cs);
  n[0] = rad * cs;
  n[1] = rad * sn;
  o = philox4x32_10((uint32_t)v, (uint32_t)step, (uint32_t)(step >> 32), stream | 0x80000000u, (uint32_t)seed,
                    (uint32_t)(seed >> 32));
  u1 = philox_u53(o.v[0], o.v[1]);
  u2 = philox_u53(o.v[2], o.v[3]);
  rad = sqrt(-2.0 * log(u1));
  n[2] = rad * cospi(2.0 * u2);
}

// Momentum update of the reference leapfrog (src/hd.C:1546-1693), one vertex.
__device__ __forceinline__ void kick(const StepArgs &a, const double n[3], double pp[3], const double gg[3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double q = pp[c];
    if (a.kind == 2) q -= a.gamma * a.AK * q;
    q += -gg[c] * a.AK * 0.5;
    if (a.kind == 1) q += (1.0 / a.gamma) * a.sigma * n[c] / a.AK;
    else q += a.sigma * n[c];
    q += -gg[c] * a.AK * 0.5;
    pp[c] = q;
  }
}

__global__ void step_local_kernel(int nv, StepArgs a, const uint64_t *__restrict__ step, double *__restrict__ r,
                                  double *__restrict__ p, const double *__restrict__ g, const int *__restrict__ status) {
  if (*status) return;
  const uint64_t st = *step;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
    double n[3], gg[3] = {g[3 * (size_t)v], g[3 * (size_t)v + 1], g[3 * (size_t)v + 2]};
    normals3(a.seed, a.stream, st, v, n);
    if (a.kind == 0) {
#pragma unroll
      for (int c = 0; c < 3; ++c) r[3 * (size_t)v + c] += -a.mob_dt * gg[c] + a.sigma * n[c];
    } else {
      double pp[3] = {p[3 * (size_t)v], p[3 * (size_t)v + 1], p[3 * (size_t)v + 2]};
      kick(a, n, pp, gg);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        r[3 * (size_t)v + c] += pp[c] * a.AK;  // identity M^-1
        p[3 * (size_t)v + c] = (a.kind == 1) ? 0.0 : pp[c];
      }
    }
  }
}

__global__ void kick_kernel(int nv, StepArgs a, const uint64_t *__restrict__ step, double *__restrict__ p,
                            const double *__restrict__ g, const int *__restrict__ status) {
  if (*status) return;
  const uint64_t st = *step;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
    double n[3], gg[3] = {g[3 * (size_t)v], g[3 * (size_t)v + 1], g[3 * (size_t)v + 2]};
    normals3(a.seed, a.stream, st, v, n);
    double pp[3] = {p[3 * (size_t)v], p[3 * (size_t)v + 1], p[3 * (size_t)v + 2]};
    kick(a, n, pp, gg);
#pragma unroll
    for (int c = 0; c < 3; ++c) p[3 * (size_t)v + c] = pp[c];
  }
}

__global__ void drift_kernel(int nv, StepArgs a, double *__restrict__ r, double *__restrict__ p,
                             const double *__restrict__ qdot, const int *__restrict__ status) {
  if (*status) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * nv; i += gridDim.x * blockDim.x) {
    r[i] += qdot[i] * a.AK;
    if (a.kind == 1) p[i] = 0.0;
  }
}

// One warp per row; lanes stride the row's nonzeros (coalesced reads of the
// value/column streams), warp-shuffle sum in fixed order.
__global__ void spmv_kernel(int nrow, const int *__restrict__ row_ptr, const int *__restrict__ col,
                            const double *__restrict__ val, const double *__restrict__ scalev, double scale,
                            const double *__restrict__ alphas, const double *__restrict__ in, double *__restrict__ out,
                            int accumulate) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  double f[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double a = alphas ? alphas[c] : 1.0;
    f[c] = scale / (a * a);
  }
  for (int i = warp; i < nrow; i += nwarps) {
    double s0 = 0, s1 = 0, s2 = 0;
    for (int k = row_ptr[i] + lane; k < row_ptr[i + 1]; k += 32) {
      const double v = val[k];
      const int j = col[k];
      s0 += v * in[3 * (size_t)j];
      s1 += v * in[3 * (size_t)j + 1];
      s2 += v * in[3 * (size_t)j + 2];
    }
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
      s0 += __shfl_xor_sync(0xffffffffu, s0, off);
      s1 += __shfl_xor_sync(0xffffffffu, s1, off);
      s2 += __shfl_xor_sync(0xffffffffu, s2, off);
    }
    if (lane == 0) {
      double o[3] = {s0 * f[0], s1 * f[1], s2 * f[2]};
      if (scalev)
#pragma unroll
        for (int c = 0; c < 3; ++c) o[c] *= scalev[(size_t)c * nrow + i];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (accumulate) out[3 * (size_t)i + c] += o[c];
        else out[3 * (size_t)i + c] = o[c];
      }
    }
  }
}

__global__ void record_energy_kernel(const double *E, double *energies, const uint64_t *runidx, double threshold,
                                     int *status) {
  const uint64_t idx = *runidx;
  const double e = E[0];
  if (energies) energies[idx] = e;
  if (!isfinite(e)) atomicOr(status, kStatusNonFinite);
  if (threshold > 0 && idx > 0 && energies && e - energies[idx - 1] > threshold) atomicOr(status, kStatusDiverged);
}

__global__ void advance_step_kernel(uint64_t *step, uint64_t *runidx) {
  *step += 1;
  *runidx += 1;
}

}  // namespace dev

static int grid_for(int n, int per_block) {
  int g = (n + per_block - 1) / per_block;
  return g < 1 ? 1 : g;
}

template <typename T>
cudaError_t launch_faces(const dev::FaceLaunch &L, const int *dest, int ncp, int npt, const dev::SurfaceParams &P,
                         const double *r, T *partial, double *terms, int *status, int grid, cudaStream_t s) {
  if (L.nfaces <= 0) return cudaSuccess;
  if (grid <= 0) grid = grid_for(L.nfaces, dev::kHalfWarps);
  if (ncp == 12 && npt == 15)
    dev::face_kernel<T, 12, 15><<<grid, dev::kThreads, 0, s>>>(L, dest, P, r, partial, terms, status);
  else if (ncp == 11 && npt == 16)
    dev::face_kernel<T, 11, 16><<<grid, dev::kThreads, 0, s>>>(L, dest, P, r, partial, terms, status);
  else if (ncp == 13 && npt == 16)
    dev::face_kernel<T, 13, 16><<<grid, dev::kThreads, 0, s>>>(L, dest, P, r, partial, terms, status);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}
template cudaError_t launch_faces<double>(const dev::FaceLaunch &, const int *, int, int, const dev::SurfaceParams &,
                                          const double *, double *, double *, int *, int, cudaStream_t);
template cudaError_t launch_faces<float>(const dev::FaceLaunch &, const int *, int, int, const dev::SurfaceParams &,
                                         const double *, float *, double *, int *, int, cudaStream_t);

template <typename T>
cudaError_t launch_gather(int nv, const T *partial, const int *off, double *g, cudaStream_t s) {
  if (nv <= 0) return cudaSuccess;
  dev::gather_kernel<T><<<grid_for(nv, 256), 256, 0, s>>>(nv, partial, off, g);
  return cudaGetLastError();
}
template cudaError_t launch_gather<double>(int, const double *, const int *, double *, cudaStream_t);
template cudaError_t launch_gather<float>(int, const float *, const int *, double *, cudaStream_t);

cudaError_t launch_reduce_terms(int nmesh, const int *seg, const double *terms, double *E, double *parts,
                                double *galpha, cudaStream_t s) {
  dev::reduce_terms_kernel<<<nmesh, 256, 0, s>>>(seg, terms, E, parts, galpha);
  return cudaGetLastError();
}

cudaError_t launch_step_local(int nv, const StepArgs &a, const uint64_t *step, double *r, double *p, const double *g,
                              const int *status, cudaStream_t s) {
  dev::step_local_kernel<<<grid_for(nv, 256), 256, 0, s>>>(nv, a, step, r, p, g, status);
  return cudaGetLastError();
}
cudaError_t launch_kick(int nv, const StepArgs &a, const uint64_t *step, double *p, const double *g, const int *status,
                        cudaStream_t s) {
  dev::kick_kernel<<<grid_for(nv, 256), 256, 0, s>>>(nv, a, step, p, g, status);
  return cudaGetLastError();
}
cudaError_t launch_drift(int nv, const StepArgs &a, double *r, double *p, const double *qdot, const int *status,
                         cudaStream_t s) {
  dev::drift_kernel<<<grid_for(3 * nv, 256), 256, 0, s>>>(nv, a, r, p, qdot, status);
  return cudaGetLastError();
}
cudaError_t launch_spmv(int nrow, const int *row_ptr, const int *col, const double *val, const double *scalev,
                        double scale, const double *alphas, const double *in, double *out, int accumulate,
                        cudaStream_t s) {
  if (nrow <= 0) return cudaSuccess;
  int warps_per_block = 8;
  int grid = grid_for(nrow, warps_per_block);
  if (grid > 152 * 16) grid = 152 * 16;
  dev::spmv_kernel<<<grid, 32 * warps_per_block, 0, s>>>(nrow, row_ptr, col, val, scalev, scale, alphas, in, out,
                                                        accumulate);
  return cudaGetLastError();
}
cudaError_t launch_record_energy(const double *E, double *energies, const uint64_t *runidx, double threshold,
                                 int *status, cudaStream_t s) {
  dev::record_energy_kernel<<<1, 1, 0, s>>>(E, energies, runidx, threshold, status);
  return cudaGetLastError();
}
cudaError_t launch_advance_step(uint64_t *step, uint64_t *runidx, cudaStream_t s) {
  dev::advance_step_kernel<<<1, 1, 0, s>>>(step, runidx);
  return cudaGetLastError();
}

}  // namespace umcp
