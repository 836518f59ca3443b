// Kernels of the membrane-surface hot path. See kernels.cuh for the model
// and launch.h for the contracts.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <mutex>

#include "kernels.cuh"
#include "launch.h"
#include "philox.h"

namespace umcp {
namespace dev {

template <typename T>
struct alignas(4 * sizeof(T)) Q4 {
  T x, y, z, w;
};

template <typename T, int NCP, int NPT>
struct FaceSmem {
  static constexpr int NC4 = (NCP + 3) / 4;  // control points in chunks of four
  static constexpr int NCPP = NC4 * 4;
  static constexpr int HW = FaceCfg<T>::half_warps;
  Q4<T> B[NPT][5][NC4];           // basis rows u,v,uu,uv,vv of point p
  Q4<T> X[HW][NCPP];              // centred, alpha-scaled control points
  Q4<T> Tc[HW][NPT][NCPP + 1];    // point p's contribution to each control point (+1 row pad: no bank conflicts)
  T W[NPT];
  double red[HW][6];
  __device__ __forceinline__ void *scratch() { return &Tc[0][0][0]; }
};

// Precision form (the half-warp kernel runs the irregular faces there; the
// regular ones take face_tpf_kernel): control points and per-point contributions are stored
// coordinate-major, so four control points of one coordinate are one float4
// and both contractions run as paired FP32 multiply-adds (two control points
// per instruction).
//  Xt[hw][c][cp]                 coordinate c of the centred control points
//  Tc[hw][(c * NPT + p) * TROW + cp]  point p's contribution to control point cp
// TROW makes the 16-byte row stride odd (conflict-free float4 stores by the
// point lanes); THW puts the two half-warps of a warp 16 banks apart, so the
// control-point lanes' scalar reads do not conflict either.
template <int NCP, int NPT>
struct FaceSmem<float, NCP, NPT> {
  static constexpr int NC4 = (NCP + 3) / 4;
  static constexpr int NCPP = NC4 * 4;
  static constexpr int HW = FaceCfg<float>::half_warps;
  static constexpr int TROW = NCPP + ((NC4 % 2 == 0) ? 4 : 0);
  static constexpr int TSZ = 3 * NPT * TROW;
  static constexpr int THW = TSZ + (48 - TSZ % 32) % 32;
  static_assert(THW % 32 == 16 && THW % 4 == 0, "half-warp stride");
  Q4<float> B[NPT][5][NC4];
  alignas(16) float Xt[HW][3][NCPP];
  alignas(16) float Dt[HW][3][NCPP];  // the same control points' change from the reference state
  alignas(16) float Tc[HW][THW];
  float W[NPT];
  double red[HW][6];
  __device__ __forceinline__ void *scratch() { return &Tc[0][0]; }
};

// Error-free sum: s + e == a + b exactly (Knuth's two-sum).
// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization may start while the kernel before it on the stream finishes;
// it waits here, before its first read of that kernel's results (a no-op
// when it was launched without the attribute).
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Per-half-warp sums of a face's energy terms and dE/dalpha: FP64 in the
// plain path; FP32 with Kahan compensation in the precision form, which keeps
// the FP64 pipe out of the face loop.
template <typename T>
struct HalfWarpSums;
template <>
struct HalfWarpSums<double> {
  double s[6] = {0, 0, 0, 0, 0, 0};
  __device__ __forceinline__ void add(int q, double v) { s[q] += v; }
  __device__ __forceinline__ double get(int q) const { return s[q]; }
};
template <>
struct HalfWarpSums<float> {
  float s[6] = {0, 0, 0, 0, 0, 0}, c[6] = {0, 0, 0, 0, 0, 0};
  __device__ __forceinline__ void add(int q, float v) {
    float y = v - c[q], t = s[q] + y;
    c[q] = (t - s[q]) - y;
    s[q] = t;
  }
  __device__ __forceinline__ double get(int q) const { return (double)s[q] - (double)c[q]; }
};

// Fixed-order sum of the block partials, done by one block: thread t sums
// rows t, t+NT, ..., then a shared-memory tree. Writes E, its parts and
// dE/dalpha; in a run also records E, flags non-finite or diverging energies
// (src/hd.C:1280-1305) and advances the run index.
template <int NT>
__device__ void finish_sums(const FinishArgs &F, const double *__restrict__ blockpart, double (*red)[NT]) {
  double a[6] = {0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < F.nblk; b += NT)
#pragma unroll
    for (int q = 0; q < 6; ++q) a[q] += __ldcg(&blockpart[6 * (size_t)b + q]);
#pragma unroll
  for (int q = 0; q < 6; ++q) red[q][threadIdx.x] = a[q];
  __syncthreads();
  for (int width = NT / 2; width > 0; width >>= 1) {
    if ((int)threadIdx.x < width)
#pragma unroll
      for (int q = 0; q < 6; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + width];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double e = red[0][0] + red[1][0] + red[2][0];
    double ga[3] = {red[3][0], red[4][0], red[5][0]};
    if (F.gterm) {  // the global restraints, summed before the face pass
      e += F.gterm[kGeoE];
      for (int c = 0; c < 3; ++c) ga[c] += F.gterm[kGeoDAlpha + c];
    }
    if (F.E) F.E[0] = e;
    if (F.parts) { F.parts[0] = red[0][0]; F.parts[1] = red[1][0]; F.parts[2] = red[2][0]; }
    if (F.galpha) { F.galpha[0] += ga[0]; F.galpha[1] += ga[1]; F.galpha[2] += ga[2]; }
    if (!isfinite(e)) atomicOr(F.status, kStatusNonFinite);
    if (F.energies) {
      const uint64_t idx = F.cnt[1];
      F.energies[idx] = e;
      if (F.threshold > 0 && idx > 0 && e - F.energies[idx - 1] > F.threshold) atomicOr(F.status, kStatusDiverged);
      F.cnt[1] = idx + 1;
    }
  }
}

template <typename T>
__device__ __forceinline__ T point_data(const double *d64, const float *d32, size_t i) {
  if constexpr (sizeof(T) == 8) return d64[i];
  else return d32[i];
}

// The moduli in the arithmetic type, converted once per launch (or per
// tile) rather than per face: conversions from FP64 run on the narrow FP64 pipe.
template <typename T>
struct Moduli {
  T kc, KA, kg, k_reg;
  __device__ __forceinline__ explicit Moduli(const SurfaceParams &P)
      : kc((T)P.kc), KA((T)P.KA), kg((T)P.kg), k_reg((T)P.k_reg) {}
};

// Global data of one face, loaded one face ahead (control-point indices two
// ahead) so the loads are in flight while the previous face computes.
template <typename T>
struct FaceAhead {
  int img[3] = {0, 0, 0};
  float hi[3] = {0, 0, 0}, lo[3] = {0, 0, 0};  // precision form
  float dsp[3] = {0, 0, 0};                    // precision form: r - r0
  double X[3] = {0, 0, 0};                     // plain path (image position)
  T g0 = 1, rr0 = 0, P2 = 0, Hbar = 0, Pres = 0;
  int dest = 0;
};

// Faces at or past end are not loaded.
template <int NCP>
__device__ __forceinline__ uint32_t load_cp(const FaceSrc &S, int f, int end, int lane) {
  return (f >= 0 && f < end && lane < NCP) ? __ldg(&S.cp[(size_t)f * NCP + lane]) : 0u;
}

template <typename T, int NCP, int NPT>
__device__ __forceinline__ void load_ahead(const FaceSrc &S, const SurfaceParams &P, int f, int end, uint32_t packed,
                                           int lane, FaceAhead<T> &a) {
  if (f < 0 || f >= end) return;
  if (lane < NCP) {
    const int v = (int)(packed & kVertexMask), code = (int)(packed >> kVertexBits);
    a.img[0] = code % 3 - 1; a.img[1] = (code / 3) % 3 - 1; a.img[2] = code / 9 - 1;
    if constexpr (sizeof(T) == 8) {
#pragma unroll
      for (int c = 0; c < 3; ++c)
        a.X[c] = S.r[3 * (size_t)v + c] + a.img[0] * P.box[0][c] + a.img[1] * P.box[1][c] + a.img[2] * P.box[2][c];
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        a.hi[c] = S.rhi[3 * (size_t)v + c];
        a.lo[c] = S.rlo[3 * (size_t)v + c];
        a.dsp[c] = S.dsp[3 * (size_t)v + c];
      }
    }
    a.dest = __ldg(&S.dest[(size_t)f * NCP + lane]);
  }
  if (lane < NPT) {
    const size_t pi = (size_t)f * NPT + lane;
    a.g0 = point_data<T>(S.g0, S.g0f, pi);
    a.rr0 = point_data<T>(S.rr0, S.rr0f, pi);
  }
  a.P2 = point_data<T>(S.comp, S.compf, 3 * (size_t)f);
  a.Hbar = point_data<T>(S.comp, S.compf, 3 * (size_t)f + 1);
  a.Pres = point_data<T>(S.comp, S.compf, 3 * (size_t)f + 2);
}

// Stage the block's copy of the patch type's basis rows and weights.
template <typename T, int NCP, int NPT, int NT>
__device__ __forceinline__ void stage_basis(FaceSmem<T, NCP, NPT> &sm, const double *basis, const double *weight) {
  constexpr int NCPP = FaceSmem<T, NCP, NPT>::NCPP, HW = FaceSmem<T, NCP, NPT>::HW;
  T *b = &sm.B[0][0][0].x;
  for (int i = threadIdx.x; i < NPT * 5 * NCPP; i += NT) b[i] = (T)basis[i];
  for (int i = threadIdx.x; i < NPT; i += NT) sm.W[i] = (T)weight[i];
  // padding control points stay zero
  if constexpr (sizeof(T) == 4)
    for (int i = threadIdx.x; i < HW * 3 * NCPP; i += NT) (&sm.Xt[0][0][0])[i] = (&sm.Dt[0][0][0])[i] = 0.f;
  else
    for (int i = threadIdx.x; i < HW * NCPP; i += NT) sm.X[i / NCPP][i % NCPP] = Q4<T>{0, 0, 0, 0};
}

// Precision form, lane = quadrature point p: the five contractions, the
// pointwise energy and adjoint, and p's contribution to every control point.
// Both contractions use paired FP32 multiply-adds over two control points at
// once (__ffma2_rn), which halves their instruction count:
//   K[k]_c = sum_j B[p][k][j] X_c[j]    even j in the pair's first half, odd j
//                                       in its second; the halves added last
//   T_c[j] = sum_k B[p][k][j] Kb[k]_c   j, j+1 in one pair, Kb duplicated
template <int NCP, int NPT>
__device__ __forceinline__ void point_pass_f32(FaceSmem<float, NCP, NPT> &sm, int hw, int lane,
                                               const FaceAhead<float> &cur, float dudv, const Moduli<float> &mod,
                                               bool reg_alpha, float *ea, float *ec, float *er, float dreg[3]) {
  using S = FaceSmem<float, NCP, NPT>;
  constexpr int NC4 = S::NC4, TROW = S::TROW;
  float2 A[5][3], Ad[2][3];  // Ad: the u and v rows contracted with the displacements (Dt)
#pragma unroll
  for (int k = 0; k < 5; ++k)
#pragma unroll
    for (int c = 0; c < 3; ++c) A[k][c] = make_float2(0.f, 0.f);
#pragma unroll
  for (int k = 0; k < 2; ++k)
#pragma unroll
    for (int c = 0; c < 3; ++c) Ad[k][c] = make_float2(0.f, 0.f);
#pragma unroll 1
  for (int c4 = 0; c4 < NC4; ++c4) {
    float4 x[3], d[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      x[c] = *reinterpret_cast<const float4 *>(&sm.Xt[hw][c][4 * c4]);
      d[c] = *reinterpret_cast<const float4 *>(&sm.Dt[hw][c][4 * c4]);
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const Q4<float> b = sm.B[lane][k][c4];
      const float2 b01 = make_float2(b.x, b.y), b23 = make_float2(b.z, b.w);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        A[k][c] = __ffma2_rn(b01, make_float2(x[c].x, x[c].y), A[k][c]);
        A[k][c] = __ffma2_rn(b23, make_float2(x[c].z, x[c].w), A[k][c]);
        if (k < 2) {
          Ad[k][c] = __ffma2_rn(b01, make_float2(d[c].x, d[c].y), Ad[k][c]);
          Ad[k][c] = __ffma2_rn(b23, make_float2(d[c].z, d[c].w), Ad[k][c]);
        }
      }
    }
  }
  Vec3<float> K[5], dR[2];
#pragma unroll
  for (int k = 0; k < 5; ++k) K[k] = {A[k][0].x + A[k][0].y, A[k][1].x + A[k][1].y, A[k][2].x + A[k][2].y};
#pragma unroll
  for (int k = 0; k < 2; ++k) dR[k] = {Ad[k][0].x + Ad[k][0].y, Ad[k][1].x + Ad[k][1].y, Ad[k][2].x + Ad[k][2].y};
  Vec3<float> Kb[5], Kreg[2];
  point_adjoint<float>(K, sm.W[lane], cur.g0, cur.rr0, dudv, cur.P2, cur.Hbar, cur.Pres, mod.kc, mod.KA, mod.kg,
                       mod.k_reg, ea, ec, er, Kb, Kreg, dR);
  float2 Kd[5][3];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    Kd[k][0] = make_float2(Kb[k].x, Kb[k].x);
    Kd[k][1] = make_float2(Kb[k].y, Kb[k].y);
    Kd[k][2] = make_float2(Kb[k].z, Kb[k].z);
  }
  float *tc = &sm.Tc[hw][lane * TROW];
#pragma unroll 1
  for (int c4 = 0; c4 < NC4; ++c4) {
    Q4<float> b[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) b[k] = sm.B[lane][k][c4];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float2 t01 = __fmul2_rn(make_float2(b[0].x, b[0].y), Kd[0][c]);
      float2 t23 = __fmul2_rn(make_float2(b[0].z, b[0].w), Kd[0][c]);
#pragma unroll
      for (int k = 1; k < 5; ++k) {
        t01 = __ffma2_rn(make_float2(b[k].x, b[k].y), Kd[k][c], t01);
        t23 = __ffma2_rn(make_float2(b[k].z, b[k].w), Kd[k][c], t23);
      }
      *reinterpret_cast<float4 *>(&tc[c * NPT * TROW + 4 * c4]) = make_float4(t01.x, t01.y, t23.x, t23.y);
    }
    if (reg_alpha) {
      // igrad's box-scale derivative takes the angle-term adjoint with one
      // more alpha factor (src/grad.C:7414-7421).
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float bk0 = (&b[0].x)[j], bk1 = (&b[1].x)[j];
        dreg[0] += (bk0 * Kreg[0].x + bk1 * Kreg[1].x) * sm.Xt[hw][0][4 * c4 + j];
        dreg[1] += (bk0 * Kreg[0].y + bk1 * Kreg[1].y) * sm.Xt[hw][1][4 * c4 + j];
        dreg[2] += (bk0 * Kreg[0].z + bk1 * Kreg[1].z) * sm.Xt[hw][2][4 * c4 + j];
      }
    }
  }
}

// Energy, adjoint and gradient partials of one face by one half-warp:
//  1. lanes = control points: the control point's position relative to the
//     patch corner (control point 0) in its lattice image, times alpha. The
//     plain path forms it in FP64; the precision form from FP32 hi/lo pairs
//     with error-free sums, so the local coordinates carry full FP32
//     precision even across periodic images.
//  2. lanes = quadrature points: the five contractions (basis rows held per
//     point, control points broadcast), pointwise energy and adjoint, and the
//     adjoint's contribution to every control point (written transposed).
//  3. lanes = control points: sum the contributions over the points; write the
//     alpha-scaled gradient partial to its slot.
// Returns the face's energy terms and dE/dalpha summed over the half-warp.
template <typename T, int NCP, int NPT>
__device__ __forceinline__ void face_compute(FaceSmem<T, NCP, NPT> &sm, int hw, int lane, unsigned hmask,
                                             const FaceAhead<T> &cur, const SurfaceParams &P, const T alpha[3],
                                             const T ialpha[3], const T am1[3], const Moduli<T> &mod, T dudv,
                                             bool reg_alpha, T *__restrict__ partial, T e3[3], T da[3]) {
  constexpr int NC4 = FaceSmem<T, NCP, NPT>::NC4;
  const T kc = mod.kc, KA = mod.KA, kg = mod.kg, k_reg = mod.k_reg;
  // ---- 1. control points, relative to the patch corner
  T xl[3] = {0, 0, 0}, dx[3] = {0, 0, 0};
  if constexpr (sizeof(T) == 8) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double a = __shfl_sync(hmask, cur.X[c], 0, 16);
      xl[c] = alpha[c] * (cur.X[c] - a);
    }
  } else {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float ahi = __shfl_sync(hmask, cur.hi[c], 0, 16), alo = __shfl_sync(hmask, cur.lo[c], 0, 16);
      // lattice shift hi + lo (each term exact: images are -1, 0 or +1)
      float sh = 0.f, she = 0.f, shl = 0.f;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        float t, e;
        two_sum(sh, (float)cur.img[d] * P.box_hi[d][c], t, e);
        sh = t;
        she += e;
        shl += (float)cur.img[d] * P.box_lo[d][c];
      }
      float s1, e1, s2, e2;
      two_sum(cur.hi[c], sh, s1, e1);
      two_sum(s1, -ahi, s2, e2);
      const float lc = s2 + ((e1 + e2) + ((cur.lo[c] - alo) + (she + shl)));
      xl[c] = alpha[c] * lc;
      // change from the reference state (box scales 1 there): alpha L - L0 = (alpha - 1) L + (L - L0),
      // L - L0 = dsp - dsp of the corner (the lattice shifts cancel)
      const float d0 = __shfl_sync(hmask, cur.dsp[c], 0, 16);
      dx[c] = fmaf(am1[c], lc, cur.dsp[c] - d0);
    }
  }
  if constexpr (sizeof(T) == 4) {
    if (lane < NCP) {
      sm.Xt[hw][0][lane] = xl[0];
      sm.Xt[hw][1][lane] = xl[1];
      sm.Xt[hw][2][lane] = xl[2];
      sm.Dt[hw][0][lane] = dx[0];
      sm.Dt[hw][1][lane] = dx[1];
      sm.Dt[hw][2][lane] = dx[2];
    }
  } else {
    if (lane < NCP) sm.X[hw][lane] = Q4<T>{xl[0], xl[1], xl[2], T(0)};
  }
  __syncwarp(hmask);

  // ---- 2. lanes as quadrature points
  T ea = 0, ec = 0, er = 0;
  T dreg[3] = {0, 0, 0};
  if constexpr (sizeof(T) == 4) {
    if (lane < NPT) point_pass_f32<NCP, NPT>(sm, hw, lane, cur, dudv, mod, reg_alpha, &ea, &ec, &er, dreg);
  } else if (lane < NPT) {
    Vec3<T> K[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) K[k] = {0, 0, 0};
#pragma unroll 1
    for (int c4 = 0; c4 < NC4; ++c4) {
      const Q4<T> x0 = sm.X[hw][4 * c4], x1 = sm.X[hw][4 * c4 + 1], x2 = sm.X[hw][4 * c4 + 2],
                  x3 = sm.X[hw][4 * c4 + 3];
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        const Q4<T> b = sm.B[lane][k][c4];
        K[k].x += b.x * x0.x + b.y * x1.x + b.z * x2.x + b.w * x3.x;
        K[k].y += b.x * x0.y + b.y * x1.y + b.z * x2.y + b.w * x3.y;
        K[k].z += b.x * x0.z + b.y * x1.z + b.z * x2.z + b.w * x3.z;
      }
    }
    Vec3<T> Kb[5], Kreg[2];
    point_adjoint<T>(K, sm.W[lane], cur.g0, cur.rr0, dudv, cur.P2, cur.Hbar, cur.Pres, kc, KA, kg, k_reg, &ea, &ec,
                     &er, Kb, Kreg);
#pragma unroll 1
    for (int c4 = 0; c4 < NC4; ++c4) {
      Q4<T> b[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) b[k] = sm.B[lane][k][c4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const T bk0 = (&b[0].x)[j], bk1 = (&b[1].x)[j], bk2 = (&b[2].x)[j], bk3 = (&b[3].x)[j],
                bk4 = (&b[4].x)[j];
        Q4<T> t;
        t.x = bk0 * Kb[0].x + bk1 * Kb[1].x + bk2 * Kb[2].x + bk3 * Kb[3].x + bk4 * Kb[4].x;
        t.y = bk0 * Kb[0].y + bk1 * Kb[1].y + bk2 * Kb[2].y + bk3 * Kb[3].y + bk4 * Kb[4].y;
        t.z = bk0 * Kb[0].z + bk1 * Kb[1].z + bk2 * Kb[2].z + bk3 * Kb[3].z + bk4 * Kb[4].z;
        t.w = T(0);
        sm.Tc[hw][lane][4 * c4 + j] = t;
        if (reg_alpha) {
          // igrad's box-scale derivative takes the angle-term adjoint with
          // one more alpha factor (src/grad.C:7414-7421).
          const Q4<T> xx = sm.X[hw][4 * c4 + j];
          dreg[0] += (bk0 * Kreg[0].x + bk1 * Kreg[1].x) * xx.x;
          dreg[1] += (bk0 * Kreg[0].y + bk1 * Kreg[1].y) * xx.y;
          dreg[2] += (bk0 * Kreg[0].z + bk1 * Kreg[1].z) * xx.z;
        }
      }
    }
  }
  __syncwarp(hmask);

  // ---- 3. lanes as control points
  da[0] = da[1] = da[2] = 0;
  if (lane < NCP) {
    T G0 = 0, G1 = 0, G2 = 0;
    if constexpr (sizeof(T) == 4) {
      constexpr int TROW = FaceSmem<T, NCP, NPT>::TROW;
      const float *tc = &sm.Tc[hw][lane];
#pragma unroll
      for (int p = 0; p < NPT; ++p) {
        G0 += tc[p * TROW];
        G1 += tc[(NPT + p) * TROW];
        G2 += tc[(2 * NPT + p) * TROW];
      }
    } else {
#pragma unroll
      for (int p = 0; p < NPT; ++p) {
        const Q4<T> t = sm.Tc[hw][p][lane];
        G0 += t.x;
        G1 += t.y;
        G2 += t.z;
      }
    }
    const int d = cur.dest;
    partial[3 * (size_t)d] = alpha[0] * G0;
    partial[3 * (size_t)d + 1] = alpha[1] * G1;
    partial[3 * (size_t)d + 2] = alpha[2] * G2;
    // dE/dalpha_c = sum_x G_xc (X - X_0)_xc: the patch gradient sums to
    // zero, so coordinates relative to the corner give the same sum.
    da[0] = G0 * xl[0] * ialpha[0];
    da[1] = G1 * xl[1] * ialpha[1];
    da[2] = G2 * xl[2] * ialpha[2];
  }
  if (reg_alpha)
#pragma unroll
    for (int c = 0; c < 3; ++c) da[c] += (alpha[c] - T(1)) * ialpha[c] * dreg[c];
  e3[0] = ea; e3[1] = ec; e3[2] = er;
#pragma unroll
  for (int off = 8; off >= 1; off >>= 1)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      e3[c] += __shfl_xor_sync(hmask, e3[c], off, 16);
      da[c] += __shfl_xor_sync(hmask, da[c], off, 16);
    }
}

// Single mesh: one half-warp per face, persistent over the mesh's faces.
// Energy terms and dE/dalpha are summed per half-warp, then per block in a
// fixed order, and written as one block partial (no atomics on floats).
template <typename T, int NCP, int NPT>
__global__ void __launch_bounds__(FaceCfg<T>::threads, FaceCfg<T>::min_blocks)
    face_kernel(FaceLaunch L, const int *__restrict__ dest, SurfaceParams P, const double *__restrict__ r,
                const float *__restrict__ rhi, const float *__restrict__ rlo, const float *__restrict__ dsp,
                T *__restrict__ partial, double *__restrict__ blockpart, int *__restrict__ status, FinishArgs fin) {
  using S = FaceSmem<T, NCP, NPT>;
  constexpr int HW = S::HW, NT = FaceCfg<T>::threads;
  __shared__ S sm;
  stage_basis<T, NCP, NPT, NT>(sm, L.basis, L.weight);
  __syncthreads();
  grid_dependency_wait();  // the state comes from the kernels before

  const int hw = threadIdx.x >> 4, lane = threadIdx.x & 15;
  const unsigned hmask = (threadIdx.x & 16) ? 0xFFFF0000u : 0x0000FFFFu;
  const T alpha[3] = {(T)r[3 * P.nv], (T)r[3 * P.nv + 1], (T)r[3 * P.nv + 2]};
  const T ialpha[3] = {T(1) / alpha[0], T(1) / alpha[1], T(1) / alpha[2]};
  const T am1[3] = {(T)(r[3 * P.nv] - 1.0), (T)(r[3 * P.nv + 1] - 1.0), (T)(r[3 * P.nv + 2] - 1.0)};
  const T dudv = (T)L.dudv;
  const bool reg_alpha = L.irregular && P.k_reg != 0.0;
  const Moduli<T> mod(P);
  const FaceSrc src{L.cp, L.g0, L.rr0, L.comp, L.g0f, L.rr0f, L.compf, dest, r, rhi, rlo, dsp, L.nfaces};
  HalfWarpSums<T> acc;

  const int stride = gridDim.x * HW;
  int f = blockIdx.x * HW + hw;
  FaceAhead<T> cur, nxt;
  const int end = L.nfaces;
  uint32_t cp_next = load_cp<NCP>(src, f + stride, end, lane);
  load_ahead<T, NCP, NPT>(src, P, f, end, load_cp<NCP>(src, f, end, lane), lane, cur);

  for (; f < end; f += stride) {
    const uint32_t cp_after = load_cp<NCP>(src, f + 2 * stride, end, lane);
    load_ahead<T, NCP, NPT>(src, P, f + stride, end, cp_next, lane, nxt);
    cp_next = cp_after;
    T e3[3], da[3];
    face_compute<T, NCP, NPT>(sm, hw, lane, hmask, cur, P, alpha, ialpha, am1, mod, dudv, reg_alpha, partial, e3, da);
    acc.add(0, e3[0]); acc.add(1, e3[1]); acc.add(2, e3[2]);
    acc.add(3, da[0]); acc.add(4, da[1]); acc.add(5, da[2]);
    if (lane == 0 && !isfinite(e3[0] + e3[1] + e3[2])) atomicOr(status, kStatusNonFinite);
    cur = nxt;
    __syncwarp(hmask);
  }
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < 6; ++q) sm.red[hw][q] = acc.get(q);
  __syncthreads();
  if (threadIdx.x < 6) {
    double s = 0;
#pragma unroll
    for (int h = 0; h < HW; ++h) s += sm.red[h][threadIdx.x];
    blockpart[6 * (size_t)(L.block_base + blockIdx.x) + threadIdx.x] = s;
  }
  if (fin.done) {
    // The last block of the mesh's last face launch to finish sums all block
    // partials (the order of that sum does not depend on which block it is).
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(fin.done, 1u) == (unsigned)fin.nblk - 1u);
    __syncthreads();
    if (last) {
      __threadfence();
      static_assert(sizeof(sm.Tc) >= sizeof(double) * 6 * NT, "finish scratch must fit in the transpose buffer");
      finish_sums<NT>(fin, blockpart, reinterpret_cast<double(*)[NT]>(sm.scratch()));
      if (threadIdx.x == 0) *fin.done = 0u;
    }
  }
}

// ---------------------------------------------------------------- tensor-core face pass
//
// Regular faces in the precision form, with the two basis contractions on the
// 5th-generation tensor cores (tcgen05, kind::f16 on fp16 hi/lo splits) and the
// pointwise energy and adjoint on the FP32 pipes. A CTA owns a tile of 128
// faces (the MMA's M; face = TMEM lane) and 256 threads: thread (face, half)
// takes the half-th quadrature point of each 2-point chunk.
//
// Affine centring. The box splines reproduce affine functions, so with the
// patch frame Eu = X2 - X0, Ev = X1 - X0 (control points 2 and 1 sit at
// lattice (1,0) and (0,1)) and X'_x = X_x - X0 - u_x Eu - v_x Ev:
//   Ru = Eu + sum b_u X',  Rv = Ev + sum b_v X',  S.. = sum b_.. X'.
// X' is of the size of the curvature, not of the patch, so the fp16 split
// errors scale with the curvature terms themselves.
//
// Per chunk j (points 2j, 2j+1):
//   GEMM1_j  D1[f, n] = sum_x X'[f, x] B1_j[n, x]      n = 8 h + k (point 2j+h, kind k)
//   pointwise: K -> energy terms, adjoint Kb (tcgen05.ld from D1, tcgen05.st into A2)
//   GEMM2_j  D2[f, x] += sum_n A2[f, n] B2_j[x, n]    (A from tensor memory)
// GEMM2_j and GEMM1_{j+1} are issued together behind one commit.
namespace tc {
// Tensor-core form of the regular-face pass (precision form, 12 control
// points, 15 quadrature points). A CTA owns a tile of 128 faces, one face per
// TMEM lane, and evaluates its points in four chunks of four; thread half h
// (threads 128 h .. 128 h + 127) evaluates points 4 j + 2 h and 4 j + 2 h + 1
// of chunk j and owns control points 8 h .. 8 h + 7 (those below 12).
//
// Per chunk, with fp16 operands split in two (x = hi + lo, about 22 bits) and
// FP32 accumulation in TMEM:
//   GEMM1  D1[face][n] = sum_k X'[face][k] B1[n][k]   per coordinate, K = 32, N = 48
//   GEMM2  D2[face][n] = sum_k Kb[face][k] B2[n][k]   per coordinate, K = 48, N = 32
// X' are the affine-centred control points, Kb the pointwise adjoints. The
// three products of a split (hi hi, lo hi, hi lo) come out of one pass:
// A = [a_hi | a_lo] along K and B's columns [b_hi | b_lo] along N, the lo-lo
// block left zero. Each instruction costs about the same time whatever its N,
// so the contractions are laid out for the fewest instructions: 6 (GEMM1) +
// 9 (GEMM2) per chunk, 60 per tile.
//
// Scaling: every A row is scaled by a power of two that puts its largest
// magnitude in [2^13, 2^14) (per face, coordinate and, for Kb, chunk), the
// basis by 2^8, so neither fp16 half of an operand leaves fp16's normal range
// in a way that costs accuracy. D2 is read back per chunk and summed in
// registers, which lets each chunk's Kb carry its own scale.
constexpr int kThreads = 256, kFaces = 128, kNpt = 15, kNcp = 12, kChunks = 4;
constexpr int kN1 = 48, kK1 = 32, kN2 = 32, kK2 = 48;
constexpr int kSbo1 = kK1 / 8 * 128, kSbo2 = kK2 / 8 * 128;  // bytes between 8-row core-matrix groups
constexpr uint32_t kTmemCols = 256, kD1 = 0, kD2 = 3 * kN1;  // TMEM column bases
constexpr float kBasisScale = 256.f, kInvBasisScale = 1.f / 256.f;
// lattice position of control point x in the regular patch (ceff order)
__constant__ int kLatU[12] = {0, 0, 1, 1, 0, -1, -1, -1, 0, 1, 2, 2};
__constant__ int kLatV[12] = {0, 1, 0, -1, -1, 0, 1, 2, 2, 1, 0, -1};

struct Smem {
  uint4 A1[3][kFaces * kK1 / 8];  // X' (hi at k 0..11, lo at k 16..27), K-major core matrices of 8 rows x 16 B
  uint4 A2[3][kFaces * kK2 / 8];  // Kb: thread half h's slots at k 24 h .. 24 h + 23
  uint4 B1[kChunks][kN1 * kK1 / 8];
  uint4 B2[kChunks][kN2 * kK2 / 8];
  float xmax[2][3][kFaces];       // per-row maxima exchanged between the two thread halves
  float Dd[3][kNcp][kFaces];      // control points' change from the reference state (FP32, per face)
  float Buv[kNpt][2][kNcp];       // basis rows u, v in FP32, for the area strain's tangent changes
  float W[16];
  uint64_t mbar;
  uint32_t tmem;
  int abort;
};
constexpr size_t kSmemBytes = sizeof(Smem) + 1024;

// byte offset of element (row, k) of a K-major fp16 operand whose 8-row groups are sbo bytes apart
__host__ __device__ constexpr int core_off(int row, int k, int sbo) {
  return (row >> 3) * sbo + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}
// GEMM1 column of thread half h's slot s (s < 20): slots 0..15 at 16 h + s,
// slots 16..19 at 32 + 8 h + s - 16, so both halves read them with one x16
// and one x8 load at aligned columns.
__host__ __device__ constexpr int d1_col(int h, int s) { return s < 16 ? 16 * h + s : 32 + 8 * h + (s - 16); }

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
// shared-memory matrix descriptor: K-major, no swizzle, 128 B between K-adjacent core matrices
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         ((uint64_t)1 << 46);
}
// instruction descriptor: D F32, A and B F16, both K-major, M = 128
__host__ __device__ constexpr uint32_t idesc(uint32_t n) { return (1u << 4) | ((n >> 3) << 17) | ((128u >> 4) << 24); }

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
               ::"r"(d), "l"(a), "l"(b), "r"(id), "r"(acc));
}
__device__ __forceinline__ void commit(uint64_t *mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar)));
}
// Bounded wait on the mbarrier's phase; false when it gave up.
__device__ __forceinline__ bool wait_phase(uint64_t *mbar, uint32_t phase) {
  uint32_t done = 0;
  for (int it = 0; it < (1 << 24) && !done; ++it)
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done) : "r"(smem_u32(mbar)), "r"(phase));
  return done != 0;
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;"); }

// TMEM loads of 8 + 8 consecutive columns of this warp's 32 lanes; the wait is
// inside the same statement, so no use of a result can move above it.
__device__ __forceinline__ void ld8_8(uint32_t ta, uint32_t tb, float v[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%16];\n"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8,%9,%10,%11,%12,%13,%14,%15}, [%17];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(ta), "r"(tb));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// The GEMM1 results of this thread's two points, all three coordinates: per
// coordinate c, 16 + 8 columns at ta[c], tb[c], with one wait.
__device__ __forceinline__ void ld_d1(const uint32_t ta[3], const uint32_t tb[3], float v[3][24]) {
  uint32_t r[72];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%72];\n"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%16,%17,%18,%19,%20,%21,%22,%23}, [%73];\n"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39}, [%74];\n"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%40,%41,%42,%43,%44,%45,%46,%47}, [%75];\n"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%76];\n"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%64,%65,%66,%67,%68,%69,%70,%71}, [%77];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63]), "=r"(r[64]), "=r"(r[65]), "=r"(r[66]), "=r"(r[67]), "=r"(r[68]), "=r"(r[69]), "=r"(r[70]), "=r"(r[71])
      : "r"(ta[0]), "r"(tb[0]), "r"(ta[1]), "r"(tb[1]), "r"(ta[2]), "r"(tb[2]));
#pragma unroll
  for (int i = 0; i < 72; ++i) v[i / 24][i % 24] = __uint_as_float(r[i]);
}
// 2^e with m * 2^e in [2^13, 2^14) for a finite m > 0 (and its inverse); for
// m = 0 or tiny m the largest scale whose inverse is a normal float; an
// infinite or NaN m gives a small scale, so the values stay non-finite.
__device__ __forceinline__ void pow2_scale(float m, float &s, float &inv) {
  const int e = (int)((__float_as_uint(m) >> 23) & 0xFFu);
  const int f = e == 0 ? 253 : min(253, 267 - e);  // biased exponent of the scale
  s = __uint_as_float((uint32_t)f << 23);
  inv = __uint_as_float((uint32_t)(254 - f) << 23);
}
// (a, b) as an fp16 pair, a in the low half
__device__ __forceinline__ uint32_t cvt2(float a, float b) {
  uint32_t r;
  asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(b), "f"(a));
  return r;
}
// x0, x1 (already scaled) = hi + lo: hi rounded to 11 significant bits by
// Veltkamp's split (factor 2^13 + 1; explicitly rounded operations, so
// nothing is contracted), exact in fp16; lo = x - hi, exact in FP32 and
// rounded to fp16.
__device__ __forceinline__ void split_pair(float x0, float x1, uint32_t &hi, uint32_t &lo) {
  const float g0 = __fmul_rn(x0, 8193.f), g1 = __fmul_rn(x1, 8193.f);
  const float h0 = __fsub_rn(g0, __fsub_rn(g0, x0)), h1 = __fsub_rn(g1, __fsub_rn(g1, x1));
  hi = cvt2(h0, h1);
  lo = cvt2(__fsub_rn(x0, h0), __fsub_rn(x1, h1));
}

// CTA set-up: mbarrier, TMEM, the basis operands of every chunk, the weights.
__device__ void setup(Smem &sm, const double *__restrict__ basis, const double *__restrict__ weight) {
  const int tid = threadIdx.x;
  // fp16 hi or lo part of the scaled basis value of point p, derivative d, control point x
  auto bval = [&](int p, int d, int x, bool lo) -> __half {
    const double b = basis[((size_t)p * 5 + d) * kNcp + x] * (double)kBasisScale;
    const __half hi = __float2half_rn((float)b);
    return lo ? __float2half_rn((float)(b - (double)__half2float(hi))) : hi;
  };
  __half *b1 = reinterpret_cast<__half *>(&sm.B1[0][0]);
  for (int e = tid; e < kChunks * kN1 * kK1; e += kThreads) {
    const int j = e / (kN1 * kK1), n = (e / kK1) % kN1, k = e % kK1;
    const int h = n < 32 ? n >> 4 : (n - 32) >> 3, s = n < 32 ? n & 15 : 16 + ((n - 32) & 7);
    const int x = k & 15;
    __half v = __float2half_rn(0.f);
    if (s < 20 && x < kNcp) {
      const int q = (s % 10) / 5, d = s % 5, p = 4 * j + 2 * h + q;
      if (p < kNpt) {
        if (s < 10) v = bval(p, d, x, false);  // (a_hi + a_lo) b_hi
        else if (k < 16) v = bval(p, d, x, true);  // a_hi b_lo
      }
    }
    b1[(size_t)j * kN1 * kK1 + core_off(n, k, kSbo1) / 2] = v;
  }
  __half *b2 = reinterpret_cast<__half *>(&sm.B2[0][0]);
  for (int e = tid; e < kChunks * kN2 * kK2; e += kThreads) {
    const int j = e / (kN2 * kK2), n = (e / kK2) % kN2, k = e % kK2;
    const int x = n & 15, h = k / 24, s = k % 24;
    __half v = __float2half_rn(0.f);
    if (x < kNcp && s < 20) {
      const int q = (s % 10) / 5, d = s % 5, p = 4 * j + 2 * h + q;
      if (p < kNpt) {
        if (s < 10) v = bval(p, d, x, n >= 16);  // a_hi rows: [b_hi | b_lo]
        else if (n < 16) v = bval(p, d, x, false);  // a_lo rows: [b_hi | 0]
      }
    }
    b2[(size_t)j * kN2 * kK2 + core_off(n, k, kSbo2) / 2] = v;
  }
  if (tid < 16) sm.W[tid] = tid < kNpt ? (float)weight[tid] : 0.f;
  for (int e = tid; e < kNpt * 2 * kNcp; e += kThreads) {
    const int p = e / (2 * kNcp), k = (e / kNcp) % 2, x = e % kNcp;
    sm.Buv[p][k][x] = (float)basis[((size_t)p * 5 + k) * kNcp + x];
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&sm.mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
    sm.abort = 0;
  }
  if ((tid >> 5) == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("fence.proxy.async.shared::cta;");
  fence_before();
  __syncthreads();
  fence_after();
}

__device__ void teardown(Smem &sm, uint32_t phase, bool pending) {
  // An aborted tile may leave MMAs in flight: give them a bounded wait before
  // the tensor memory they write is freed.
  if (pending && threadIdx.x == 0) wait_phase(&sm.mbar, phase);
  fence_before();
  __syncthreads();
  fence_after();
  if ((threadIdx.x >> 5) == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(sm.tmem), "r"(kTmemCols));
}

__device__ __forceinline__ void issue_gemm1(Smem &sm, uint32_t tmem, int j) {
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int ks = 0; ks < kK1 / 16; ++ks)
      mma(tmem + kD1 + kN1 * c, sdesc(smem_u32(sm.A1[c]) + 256 * ks, kSbo1), sdesc(smem_u32(sm.B1[j]) + 256 * ks, kSbo1),
          idesc(kN1), ks);
}
__device__ __forceinline__ void issue_gemm2(Smem &sm, uint32_t tmem, int j) {
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int ks = 0; ks < kK2 / 16; ++ks)
      mma(tmem + kD2 + kN2 * c, sdesc(smem_u32(sm.A2[c]) + 256 * ks, kSbo2), sdesc(smem_u32(sm.B2[j]) + 256 * ks, kSbo2),
          idesc(kN2), ks);
}

// Adds chunk D2 (scaled by inv, per coordinate) into G: the hi- and lo-basis columns of this thread's control points.
__device__ __forceinline__ void gather_d2(uint32_t tmem, uint32_t lane_base, int h, const float inv[3], float G[3][8]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float v[16];
    ld8_8(tmem + lane_base + kD2 + kN2 * c + 8 * h, tmem + lane_base + kD2 + kN2 * c + 16 + 8 * h, v);
#pragma unroll
    for (int i = 0; i < 8; ++i) G[c][i] += (v[i] + v[8 + i]) * inv[c];
  }
}

// One tile of up to 128 faces [first, first + count) of source S. Returns
// false if a wait gave up (the CTA then stops).
__device__ bool tile(Smem &sm, const FaceSrc &S, const SurfaceParams &P, const float alpha[3], const float ialpha[3],
                     const float am1[3], const Moduli<float> &mod, float dudv, int first, int count,
                     float *__restrict__ partial,
                     HalfWarpSums<float> &acc, uint32_t &phase) {
  const int tid = threadIdx.x, fs = tid & (kFaces - 1), h = tid >> 7;
  const uint32_t tmem = sm.tmem, lane_base = (uint32_t)(32 * ((tid >> 5) & 3)) << 16;
  const bool active = fs < count;
  const int f = first + fs;
  const int nx = h == 0 ? 8 : kNcp - 8;  // control points of this thread
  float Eu[3] = {0, 0, 0}, Ev[3] = {0, 0, 0}, sA[3], iA[3];
  float P2 = 0, Hbar = 0, Pres = 0;
  {
    float xp[8][3];
#pragma unroll
    for (int i = 0; i < 8; ++i) xp[i][0] = xp[i][1] = xp[i][2] = 0.f;
    if (active) {
      const uint32_t *cp = S.cp + (size_t)f * kNcp;
      // the corner (control point 0) is in the home image: coordinates are relative to its hi/lo pair
      const int v0 = (int)(__ldg(&cp[0]) & kVertexMask);
      float chi[3], clo[3], cd[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        chi[c] = S.rhi[3 * (size_t)v0 + c];
        clo[c] = S.rlo[3 * (size_t)v0 + c];
        cd[c] = S.dsp[3 * (size_t)v0 + c];
      }
      // out = alpha L; with d given, d = (alpha - 1) L + (dsp - dsp of the corner), the change from
      // the reference state (as in the thread-per-face kernel)
      auto local = [&](uint32_t packed, float out[3], float *d = nullptr) {
        const int v = (int)(packed & kVertexMask), code = (int)(packed >> kVertexBits);
        const int im[3] = {code % 3 - 1, (code / 3) % 3 - 1, code / 9 - 1};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float sh = 0.f, she = 0.f, shl = 0.f;
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            float t, e;
            two_sum(sh, (float)im[d] * P.box_hi[d][c], t, e);
            sh = t;
            she += e;
            shl += (float)im[d] * P.box_lo[d][c];
          }
          float s1, e1, s2, e2;
          const float hi = S.rhi[3 * (size_t)v + c], lo = S.rlo[3 * (size_t)v + c];
          two_sum(hi, sh, s1, e1);
          two_sum(s1, -chi[c], s2, e2);
          const float l = s2 + ((e1 + e2) + ((lo - clo[c]) + (she + shl)));
          out[c] = alpha[c] * l;
          if (d) d[c] = fmaf(am1[c], l, S.dsp[3 * (size_t)v + c] - cd[c]);
        }
      };
      local(__ldg(&cp[1]), Ev);  // lattice (0,1)
      local(__ldg(&cp[2]), Eu);  // lattice (1,0)
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        if (i < nx) {
          const int x = 8 * h + i;
          float xl[3], dx[3];
          local(__ldg(&cp[x]), xl, dx);
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            xp[i][c] = xl[c] - (float)kLatU[x] * Eu[c] - (float)kLatV[x] * Ev[c];
            sm.Dd[c][x][fs] = dx[c];
          }
        }
      }
      P2 = S.compf[3 * (size_t)f];
      Hbar = S.compf[3 * (size_t)f + 1];
      Pres = S.compf[3 * (size_t)f + 2];
    }
    // one scale per face and coordinate, from the largest |X'| of both halves
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float m = 0.f;
#pragma unroll
      for (int i = 0; i < 8; ++i) m = fmaxf(m, fabsf(xp[i][c]));
      sm.xmax[h][c][fs] = m;
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      pow2_scale(fmaxf(sm.xmax[0][c][fs], sm.xmax[1][c][fs]), sA[c], iA[c]);
      uint32_t whi[4], wlo[4];
#pragma unroll
      for (int i = 0; i < 8; i += 2) split_pair(xp[i][c] * sA[c], xp[i + 1][c] * sA[c], whi[i / 2], wlo[i / 2]);
      sm.A1[c][core_off(fs, 8 * h, kSbo1) / 16] = make_uint4(whi[0], whi[1], whi[2], whi[3]);
      sm.A1[c][core_off(fs, 16 + 8 * h, kSbo1) / 16] = make_uint4(wlo[0], wlo[1], wlo[2], wlo[3]);
      iA[c] *= kInvBasisScale;
    }
  }
  asm volatile("fence.proxy.async.shared::cta;");
  fence_before();
  __syncthreads();
  fence_after();
  if (tid == 0) {
    issue_gemm1(sm, tmem, 0);
    commit(&sm.mbar);
  }
  float e3[3] = {0, 0, 0}, G[3][8], iK[3] = {0, 0, 0};
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int i = 0; i < 8; ++i) G[c][i] = 0.f;
  bool ok = true;
#pragma unroll 1
  for (int j = 0; j < kChunks; ++j) {
    float g0[2] = {1.f, 1.f}, rr0[2] = {0.f, 0.f};
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int p = 4 * j + 2 * h + q;
      if (active && p < kNpt) {
        g0[q] = S.g0f[(size_t)f * kNpt + p];
        rr0[q] = S.rr0f[(size_t)f * kNpt + p];
      }
    }
    // warp 0 polls the mbarrier; the other warps sleep at the barrier
    ok = !__syncthreads_or((tid >> 5) == 0 && !wait_phase(&sm.mbar, phase)) && ok;
    phase ^= 1u;
    fence_after();
    if (j > 0) gather_d2(tmem, lane_base, h, iK, G);
    // the five contractions of both points, per coordinate: slot hi + slot lo
    Vec3<float> K[2][5];
    float v3[3][24];
    {
      const uint32_t t0 = tmem + lane_base + kD1;
      const uint32_t ta[3] = {t0 + 16 * h, t0 + kN1 + 16 * h, t0 + 2 * kN1 + 16 * h};
      const uint32_t tb[3] = {t0 + 32 + 8 * h, t0 + kN1 + 32 + 8 * h, t0 + 2 * kN1 + 32 + 8 * h};
      ld_d1(ta, tb, v3);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float *v = v3[c];
#pragma unroll
      for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int d = 0; d < 5; ++d) {
          const int shi = 5 * q + d, slo = 10 + 5 * q + d;
          const float val = (v[shi] + v[slo]) * iA[c];
          (c == 0 ? K[q][d].x : c == 1 ? K[q][d].y : K[q][d].z) = val;
        }
    }
    float kbv[3][2][5], km[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int p = 4 * j + 2 * h + q;
      K[q][0].x += Eu[0]; K[q][0].y += Eu[1]; K[q][0].z += Eu[2];
      K[q][1].x += Ev[0]; K[q][1].y += Ev[1]; K[q][1].z += Ev[2];
      Vec3<float> Kb[5], Kreg[2];
      if (active && p < kNpt) {
        // the tangents' change from the reference state, for the area strain
        Vec3<float> dR[2] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
#pragma unroll
        for (int x = 0; x < kNcp; ++x) {
          const float bu = sm.Buv[p][0][x], bv = sm.Buv[p][1][x];
          const float d0 = sm.Dd[0][x][fs], d1 = sm.Dd[1][x][fs], d2 = sm.Dd[2][x][fs];
          dR[0].x = fmaf(bu, d0, dR[0].x); dR[0].y = fmaf(bu, d1, dR[0].y); dR[0].z = fmaf(bu, d2, dR[0].z);
          dR[1].x = fmaf(bv, d0, dR[1].x); dR[1].y = fmaf(bv, d1, dR[1].y); dR[1].z = fmaf(bv, d2, dR[1].z);
        }
        float ea = 0, ec = 0, er = 0;
        point_adjoint<float>(K[q], sm.W[p], g0[q], rr0[q], dudv, P2, Hbar, Pres, mod.kc, mod.KA, mod.kg, mod.k_reg,
                             &ea, &ec, &er, Kb, Kreg, dR);
        e3[0] += ea; e3[1] += ec; e3[2] += er;
      } else {
#pragma unroll
        for (int d = 0; d < 5; ++d) Kb[d] = {0.f, 0.f, 0.f};
      }
#pragma unroll
      for (int d = 0; d < 5; ++d) {
        kbv[0][q][d] = Kb[d].x;
        kbv[1][q][d] = Kb[d].y;
        kbv[2][q][d] = Kb[d].z;
      }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
#pragma unroll
      for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int d = 0; d < 5; ++d) km[c] = fmaxf(km[c], fabsf(kbv[c][q][d]));
      sm.xmax[h][c][fs] = km[c];
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float sK;
      pow2_scale(fmaxf(sm.xmax[0][c][fs], sm.xmax[1][c][fs]), sK, iK[c]);
      iK[c] *= kInvBasisScale;
      // slots 0..9 hi, 10..19 lo, 20..23 zero; slot 5 q + d is point q's derivative d
      uint32_t hw[5], lw[5];
#pragma unroll
      for (int t = 0; t < 5; ++t) {
        const int s0 = 2 * t, s1 = 2 * t + 1;
        split_pair(kbv[c][s0 / 5][s0 % 5] * sK, kbv[c][s1 / 5][s1 % 5] * sK, hw[t], lw[t]);
      }
      uint4 *row = sm.A2[c];
      row[core_off(fs, 24 * h, kSbo2) / 16] = make_uint4(hw[0], hw[1], hw[2], hw[3]);
      row[core_off(fs, 24 * h + 8, kSbo2) / 16] = make_uint4(hw[4], lw[0], lw[1], lw[2]);
      row[core_off(fs, 24 * h + 16, kSbo2) / 16] = make_uint4(lw[3], lw[4], 0u, 0u);
    }
    asm volatile("fence.proxy.async.shared::cta;");
    fence_before();
    __syncthreads();
    fence_after();
    if (tid == 0) {
      issue_gemm2(sm, tmem, j);
      if (j + 1 < kChunks) issue_gemm1(sm, tmem, j + 1);
      commit(&sm.mbar);
    }
  }
  ok = !__syncthreads_or((tid >> 5) == 0 && !wait_phase(&sm.mbar, phase)) && ok;
  phase ^= 1u;
  if (!ok) return false;
  fence_after();
  gather_d2(tmem, lane_base, h, iK, G);
  // ---- gradient partials of this thread's control points and dE/dalpha;
  // X' comes back from the GEMM1 operand (hi + lo), the lattice part from Eu, Ev
  float da[3] = {0, 0, 0};
  if (active) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const uint4 wh = sm.A1[c][core_off(fs, 8 * h, kSbo1) / 16], wl = sm.A1[c][core_off(fs, 16 + 8 * h, kSbo1) / 16];
      const uint32_t hw[4] = {wh.x, wh.y, wh.z, wh.w}, lw[4] = {wl.x, wl.y, wl.z, wl.w};
      const float ia = iA[c] * kBasisScale;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        if (i < nx) {
          const int x = 8 * h + i;
          const __half hh = __ushort_as_half((unsigned short)(hw[i / 2] >> (16 * (i & 1))));
          const __half ll = __ushort_as_half((unsigned short)(lw[i / 2] >> (16 * (i & 1))));
          const float xl = (__half2float(hh) + __half2float(ll)) * ia + (float)kLatU[x] * Eu[c] + (float)kLatV[x] * Ev[c];
          const int dst = __ldg(&S.dest[(size_t)f * kNcp + x]);
          partial[3 * (size_t)dst + c] = alpha[c] * G[c][i];
          da[c] += G[c][i] * xl * ialpha[c];
        }
      }
    }
  }
  acc.add(0, e3[0]); acc.add(1, e3[1]); acc.add(2, e3[2]);
  acc.add(3, da[0]); acc.add(4, da[1]); acc.add(5, da[2]);
  // the next tile overwrites A1, A2 and the maxima, and its MMAs D1 and D2: everyone is done with them
  fence_before();
  __syncthreads();
  fence_after();
  return true;
}

// Fixed-order block sum of the six per-thread sums into out[6] (global). The
// reduction buffer lies over the Kb operand, which no MMA reads any more.
__device__ void block_sums(Smem &sm, const HalfWarpSums<float> &acc, double *out) {
  double(*red)[6] = reinterpret_cast<double(*)[6]>(&sm.A2[0][0]);
  for (int q = 0; q < 6; ++q) red[threadIdx.x][q] = acc.get(q);
  __syncthreads();
  if (threadIdx.x < 6) {
    double s = 0;
    for (int t = 0; t < kThreads; ++t) s += red[t][threadIdx.x];
    out[threadIdx.x] = s;
  }
  __syncthreads();
}
static_assert(sizeof(double) * 6 * kThreads <= sizeof(uint4) * 3 * kFaces * kK2 / 8, "reduction buffer");
}  // namespace tc

// Single mesh: persistent CTAs over the 128-face tiles of the regular group.
__global__ void __launch_bounds__(tc::kThreads, 2)
    face_tc_kernel(FaceLaunch L, const int *__restrict__ dest, SurfaceParams P, const double *__restrict__ r,
                   const float *__restrict__ rhi, const float *__restrict__ rlo, const float *__restrict__ dsp,
                   float *__restrict__ partial, double *__restrict__ blockpart, int *__restrict__ status,
                   FinishArgs fin) {
  extern __shared__ uint8_t tc_smem_raw[];
  tc::Smem &sm = *reinterpret_cast<tc::Smem *>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~(uintptr_t)1023);
  tc::setup(sm, L.basis, L.weight);
  const float alpha[3] = {(float)r[3 * P.nv], (float)r[3 * P.nv + 1], (float)r[3 * P.nv + 2]};
  const float ialpha[3] = {1.f / alpha[0], 1.f / alpha[1], 1.f / alpha[2]};
  const float am1[3] = {(float)(r[3 * P.nv] - 1.0), (float)(r[3 * P.nv + 1] - 1.0), (float)(r[3 * P.nv + 2] - 1.0)};
  const Moduli<float> mod(P);
  const FaceSrc src{L.cp, L.g0, L.rr0, L.comp, L.g0f, L.rr0f, L.compf, dest, r, rhi, rlo, dsp, L.nfaces};
  HalfWarpSums<float> acc;
  uint32_t phase = 0;
  bool ok = true;
  const int ntiles = (L.nfaces + tc::kFaces - 1) / tc::kFaces;
  for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
    const int first = t * tc::kFaces;
    ok = tc::tile(sm, src, P, alpha, ialpha, am1, mod, (float)L.dudv, first, min(tc::kFaces, L.nfaces - first), partial,
                  acc, phase);
  }
  if (!ok && threadIdx.x == 0) atomicOr(status, kStatusTimeout);
  tc::teardown(sm, phase, !ok);
  tc::block_sums(sm, acc, blockpart + 6 * (size_t)(L.block_base + blockIdx.x));
  if (fin.done) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(fin.done, 1u) == (unsigned)fin.nblk - 1u);
    __syncthreads();
    if (last) {
      __threadfence();
      finish_sums<tc::kThreads>(fin, blockpart, reinterpret_cast<double(*)[tc::kThreads]>(&sm.A2[0][0]));
      if (threadIdx.x == 0) *fin.done = 0u;
    }
  }
}

// The precision form's FP32 copies of one position coordinate x = r[i]:
// x = hi + lo to about 2^-48 relative, and dsp = x - r0[i] (the displacement
// from the reference state, rounded once from FP64).
__device__ __forceinline__ void store_f32_position(size_t i, double x, float *__restrict__ hi,
                                                   float *__restrict__ lo, const double *__restrict__ r0,
                                                   float *__restrict__ dsp) {
  const float h = (float)x;
  hi[i] = h;
  lo[i] = (float)(x - (double)h);
  dsp[i] = (float)(x - r0[i]);
}

__global__ void split_positions_kernel(int n, const double *__restrict__ r, float *__restrict__ hi,
                                       float *__restrict__ lo, const double *__restrict__ r0,
                                       float *__restrict__ dsp) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    store_f32_position(i, r[i], hi, lo, r0, dsp);
}

// dst |= *src (one thread): a status word handed on to another.
__global__ void status_merge_kernel(const int *__restrict__ src, int *__restrict__ dst) {
  const int v = *src;
  if (v) *dst |= v;
}

// Stand-alone form of the block-partial sum (used when the face launches do
// not finish themselves).
__global__ void finish_kernel(FinishArgs F, const double *__restrict__ blockpart) {
  __shared__ double red[6][256];
  finish_sums<256>(F, blockpart, red);
}

// Sum of a vertex's gradient partials in slot order: FP64 in the plain path,
// FP32 with Kahan compensation in the precision form.
// Sum of vertex v's gradient partials: its slots are loc[2 v] + 32 k for
// k < loc[2 v + 1] (32 vertices interleaved, so the 32 lanes of a warp read
// consecutive slots), summed in k order (FP64, or Kahan FP32).
template <typename T>
__device__ __forceinline__ void vertex_gradient(const T *__restrict__ partial, const int *__restrict__ loc, int v,
                                                double gg[3]) {
  const int base = loc[2 * (size_t)v], n = loc[2 * (size_t)v + 1];
  if constexpr (sizeof(T) == 8) {
    double a0 = 0, a1 = 0, a2 = 0;
    for (int k = 0; k < n; ++k) {
      const size_t s = (size_t)base + 32 * (size_t)k;
      a0 += partial[3 * s];
      a1 += partial[3 * s + 1];
      a2 += partial[3 * s + 2];
    }
    gg[0] = a0; gg[1] = a1; gg[2] = a2;
  } else {
    float s3[3] = {0, 0, 0}, c3[3] = {0, 0, 0};
    for (int k = 0; k < n; ++k) {
      const size_t s = (size_t)base + 32 * (size_t)k;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float y = partial[3 * s + c] - c3[c], t = s3[c] + y;
        c3[c] = (t - s3[c]) - y;
        s3[c] = t;
      }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) gg[c] = (double)s3[c] - (double)c3[c];
  }
}

// The same sum in the precision form, its compensated total rounded to FP32.
// Eight slots' loads are issued before they are summed (in the same order), so
// each thread keeps 96 bytes in flight; the partials are read once, so the
// loads are marked evict-first. 839 -> 827 us per 256-vesicle step.
__device__ __forceinline__ void vertex_gradient_f32(const float *__restrict__ partial, const int *__restrict__ loc,
                                                    int v, float g[3]) {
  const int base = loc[2 * (size_t)v], n = loc[2 * (size_t)v + 1];
  float s3[3] = {0, 0, 0}, c3[3] = {0, 0, 0};
  auto add = [&](int c, float x) {
    const float y = x - c3[c], t = s3[c] + y;
    c3[c] = (t - s3[c]) - y;
    s3[c] = t;
  };
  int k = 0;
  for (; k + 8 <= n; k += 8) {
    float x[8][3];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const size_t s = (size_t)base + 32 * (size_t)(k + q);
#pragma unroll
      for (int c = 0; c < 3; ++c) x[q][c] = __ldcs(&partial[3 * s + c]);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q)
#pragma unroll
      for (int c = 0; c < 3; ++c) add(c, x[q][c]);
  }
  for (; k < n; ++k) {
    const size_t s = (size_t)base + 32 * (size_t)k;
#pragma unroll
    for (int c = 0; c < 3; ++c) add(c, __ldcs(&partial[3 * s + c]));
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) g[c] = s3[c] - c3[c];
}

template <typename T>
__global__ void gather_kernel(int nv, const T *__restrict__ partial, const int *__restrict__ off,
                              double *__restrict__ g) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
    double gg[3];
    vertex_gradient(partial, off, v, gg);
    g[3 * (size_t)v] += gg[0];
    g[3 * (size_t)v + 1] += gg[1];
    g[3 * (size_t)v + 2] += gg[2];
  }
}

// Three unit normals per vertex from two Philox draws (Box-Muller). The
// plain path transforms in FP64 (bit-for-bit the oracle's draws up to libm
// rounding); the precision form in FP32 from 24-bit uniforms.
__device__ __forceinline__ void normals3_f32(uint64_t seed, uint32_t stream, uint64_t step, int v, float n[3]) {
  philox_out o = philox4x32_10((uint32_t)v, (uint32_t)step, (uint32_t)(step >> 32), stream, (uint32_t)seed,
                               (uint32_t)(seed >> 32));
  const float k = 1.0f / 16777216.0f;
  float u1 = ((float)(o.v[0] >> 8) + 0.5f) * k, u2 = ((float)(o.v[1] >> 8) + 0.5f) * k;
  float u3 = ((float)(o.v[2] >> 8) + 0.5f) * k, u4 = ((float)(o.v[3] >> 8) + 0.5f) * k;
  float rad = sqrtf(-2.0f * logf(u1)), sn, cs;
  sincospif(2.0f * u2, &sn, &cs);
  n[0] = rad * cs;
  n[1] = rad * sn;
  n[2] = sqrtf(-2.0f * logf(u3)) * cospif(2.0f * u4);
}
__device__ __forceinline__ void normals3_f32(uint64_t seed, uint32_t stream, uint64_t step, int v, double n[3]) {
  float f[3];
  normals3_f32(seed, stream, step, v, f);
  n[0] = f[0];
  n[1] = f[1];
  n[2] = f[2];
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
// Every product and sum is rounded on its own (no fused multiply-add), in the
// reference's order of operations, so each kernel that uses it rounds alike.
__device__ __forceinline__ void kick(const StepArgs &a, const double n[3], double pp[3], const double gg[3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double q = pp[c];
    if (a.kind == 2) q = __dsub_rn(q, __dmul_rn(__dmul_rn(a.gamma, a.AK), q));  // friction
    const double half = __dmul_rn(__dmul_rn(-gg[c], a.AK), 0.5);                 // half kick
    q = __dadd_rn(q, half);
    if (a.kind == 1)
      q = __dadd_rn(q, __ddiv_rn(__dmul_rn(__dmul_rn(__ddiv_rn(1.0, a.gamma), a.sigma), n[c]), a.AK));
    else
      q = __dadd_rn(q, __dmul_rn(a.sigma, n[c]));
    q = __dadd_rn(q, half);
    pp[c] = q;
  }
}

// The vertex-local update of one step with identity mass: overdamped BD
// (r += -(D dt/kT) g + sqrt(2 D dt) xi), or the leapfrog kick followed by
// r += p AK (p reset for BD). Rounded as kick() is.
__device__ __forceinline__ void vertex_update(const StepArgs &a, const double gg[3], const double n[3], double rn[3],
                                              double pp[3]) {
  if (a.kind == 0) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
      rn[c] = __dadd_rn(rn[c], __dadd_rn(__dmul_rn(-a.mob_dt, gg[c]), __dmul_rn(a.sigma, n[c])));
    return;
  }
  kick(a, n, pp, gg);
#pragma unroll
  for (int c = 0; c < 3; ++c) rn[c] = __dadd_rn(rn[c], __dmul_rn(pp[c], a.AK));
}

// Step index of the current step: the run's first step plus the run index,
// which finish_kernel has already advanced past this step.
__device__ __forceinline__ uint64_t current_step(const uint64_t *cnt) { return cnt[0] + cnt[1] - 1; }

// The precision form's overdamped BD step of one vertex: the gradient total
// and the Box-Muller normals stay in FP32, and so does the increment
// -(D dt / kT) g + sqrt(2 D dt) xi (about 2^-23 relative, 1e-9 A at a 0.02 A
// step); it is added to the FP64 position, from which the FP32 copies are
// then taken. The FP64 work is the position and its copies only: 8 operations
// per coordinate instead of 14 on GB300's narrow FP64 pipe. Explicitly
// rounded, so every kernel that inlines it rounds alike.
__device__ __forceinline__ void bd_vertex_f32(const float *__restrict__ partial, const int *__restrict__ off, int v,
                                              const StepArgs &a, uint64_t st, double *__restrict__ r,
                                              float *__restrict__ rhi, float *__restrict__ rlo,
                                              const double *__restrict__ r0, float *__restrict__ dsp) {
  float g[3], n[3];
  vertex_gradient_f32(partial, off, v, g);
  normals3_f32(a.seed, a.stream, st, v, n);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const size_t i = 3 * (size_t)v + c;
    const float d = __fmaf_rn(-a.mob_dt_f, g[c], __fmul_rn(a.sigma_f, n[c]));
    const double x = __dadd_rn(r[i], (double)d);
    r[i] = x;
    if (rhi) store_f32_position(i, x, rhi, rlo, r0, dsp);
  }
}

// Gather fused with the vertex-local update (overdamped BD, or the leapfrog
// kinds with identity mass).
template <typename T>
__global__ void gather_step_kernel(int nv, const T *__restrict__ partial, const int *__restrict__ off, StepArgs a,
                                   const uint64_t *__restrict__ cnt, double *__restrict__ r, double *__restrict__ p,
                                   float *__restrict__ rhi, float *__restrict__ rlo, const double *__restrict__ r0,
                                   float *__restrict__ dsp, const int *__restrict__ status) {
  grid_dependency_wait();  // the partials and the status come from the face launches
  if (*status) return;
  const uint64_t st = current_step(cnt);
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
    if constexpr (sizeof(T) == 4) {
      if (a.kind == 0) {
        bd_vertex_f32((const float *)partial, off, v, a, st, r, rhi, rlo, r0, dsp);
        continue;
      }
    }
    double gg[3], n[3];
    vertex_gradient(partial, off, v, gg);
    if constexpr (sizeof(T) == 8) normals3(a.seed, a.stream, st, v, n);
    else normals3_f32(a.seed, a.stream, st, v, n);
    double rn[3] = {r[3 * (size_t)v], r[3 * (size_t)v + 1], r[3 * (size_t)v + 2]};
    double pp[3] = {0, 0, 0};
    if (a.kind != 0)
#pragma unroll
      for (int c = 0; c < 3; ++c) pp[c] = p[3 * (size_t)v + c];
    vertex_update(a, gg, n, rn, pp);
    if (a.kind != 0)
#pragma unroll
      for (int c = 0; c < 3; ++c) p[3 * (size_t)v + c] = (a.kind == 1) ? 0.0 : pp[c];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      r[3 * (size_t)v + c] = rn[c];
      if (rhi) store_f32_position(3 * (size_t)v + c, rn[c], rhi, rlo, r0, dsp);
    }
  }
}

__global__ void kick_kernel(int nv, StepArgs a, const uint64_t *__restrict__ cnt, double *__restrict__ p,
                            const double *__restrict__ g, const int *__restrict__ status) {
  grid_dependency_wait();
  if (*status) return;
  const uint64_t st = current_step(cnt);
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
                             const double *__restrict__ qdot, float *__restrict__ rhi, float *__restrict__ rlo,
                             const double *__restrict__ r0, float *__restrict__ dsp, const int *__restrict__ status) {
  grid_dependency_wait();
  if (*status) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * nv; i += gridDim.x * blockDim.x) {
    const double x = __dadd_rn(r[i], __dmul_rn(qdot[i], a.AK));
    r[i] = x;
    if (a.kind == 1) p[i] = 0.0;
    if (rhi) store_f32_position(i, x, rhi, rlo, r0, dsp);
  }
}

// ---------------------------------------------------------------- batches
//
// Many meshes advance together. A tile is a run of up to tile_faces faces of
// one patch type of one mesh (tiles never straddle meshes); a block takes
// tiles in turn and sums each tile's energy terms in a fixed order, and each
// mesh sums its own tiles in listed order. Every mesh keeps its own state,
// noise stream, step counter and step limit, so a mesh's trajectory does not
// depend on what else is in the batch. Tile and job counts are read from
// device memory, so a captured step stays valid when the membership changes.

// A job takes the step when it has neither stopped nor reached its limit.
__device__ __forceinline__ bool job_active(const BatchFaceJob &J) { return !*J.status && J.cnt[1] < J.limit; }

template <typename T, int NCP, int NPT>
__global__ void __launch_bounds__(FaceCfg<T>::threads, FaceCfg<T>::min_blocks)
    batch_face_kernel(const BatchJob *__restrict__ jobs, int group, const BatchTile *__restrict__ tiles,
                      const int *__restrict__ counts, const double *__restrict__ basis,
                      const double *__restrict__ weight, double dudv_d, int irregular,
                      double *__restrict__ tile_sums) {
  using S = FaceSmem<T, NCP, NPT>;
  constexpr int HW = S::HW, NT = FaceCfg<T>::threads;
  __shared__ S sm;
  __shared__ BatchFaceJob sj;
  __shared__ int s_active;
  const int ntiles = counts[group], tile_base = counts[3 + group];
  if ((int)blockIdx.x >= ntiles) return;
  stage_basis<T, NCP, NPT, NT>(sm, basis, weight);
  const int hw = threadIdx.x >> 4, lane = threadIdx.x & 15;
  const unsigned hmask = (threadIdx.x & 16) ? 0xFFFF0000u : 0x0000FFFFu;
  const T dudv = (T)dudv_d;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const BatchTile tile = tiles[tile_base + t];
    __syncthreads();  // the previous tile's readers of sj and sm.red are done
    {
      const int *src = reinterpret_cast<const int *>(&jobs[tile.job].f);
      int *dst = reinterpret_cast<int *>(&sj);
      for (int i = threadIdx.x; i < (int)(sizeof(BatchFaceJob) / sizeof(int)); i += NT) dst[i] = src[i];
    }
    __syncthreads();
    if (threadIdx.x == 0) s_active = job_active(sj);  // one read for the whole block
    __syncthreads();
    HalfWarpSums<T> acc;
    if (s_active) {
      const FaceSrc &src = sj.src[group];
      const SurfaceParams &P = sj.P;
      const double *r = src.r;
      const T alpha[3] = {(T)r[3 * P.nv], (T)r[3 * P.nv + 1], (T)r[3 * P.nv + 2]};
      const T ialpha[3] = {T(1) / alpha[0], T(1) / alpha[1], T(1) / alpha[2]};
      const T am1[3] = {(T)(r[3 * P.nv] - 1.0), (T)(r[3 * P.nv + 1] - 1.0), (T)(r[3 * P.nv + 2] - 1.0)};
      const bool reg_alpha = irregular && P.k_reg != 0.0;
      const Moduli<T> mod(P);
      const int end = tile.first + tile.count;
      int f = tile.first + hw;
      FaceAhead<T> cur, nxt;
      uint32_t cp_next = load_cp<NCP>(src, f + HW, end, lane);
      load_ahead<T, NCP, NPT>(src, P, f, end, load_cp<NCP>(src, f, end, lane), lane, cur);
      for (; f < end; f += HW) {
        const uint32_t cp_after = load_cp<NCP>(src, f + 2 * HW, end, lane);
        load_ahead<T, NCP, NPT>(src, P, f + HW, end, cp_next, lane, nxt);
        cp_next = cp_after;
        T e3[3], da[3];
        face_compute<T, NCP, NPT>(sm, hw, lane, hmask, cur, P, alpha, ialpha, am1, mod, dudv, reg_alpha,
                                  (T *)sj.partial, e3, da);
        acc.add(0, e3[0]); acc.add(1, e3[1]); acc.add(2, e3[2]);
        cur = nxt;
        __syncwarp(hmask);
      }
    }
    if (lane == 0)
#pragma unroll
      for (int q = 0; q < 3; ++q) sm.red[hw][q] = acc.get(q);
    __syncthreads();
    if (threadIdx.x < 3) {
      double s = 0;
#pragma unroll
      for (int h = 0; h < HW; ++h) s += sm.red[h][threadIdx.x];
      tile_sums[3 * (size_t)(tile_base + t) + threadIdx.x] = s;
    }
  }
}

// ---------------------------------------------------------------- thread-per-face pass
//
// Regular faces of the precision form (12 control points, 15 quadrature
// points), one face per thread. The thread keeps its face's centred control
// points X[12][3] (and their displacements from the reference state) in its
// own columns of shared memory, its gradient sums G[12][3] in registers, and
// walks the 15 points; every thread of a warp reads the same basis row at the
// same time, so the basis comes out of shared memory as broadcasts (one
// wavefront per float4) and both contractions are plain multiply-adds:
//   K[k]_c = sum_j B[p][k][j] X[j]_c          (Ru, Rv, Suu, Suv, Svv)
//   G[j]_c += B[p][u][j] Kb[u]_c + B[p][v][j] Kb[v]_c + s[j] m_c,
//   s[j] = B[p][uu][j] lb + B[p][uv][j] kb + B[p][vv][j] nb
// (the adjoints of Suu, Suv, Svv are lb m, kb m, nb m: one scalar per control
// point times the normal instead of three vector rows). Nothing is shuffled
// or transposed per face. Energy terms and dE/dalpha are Kahan-summed per
// thread over its faces and reduced once at the end, in a fixed order.
namespace tpf {
constexpr int kNcp = 12, kNpt = 15, kNc4 = 3;
constexpr int kThreads = 128, kWarps = kThreads / 32, kMinBlocks = 3;
struct Smem {
  Q4<float> B[kNpt][5][kNc4];  // basis rows u, v, uu, uv, vv of point p, control points in fours
  // each thread's centred control points, coordinate-major: float4 3 c + q
  // holds coordinate c of control points 4 q .. 4 q + 3; the 144-byte stride
  // is an odd number of 16-byte chunks, so the float4 reads of a warp do not
  // conflict
  float4 X[kThreads][9];
  float4 D[kThreads][9];  // the same control points' change from the reference state, same layout
  float W[kNpt];
  double red[kWarps][6];
};
constexpr size_t kSumBytes = sizeof(float) * 12 * kThreads;  // per-thread Kahan totals (dynamic shared memory)
// Thread-private float4 in shared memory, stored and loaded through volatile
// asm so the compiler re-reads it instead of keeping the stored registers
// alive across the point loop (which is the register pressure this layout
// exists to avoid).
__device__ __forceinline__ void st4(float4 *p, float4 v) {
  asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"((uint32_t)__cvta_generic_to_shared(p)), "f"(v.x),
               "f"(v.y), "f"(v.z), "f"(v.w));
}
__device__ __forceinline__ float4 ld4(const float4 *p) {
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"((uint32_t)__cvta_generic_to_shared(p)));
  return v;
}
__device__ __forceinline__ void prefetch_l1(const void *p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }
// Point of the face loop at which the thread prefetches its next face's table
// rows (control points, g0, composition, slot destinations) into L1. Those
// rows are otherwise first touched when the next face starts (control points,
// composition) or point by point (g0), each a round trip to L2.
constexpr int kPrefetchPoint = 10;
}  // namespace tpf

__device__ __forceinline__ void tpf_stage(tpf::Smem &sm, const double *basis, const double *weight) {
  float *b = &sm.B[0][0][0].x;
  for (int i = threadIdx.x; i < tpf::kNpt * 5 * tpf::kNc4 * 4; i += blockDim.x) b[i] = (float)basis[i];
  for (int i = threadIdx.x; i < tpf::kNpt; i += blockDim.x) sm.W[i] = (float)weight[i];
}

// Face f's energy terms and dE/dalpha; writes its alpha-scaled gradient
// partials to the face's slots. vec: cp and dest are 16-byte aligned.
// am1 = alpha - 1 (formed in FP64): the box scales' part of the change from
// the reference state. fn: the face this thread takes next (its rows are
// prefetched), or -1.
template <bool KG_REG>
__device__ __forceinline__ void tpf_face(tpf::Smem &sm, const FaceSrc &S, const SurfaceParams &P, int f,
                                         const float alpha[3], const float ialpha[3], const float am1[3],
                                         const Moduli<float> &mod, float dudv, bool vec, float *__restrict__ partial,
                                         float e3[3], float da[3], int fn) {
  using namespace tpf;
  uint32_t cp[kNcp];
  if (vec) {
    const uint4 *q = reinterpret_cast<const uint4 *>(S.cp + (size_t)f * kNcp);
#pragma unroll
    for (int i = 0; i < kNc4; ++i) {
      const uint4 v = __ldg(q + i);
      cp[4 * i] = v.x; cp[4 * i + 1] = v.y; cp[4 * i + 2] = v.z; cp[4 * i + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int j = 0; j < kNcp; ++j) cp[j] = __ldg(&S.cp[(size_t)f * kNcp + j]);
  }
  const float P2 = __ldg(&S.compf[3 * (size_t)f]), Hbar = __ldg(&S.compf[3 * (size_t)f + 1]),
              Pres = __ldg(&S.compf[3 * (size_t)f + 2]);
  // ---- control points relative to the patch corner (control point 0), in
  // their lattice images, times alpha; error-free sums on the hi/lo pairs as
  // in face_compute, so the local coordinates carry full FP32 precision. Their
  // change from the reference state: alpha L - L0 = (alpha - 1) L + (dsp -
  // dsp of the corner). Formed and stored four control points at a time.
  float4 *xs = sm.X[threadIdx.x], *ds = sm.D[threadIdx.x];
  float ahi[3], alo[3], ad[3];
  {
    const int v0 = (int)(cp[0] & kVertexMask);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      ahi[c] = __ldg(&S.rhi[3 * (size_t)v0 + c]);
      alo[c] = __ldg(&S.rlo[3 * (size_t)v0 + c]);
      ad[c] = __ldg(&S.dsp[3 * (size_t)v0 + c]);
    }
  }
#pragma unroll
  for (int c4 = 0; c4 < kNc4; ++c4) {
    float X[4][3], Dx[4][3];
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const int j = 4 * c4 + jj;
      const int v = (int)(cp[j] & kVertexMask), code = (int)(cp[j] >> kVertexBits);
      float hi[3], lo[3], dv[3], l[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        hi[c] = __ldg(&S.rhi[3 * (size_t)v + c]);
        lo[c] = __ldg(&S.rlo[3 * (size_t)v + c]);
        dv[c] = __ldg(&S.dsp[3 * (size_t)v + c]);
      }
      if (code == 13) {  // the home image (every control point of a closed vesicle)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float s2, e2;
          two_sum(hi[c], -ahi[c], s2, e2);
          l[c] = s2 + (e2 + (lo[c] - alo[c]));
        }
      } else {  // a periodic image: the lattice shift as hi + lo (each term exact)
        const int img[3] = {code % 3 - 1, (code / 3) % 3 - 1, code / 9 - 1};
        float sh[3] = {0.f, 0.f, 0.f}, she[3] = {0.f, 0.f, 0.f}, shl[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            float t, e;
            two_sum(sh[c], (float)img[d] * P.box_hi[d][c], t, e);
            sh[c] = t;
            she[c] += e;
            shl[c] += (float)img[d] * P.box_lo[d][c];
          }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float s1, e1, s2, e2;
          two_sum(hi[c], sh[c], s1, e1);
          two_sum(s1, -ahi[c], s2, e2);
          l[c] = s2 + ((e1 + e2) + ((lo[c] - alo[c]) + (she[c] + shl[c])));
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        X[jj][c] = alpha[c] * l[c];
        Dx[jj][c] = fmaf(am1[c], l[c], dv[c] - ad[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      st4(&xs[kNc4 * c + c4], make_float4(X[0][c], X[1][c], X[2][c], X[3][c]));
      st4(&ds[kNc4 * c + c4], make_float4(Dx[0][c], Dx[1][c], Dx[2][c], Dx[3][c]));
    }
  }
  // ---- the quadrature points
  float G[kNcp][3];  // gradient sums
#pragma unroll
  for (int j = 0; j < kNcp; ++j) G[j][0] = G[j][1] = G[j][2] = 0.f;
  float ea = 0.f, ec = 0.f, er = 0.f, dax = 0.f, day = 0.f, daz = 0.f;
#pragma unroll 1
  for (int p = 0; p < kNpt; ++p) {
    if (p == kPrefetchPoint && fn >= 0) {
      prefetch_l1(S.cp + (size_t)fn * kNcp);
      prefetch_l1(S.cp + (size_t)fn * kNcp + kNcp - 1);
      prefetch_l1(S.g0f + (size_t)fn * kNpt);
      prefetch_l1(S.g0f + (size_t)fn * kNpt + kNpt - 1);
      prefetch_l1(S.compf + (size_t)fn * 3);
      prefetch_l1(S.dest + (size_t)fn * kNcp);
      prefetch_l1(S.dest + (size_t)fn * kNcp + kNcp - 1);
    }
    const float g0 = __ldg(&S.g0f[(size_t)f * kNpt + p]);
    float rr0 = 0.f;
    if constexpr (KG_REG) rr0 = __ldg(&S.rr0f[(size_t)f * kNpt + p]);
    // K[k]_c as two partial sums (even, odd control points) in one pair; the
    // u and v rows also over the displacements (dR, the tangents' change
    // from the reference state)
    float2 A[5][3], Ad[2][3];
#pragma unroll
    for (int k = 0; k < 5; ++k) A[k][0] = A[k][1] = A[k][2] = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 2; ++k) Ad[k][0] = Ad[k][1] = Ad[k][2] = make_float2(0.f, 0.f);
#pragma unroll
    for (int c4 = 0; c4 < kNc4; ++c4) {
      float4 x[3], d[3];  // coordinate c of control points 4 c4 .. 4 c4 + 3
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        x[c] = ld4(&xs[kNc4 * c + c4]);
        d[c] = ld4(&ds[kNc4 * c + c4]);
      }
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        const Q4<float> b = sm.B[p][k][c4];
        const float2 b01 = make_float2(b.x, b.y), b23 = make_float2(b.z, b.w);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          A[k][c] = __ffma2_rn(b01, make_float2(x[c].x, x[c].y), A[k][c]);
          A[k][c] = __ffma2_rn(b23, make_float2(x[c].z, x[c].w), A[k][c]);
          if (k < 2) {
            Ad[k][c] = __ffma2_rn(b01, make_float2(d[c].x, d[c].y), Ad[k][c]);
            Ad[k][c] = __ffma2_rn(b23, make_float2(d[c].z, d[c].w), Ad[k][c]);
          }
        }
      }
    }
    Vec3<float> K[5], dR[2];
#pragma unroll
    for (int k = 0; k < 5; ++k) K[k] = {A[k][0].x + A[k][0].y, A[k][1].x + A[k][1].y, A[k][2].x + A[k][2].y};
#pragma unroll
    for (int k = 0; k < 2; ++k) dR[k] = {Ad[k][0].x + Ad[k][0].y, Ad[k][1].x + Ad[k][1].y, Ad[k][2].x + Ad[k][2].y};
    Vec3<float> Kb[5], Kreg[2], m;
    float a, c, r, lkn[3];
    point_adjoint<float, KG_REG>(K, sm.W[p], g0, rr0, dudv, P2, Hbar, Pres, mod.kc, mod.KA, mod.kg, mod.k_reg, &a,
                                 &c, &r, Kb, Kreg, dR, lkn, &m);
    ea += a;
    ec += c;
    er += r;
    // alpha_c dE/dalpha_c over this point: sum_k Kb[k]_c K[k]_c, with Kb[2..4] = (lb, kb, nb) m
    {
      const float t[3] = {lkn[0] * K[2].x + lkn[1] * K[3].x + lkn[2] * K[4].x,
                          lkn[0] * K[2].y + lkn[1] * K[3].y + lkn[2] * K[4].y,
                          lkn[0] * K[2].z + lkn[1] * K[3].z + lkn[2] * K[4].z};
      dax = fmaf(Kb[0].x, K[0].x, fmaf(Kb[1].x, K[1].x, fmaf(m.x, t[0], dax)));
      day = fmaf(Kb[0].y, K[0].y, fmaf(Kb[1].y, K[1].y, fmaf(m.y, t[1], day)));
      daz = fmaf(Kb[0].z, K[0].z, fmaf(Kb[1].z, K[1].z, fmaf(m.z, t[2], daz)));
    }
    // G[j]_c += B[u][j] Kb[u]_c + B[v][j] Kb[v]_c + s[j] m_c in scalar multiply-adds: with the
    // forward contraction in paired ones, the mix keeps both FP32 multiply-add pipes busy
    // (all paired: 763 us, this mix: 747 us, all scalar: 776 us on the 256-vesicle pass)
    {
      const float ku[3] = {Kb[0].x, Kb[0].y, Kb[0].z}, kv[3] = {Kb[1].x, Kb[1].y, Kb[1].z}, md[3] = {m.x, m.y, m.z};
#pragma unroll
      for (int c4 = 0; c4 < kNc4; ++c4) {
        const Q4<float> bu = sm.B[p][0][c4], bv = sm.B[p][1][c4], buu = sm.B[p][2][c4], buv = sm.B[p][3][c4],
                        bvv = sm.B[p][4][c4];
        const float u[4] = {bu.x, bu.y, bu.z, bu.w}, v[4] = {bv.x, bv.y, bv.z, bv.w};
        const float uu[4] = {buu.x, buu.y, buu.z, buu.w}, uv[4] = {buv.x, buv.y, buv.z, buv.w},
                    vv[4] = {bvv.x, bvv.y, bvv.z, bvv.w};
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          const float sj = fmaf(vv[jj], lkn[2], fmaf(uv[jj], lkn[1], uu[jj] * lkn[0]));
          float *g = G[4 * c4 + jj];
#pragma unroll
          for (int cc = 0; cc < 3; ++cc) g[cc] = fmaf(sj, md[cc], fmaf(v[jj], kv[cc], fmaf(u[jj], ku[cc], g[cc])));
        }
      }
    }
  }
  // ---- dE/dalpha_c: K is linear in the alpha-scaled coordinates, so
  // alpha_c dE/dalpha_c = sum over points and k of Kb[k]_c K[k]_c
  da[0] = dax * ialpha[0]; da[1] = day * ialpha[1]; da[2] = daz * ialpha[2];
  int d[kNcp];
  if (vec) {
    const int4 *q = reinterpret_cast<const int4 *>(S.dest + (size_t)f * kNcp);
#pragma unroll
    for (int i = 0; i < kNc4; ++i) {
      const int4 v = __ldg(q + i);
      d[4 * i] = v.x; d[4 * i + 1] = v.y; d[4 * i + 2] = v.z; d[4 * i + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int j = 0; j < kNcp; ++j) d[j] = __ldg(&S.dest[(size_t)f * kNcp + j]);
  }
#pragma unroll
  for (int j = 0; j < kNcp; ++j) {
    float *o = partial + 3 * (size_t)d[j];
#pragma unroll
    for (int c = 0; c < 3; ++c) o[c] = alpha[c] * G[j][c];
  }
  e3[0] = ea; e3[1] = ec; e3[2] = er;
}

__device__ __forceinline__ bool tpf_vec(const FaceSrc &S) {
  return ((reinterpret_cast<uintptr_t>(S.cp) | reinterpret_cast<uintptr_t>(S.dest)) & 15) == 0;
}

// Kahan-compensated FP32 totals of one thread, kept in shared memory (its
// column of s[12][kThreads]) rather than in registers, which the face loop
// needs for itself.
struct SharedSums {
  float *s;
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int q = 0; q < 12; ++q) s[q * tpf::kThreads] = 0.f;
  }
  __device__ __forceinline__ void add(int q, float v) {
    float sum = s[2 * q * tpf::kThreads], c = s[(2 * q + 1) * tpf::kThreads];
    const float y = v - c, t = sum + y;
    s[(2 * q + 1) * tpf::kThreads] = (t - sum) - y;
    s[2 * q * tpf::kThreads] = t;
  }
  __device__ __forceinline__ double get(int q) const {
    return (double)s[2 * q * tpf::kThreads] - (double)s[(2 * q + 1) * tpf::kThreads];
  }
};

// Sum of q over the warp in a fixed (xor-tree) order.
__device__ __forceinline__ double warp_sum(double q) {
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) q += __shfl_xor_sync(0xFFFFFFFFu, q, off);
  return q;
}

// Single mesh, regular faces, precision form: persistent grid, warp w of the
// grid takes faces 32 w .. 32 w + 31, then 32 (w + warps in the grid) ...
// Writes one block partial of the energy terms and dE/dalpha; the last block
// to finish sums them (as face_kernel does).
__global__ void __launch_bounds__(tpf::kThreads, tpf::kMinBlocks)
    face_tpf_kernel(FaceLaunch L, const int *__restrict__ dest, SurfaceParams P, const double *__restrict__ r,
                    const float *__restrict__ rhi, const float *__restrict__ rlo, const float *__restrict__ dsp,
                    float *__restrict__ partial, double *__restrict__ blockpart, int *__restrict__ status,
                    FinishArgs fin) {
  using namespace tpf;
  __shared__ Smem sm;
  extern __shared__ __align__(16) unsigned char tpf_dyn[];
  tpf_stage(sm, L.basis, L.weight);
  __syncthreads();
  grid_dependency_wait();  // the state comes from the kernels before
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float alpha[3] = {(float)r[3 * P.nv], (float)r[3 * P.nv + 1], (float)r[3 * P.nv + 2]};
  const float ialpha[3] = {1.f / alpha[0], 1.f / alpha[1], 1.f / alpha[2]};
  const float am1[3] = {(float)(r[3 * P.nv] - 1.0), (float)(r[3 * P.nv + 1] - 1.0), (float)(r[3 * P.nv + 2] - 1.0)};
  const Moduli<float> mod(P);
  const FaceSrc src{L.cp, L.g0, L.rr0, L.comp, L.g0f, L.rr0f, L.compf, dest, r, rhi, rlo, dsp, L.nfaces};
  const bool vec = tpf_vec(src);
  const float dudv = (float)L.dudv;
  const bool kg_reg = P.kg != 0.0 || P.k_reg != 0.0;  // else the pointwise step leaves those terms out
  const int n = L.nfaces, stride = gridDim.x * kThreads;
  SharedSums acc{reinterpret_cast<float *>(tpf_dyn) + threadIdx.x};
  acc.zero();
  for (int fb = (blockIdx.x * kWarps + warp) * 32; fb < n; fb += stride) {
    const int f = fb + lane;
    if (f < n) {
      float e3[3], da[3];
      // no prefetch: a thread's next face is a grid stride away, and on the
      // 512 x 512 planar pass the prefetch cost 1% instead of gaining
      if (kg_reg) tpf_face<true>(sm, src, P, f, alpha, ialpha, am1, mod, dudv, vec, partial, e3, da, -1);
      else tpf_face<false>(sm, src, P, f, alpha, ialpha, am1, mod, dudv, vec, partial, e3, da, -1);
      acc.add(0, e3[0]); acc.add(1, e3[1]); acc.add(2, e3[2]);
      acc.add(3, da[0]); acc.add(4, da[1]); acc.add(5, da[2]);
      if (!isfinite(e3[0] + e3[1] + e3[2])) atomicOr(status, kStatusNonFinite);
    }
  }
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    const double s = warp_sum(acc.get(q));
    if (lane == 0) sm.red[warp][q] = s;
  }
  __syncthreads();  // every thread has read its sums: the finish may reuse their space
  if (threadIdx.x < 6) {
    double s = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) s += sm.red[w][threadIdx.x];
    blockpart[6 * (size_t)(L.block_base + blockIdx.x) + threadIdx.x] = s;
  }
  if (fin.done) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(fin.done, 1u) == (unsigned)fin.nblk - 1u);
    __syncthreads();
    if (last) {
      __threadfence();
      static_assert(kSumBytes >= sizeof(double) * 6 * kThreads, "finish scratch must fit in the sums' space");
      finish_sums<kThreads>(fin, blockpart, reinterpret_cast<double(*)[kThreads]>(tpf_dyn));
      if (threadIdx.x == 0) *fin.done = 0u;
    }
  }
}

// Batched regular faces, precision form: a block takes a tile (faces of one
// job), its warps 32 faces at a time; writes the tile's three energy sums.
// counter[0] hands out the tiles; counter[1] counts the blocks that are done,
// and the last of them zeroes both for the next launch. A block draws its next
// tile while it works on the current one (the draw's round trip hides behind
// the faces), and copies a job's header only when the tile's job changes.
__global__ void __launch_bounds__(tpf::kThreads, tpf::kMinBlocks)
    batch_face_tpf_kernel(const BatchJob *__restrict__ jobs, int group, const BatchTile *__restrict__ tiles,
                          const int *__restrict__ counts, const double *__restrict__ basis,
                          const double *__restrict__ weight, double dudv_d, double *__restrict__ tile_sums,
                          int *__restrict__ counter) {
  using namespace tpf;
  __shared__ Smem sm;
  __shared__ BatchFaceJob sj;
  __shared__ int s_active, s_tile[2];
  tpf_stage(sm, basis, weight);  // constant tables: before the wait
  grid_dependency_wait();        // positions, job states and the counter come from the kernels before
  const int ntiles = counts[group], tile_base = counts[3 + group];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float dudv = (float)dudv_d;
  // Tiles are handed out by a counter (zeroed before the launch), so blocks
  // that draw cheap tiles take more; each tile's sums go to its own row, so
  // the results do not depend on which block took which tile. Draw k is read
  // from s_tile[k & 1] after the barrier that opens iteration k and written
  // during iteration k - 1, after that iteration's own barrier: its readers
  // of the same slot (iteration k - 2) are done by then.
  if (threadIdx.x == 0) s_tile[0] = (int)blockIdx.x < ntiles ? atomicAdd(&counter[0], 1) : ntiles;
  int job = -1;
  for (int k = 0;; ++k) {
    __syncthreads();  // the previous tile's readers of sj, s_active and sm.red are done; draw k is visible
    const int t = s_tile[k & 1];
    if (t >= ntiles) break;
    const BatchTile tile = tiles[tile_base + t];
    if (tile.job != job) {  // the same for every thread of the block
      const int *src = reinterpret_cast<const int *>(&jobs[tile.job].f);
      int *dst = reinterpret_cast<int *>(&sj);
      for (int i = threadIdx.x; i < (int)(sizeof(BatchFaceJob) / sizeof(int)); i += kThreads) dst[i] = src[i];
      if (threadIdx.x == 0) s_active = job_active(jobs[tile.job].f);
      job = tile.job;
      __syncthreads();
    }
    if (threadIdx.x == 0) s_tile[(k + 1) & 1] = atomicAdd(&counter[0], 1);
    HalfWarpSums<float> acc;
    if (s_active) {
      const FaceSrc &src = sj.src[group];
      const SurfaceParams &P = sj.P;
      const double *r = src.r;
      const float alpha[3] = {(float)r[3 * P.nv], (float)r[3 * P.nv + 1], (float)r[3 * P.nv + 2]};
      const float ialpha[3] = {1.f / alpha[0], 1.f / alpha[1], 1.f / alpha[2]};
      const float am1[3] = {(float)(r[3 * P.nv] - 1.0), (float)(r[3 * P.nv + 1] - 1.0),
                            (float)(r[3 * P.nv + 2] - 1.0)};
      const Moduli<float> mod(P);
      const int end = tile.first + tile.count;
      float *partial = (float *)sj.partial;
      const bool kg_reg = P.kg != 0.0 || P.k_reg != 0.0;  // else the pointwise step leaves those terms out
      const bool vec = tpf_vec(src);
      for (int fb = tile.first + warp * 32; fb < end; fb += kThreads) {
        const int f = fb + lane;
        if (f < end) {
          float e3[3], da[3];
          const int fn = f + kThreads < end ? f + kThreads : -1;
          if (kg_reg) tpf_face<true>(sm, src, P, f, alpha, ialpha, am1, mod, dudv, vec, partial, e3, da, fn);
          else tpf_face<false>(sm, src, P, f, alpha, ialpha, am1, mod, dudv, vec, partial, e3, da, fn);
          acc.add(0, e3[0]); acc.add(1, e3[1]); acc.add(2, e3[2]);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const double s = warp_sum(acc.get(q));
      if (lane == 0) sm.red[warp][q] = s;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
      double s = 0;
#pragma unroll
      for (int w = 0; w < kWarps; ++w) s += sm.red[w][threadIdx.x];
      tile_sums[3 * (size_t)(tile_base + t) + threadIdx.x] = s;
    }
  }
  __threadfence();  // this block's last draw on counter[0] is ordered before its count on counter[1]
  if (threadIdx.x == 0 && atomicAdd(&counter[1], 1) == (int)gridDim.x - 1) {
    counter[0] = 0;  // every block has drawn its last tile: reset for the next launch
    counter[1] = 0;
  }
}

// Per job (one warp each): sum its tiles in listed order, record the step's
// energy in the job's run, flag non-finite or diverging energies (src/hd.C:
// 1280-1305) for that job only, advance its run index. live[j] tells the
// update whether job j took this step; prog[j] = {steps done, status}.
__global__ void batch_reduce_kernel(const BatchJob *__restrict__ jobs, const int *__restrict__ counts,
                                    const int *__restrict__ tile_off, const int *__restrict__ tile_idx,
                                    const double *__restrict__ tile_sums, int *__restrict__ live,
                                    unsigned long long *__restrict__ prog) {
  grid_dependency_wait();
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (j >= counts[6]) return;
  const BatchJob &J = jobs[j];
  const bool active = job_active(J.f);  // uniform over the warp: nothing below changes it before the sync
  __syncwarp();
  double a[3] = {0, 0, 0};
  if (active)
    for (int k = tile_off[j] + lane; k < tile_off[j + 1]; k += 32)
#pragma unroll
      for (int q = 0; q < 3; ++q) a[q] += tile_sums[3 * (size_t)tile_idx[k] + q];
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1)
#pragma unroll
    for (int q = 0; q < 3; ++q) a[q] += __shfl_xor_sync(0xffffffffu, a[q], off);
  if (lane != 0) return;
  int st = *J.f.status;
  uint64_t done = J.f.cnt[1];
  if (active) {
    const double e = a[0] + a[1] + a[2];
    J.E[0] = e;
    J.parts[0] = a[0]; J.parts[1] = a[1]; J.parts[2] = a[2];
    if (!isfinite(e)) st |= kStatusNonFinite;
    if (J.energies) {
      J.energies[done] = e;
      if (J.threshold > 0 && done > 0 && e - J.energies[done - 1] > J.threshold) st |= kStatusDiverged;
    }
    *J.f.status = st;
    // As in a single-mesh run, the step whose energy is flagged does not move.
    J.f.cnt[1] = ++done;
  }
  live[j] = active && !st;
  prog[2 * j] = done;
  prog[2 * j + 1] = (unsigned long long)st;
}

// Gather fused with each live job's vertex-local update (overdamped BD, or the
// leapfrog kinds with identity mass), with the job's own integrator settings.
template <typename T>
__global__ void batch_gather_step_kernel(const BatchJob *__restrict__ jobs, const BatchTile *__restrict__ vtiles,
                                         const int *__restrict__ counts, const int *__restrict__ live) {
  grid_dependency_wait();
  const int nvtiles = counts[7];
  for (int t = blockIdx.x; t < nvtiles; t += gridDim.x) {
    const BatchTile tile = vtiles[t];
    if (!live[tile.job] || (int)threadIdx.x >= tile.count) continue;
    const BatchJob &J = jobs[tile.job];
    const StepArgs &a = J.a;
    const int v = tile.first + threadIdx.x;
    const uint64_t st = J.f.cnt[0] + J.f.cnt[1] - 1;
    if constexpr (sizeof(T) == 4) {
      if (a.kind == 0) {
        bd_vertex_f32((const float *)J.f.partial, J.off, v, a, st, J.r, J.rhi, J.rlo, J.r0, J.dsp);
        continue;
      }
    }
    double gg[3], n[3];
    vertex_gradient((const T *)J.f.partial, J.off, v, gg);
    if constexpr (sizeof(T) == 8) normals3(a.seed, a.stream, st, v, n);
    else normals3_f32(a.seed, a.stream, st, v, n);
    double *r = J.r, *p = J.p;
    double rn[3] = {r[3 * (size_t)v], r[3 * (size_t)v + 1], r[3 * (size_t)v + 2]};
    double pp[3] = {0, 0, 0};
    if (a.kind != 0)
#pragma unroll
      for (int c = 0; c < 3; ++c) pp[c] = p[3 * (size_t)v + c];
    vertex_update(a, gg, n, rn, pp);
    if (a.kind != 0)
#pragma unroll
      for (int c = 0; c < 3; ++c) p[3 * (size_t)v + c] = (a.kind == 1) ? 0.0 : pp[c];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      r[3 * (size_t)v + c] = rn[c];
      if (J.rhi) store_f32_position(3 * (size_t)v + c, rn[c], J.rhi, J.rlo, J.r0, J.dsp);
    }
  }
}

// Start of the runs of the jobs flagged in start[]: counters {step0, 0},
// status cleared, FP32 hi/lo pairs of the positions (precision form).
__global__ void batch_start_kernel(const BatchJob *__restrict__ jobs, const BatchTile *__restrict__ vtiles,
                                   const int *__restrict__ counts, const int *__restrict__ start,
                                   const unsigned long long *__restrict__ step0) {
  const int nvtiles = counts[7];
  for (int t = blockIdx.x; t < nvtiles; t += gridDim.x) {
    const BatchTile tile = vtiles[t];
    if (!start[tile.job]) continue;
    const BatchJob &J = jobs[tile.job];
    if (tile.first == 0 && threadIdx.x == 0) {
      J.f.cnt[0] = step0[tile.job];
      J.f.cnt[1] = 0;
      *J.f.status = 0;
    }
    if (J.rhi && (int)threadIdx.x < tile.count) {
      const int v = tile.first + threadIdx.x;
      for (int c = 0; c < 3; ++c)
        store_f32_position(3 * (size_t)v + c, J.r[3 * (size_t)v + c], J.rhi, J.rlo, J.r0, J.dsp);
    }
  }
}

// Host-driven batch steps: every job's state (3 nv + 3 doubles: positions,
// then the box scales) packed in job order at pack[off[j] ..]. In: into each
// job's resident state and the precision form's FP32 copies. Out: back into
// the pack, and each job's latest energy into E[j].
__global__ void batch_unpack_kernel(const BatchJob *__restrict__ jobs, const BatchTile *__restrict__ vtiles,
                                    const int *__restrict__ counts, const long long *__restrict__ off,
                                    const double *__restrict__ pack) {
  const int nvtiles = counts[7];
  for (int t = blockIdx.x; t < nvtiles; t += gridDim.x) {
    const BatchTile tile = vtiles[t];
    const BatchJob &J = jobs[tile.job];
    const double *src = pack + off[tile.job];
    if ((int)threadIdx.x < tile.count) {
      const size_t v = (size_t)(tile.first + threadIdx.x);
      for (int c = 0; c < 3; ++c) {
        const double x = src[3 * v + c];
        // a coordinate the caller left as it was keeps its FP32 copies (compared
        // bit for bit, on the integer pipe): most of the unpacking's FP64 work
        if (__double_as_longlong(x) == __double_as_longlong(J.r[3 * v + c])) continue;
        J.r[3 * v + c] = x;
        if (J.rhi) store_f32_position(3 * v + c, x, J.rhi, J.rlo, J.r0, J.dsp);
      }
    }
    if (tile.first == 0 && threadIdx.x < 3) {
      const size_t a = 3 * (size_t)J.f.P.nv + threadIdx.x;
      J.r[a] = src[a];
    }
  }
}

__global__ void batch_pack_kernel(const BatchJob *__restrict__ jobs, const BatchTile *__restrict__ vtiles,
                                  const int *__restrict__ counts, const long long *__restrict__ off,
                                  double *__restrict__ pack, double *__restrict__ E) {
  const int nvtiles = counts[7];
  for (int t = blockIdx.x; t < nvtiles; t += gridDim.x) {
    const BatchTile tile = vtiles[t];
    const BatchJob &J = jobs[tile.job];
    double *dst = pack + off[tile.job];
    if ((int)threadIdx.x < tile.count) {
      const size_t v = (size_t)(tile.first + threadIdx.x);
      for (int c = 0; c < 3; ++c) dst[3 * v + c] = J.r[3 * v + c];
    }
    if (tile.first == 0 && threadIdx.x < 3) {
      const size_t a = 3 * (size_t)J.f.P.nv + threadIdx.x;
      dst[a] = J.r[a];
    }
    if (tile.first == 0 && threadIdx.x == 3) E[tile.job] = *J.E;
  }
}

// ---------------------------------------------------------------- area, volume
//
// One half-warp per face, as in the face pass: lanes are control points while
// the face's local coordinates are formed, then quadrature points. The value
// and first-derivative basis rows of every patch type sit in shared memory.
//
// Precision. The restraint on V is stiff (K_V (V - V0) is a force per unit
// volume), so V must be exact far below an FP32 ulp of V: on a 1000 A vesicle
// a 1e-3 A^3 error already moves every vertex's restraint force by about
// K_V 1e-3 A^3 x 300 A^2. The sums kernel therefore forms R, R_u, R_v and
// R.(R_u x R_v) in FP64 from FP64 local coordinates (relative to the patch
// corner, which is added back exactly). The area, whose restraint is soft, and
// the box-scale derivatives come from FP32 copies in the precision form. The
// gradient kernel needs only the relative accuracy of any other gradient term
// and runs in the form's own arithmetic (FP32 local coordinates from the hi/lo
// pairs, as the face pass forms them).

constexpr int kGeoHW = kGeoThreads / 16;  // faces in flight per block
constexpr int kGeoPt = 16;                // quadrature points of the largest rule

template <typename T>
struct GeoBasis {
  T B[3][kGeoPt][3][kMaxCpDev];  // [group][point][w, u, v][control point]
  T cw[3][kGeoPt];               // dudv * weight
};

template <typename T>
__device__ void stage_geo_basis(const GeoArgs &G, GeoBasis<T> &s) {
  for (int gi = 0; gi < G.ngroups; ++gi) {
    const GeoGroup &g = G.g[gi];
    for (int i = threadIdx.x; i < g.npt * g.ncp; i += blockDim.x) {
      const int p = i / g.ncp, x = i % g.ncp;
      s.B[gi][p][0][x] = (T)g.basis_w[(size_t)p * g.ncp + x];
      s.B[gi][p][1][x] = (T)g.basis[(size_t)p * 5 * g.ncpp + x];
      s.B[gi][p][2][x] = (T)g.basis[(size_t)p * 5 * g.ncpp + g.ncpp + x];
    }
    for (int p = threadIdx.x; p < g.npt; p += blockDim.x) s.cw[gi][p] = (T)(g.dudv * g.weight[p]);
  }
}

// Group of global face f (faces are numbered group after group).
__device__ __forceinline__ int geo_group(const GeoArgs &G, int f, int *local) {
  int k = 0;
  while (k + 1 < G.ngroups && f >= G.g[k + 1].face_base) ++k;
  *local = f - G.g[k].face_base;
  return k;
}

// Absolute (alpha-scaled, lattice-image) FP64 position of control point `lane` of face lf.
__device__ __forceinline__ void geo_abs64(const GeoArgs &G, const GeoGroup &g, int lf, int lane,
                                          const double alpha[3], double X[3], int *dest) {
  const uint32_t packed = __ldg(&g.cp[(size_t)lf * g.ncp + lane]);
  const int v = (int)(packed & kVertexMask), code = (int)(packed >> kVertexBits);
  const int im[3] = {code % 3 - 1, (code / 3) % 3 - 1, code / 9 - 1};
#pragma unroll
  for (int c = 0; c < 3; ++c)
    X[c] = alpha[c] * (G.r[3 * (size_t)v + c] + im[0] * G.box[0][c] + im[1] * G.box[1][c] + im[2] * G.box[2][c]);
  if (dest) *dest = __ldg(&g.dest[(size_t)lf * g.ncp + lane]);
}

__device__ __forceinline__ double shfl_d(unsigned mask, double v, int src) { return __shfl_sync(mask, v, src, 16); }

template <typename T>
__device__ __forceinline__ void cross3(const T a[3], const T b[3], T o[3]) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

// Block sums of the per-thread accumulators in a fixed order; the last block
// to finish sums the block rows (in block order) and forms E_r, dE_r/dA,
// dE_r/dV and dE_r/dalpha.
__device__ void geo_finish(const GeoArgs &G, const double acc[kGeoWords], double (*red)[kGeoThreads]) {
  __shared__ bool last;
#pragma unroll
  for (int q = 0; q < kGeoWords; ++q) red[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int w = kGeoThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
#pragma unroll
      for (int q = 0; q < kGeoWords; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < kGeoWords) G.block[(size_t)blockIdx.x * kGeoWords + threadIdx.x] = red[threadIdx.x][0];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(G.done, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  // Fixed-order sum of the block rows (thread q sums word q).
  if (threadIdx.x < kGeoWords) {
    double t = 0;
    for (unsigned b = 0; b < gridDim.x; ++b) t += __ldcg(&G.block[(size_t)b * kGeoWords + threadIdx.x]);
    red[threadIdx.x][0] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double A = red[0][0], V = red[1][0];
    const double cA = G.A0 > 0 ? G.KA * (A - G.A0) / G.A0 : 0.0, cV = G.KV * (V - G.V0);
    G.gterm[kGeoA] = A;
    G.gterm[kGeoV] = V;
    G.gterm[kGeoE] = (G.A0 > 0 ? 0.5 * G.KA * (A - G.A0) * (A - G.A0) / G.A0 : 0.0) + 0.5 * G.KV * (V - G.V0) * (V - G.V0);
    G.gterm[kGeoCA] = cA;
    G.gterm[kGeoCV] = cV;
    for (int k = 0; k < 3; ++k) G.gterm[kGeoDAlpha + k] = cA * red[2 + k][0] + cV * red[5 + k][0];
    *G.done = 0u;
  }
}

// Sums A, V and their alpha derivatives in FP64 (the plain path).
__global__ void __launch_bounds__(kGeoThreads) geo_sums_kernel(GeoArgs G) {
  __shared__ GeoBasis<double> sb;
  __shared__ double Xs[kGeoHW][kMaxCpDev][3];
  __shared__ double red[kGeoWords][kGeoThreads];
  stage_geo_basis<double>(G, sb);
  __syncthreads();
  grid_dependency_wait();  // the state comes from the kernels before
  const int hw = threadIdx.x >> 4, lane = threadIdx.x & 15;
  const unsigned hmask = (threadIdx.x & 16) ? 0xFFFF0000u : 0x0000FFFFu;
  const double alpha[3] = {G.r[3 * (size_t)G.nv], G.r[3 * (size_t)G.nv + 1], G.r[3 * (size_t)G.nv + 2]};
  const double ialpha[3] = {1.0 / alpha[0], 1.0 / alpha[1], 1.0 / alpha[2]};
  double acc[kGeoWords] = {0, 0, 0, 0, 0, 0, 0, 0};  // A, V, dA/dalpha (3), dV/dalpha (3)
  for (int f = blockIdx.x * kGeoHW + hw; f < G.nfaces; f += gridDim.x * kGeoHW) {
    int lf;
    const int gi = geo_group(G, f, &lf);
    const GeoGroup &g = G.g[gi];
    double X[3] = {0, 0, 0};
    if (lane < g.ncp) geo_abs64(G, g, lf, lane, alpha, X, nullptr);
    double X0[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) X0[c] = shfl_d(hmask, X[c], 0);
    if (lane < g.ncp)
#pragma unroll
      for (int c = 0; c < 3; ++c) Xs[hw][lane][c] = X[c] - X0[c];
    __syncwarp(hmask);
    if (lane < g.npt) {
      double R[3] = {0, 0, 0}, Ru[3] = {0, 0, 0}, Rv[3] = {0, 0, 0};
      const double *bw = sb.B[gi][lane][0], *bu = sb.B[gi][lane][1], *bv = sb.B[gi][lane][2];
#pragma unroll
      for (int x = 0; x < kMaxCpDev; ++x) {
        if (x < g.ncp) {
          const double w = bw[x], u = bu[x], v = bv[x];
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const double xx = Xs[hw][x][c];
            R[c] = fma(w, xx, R[c]);
            Ru[c] = fma(u, xx, Ru[c]);
            Rv[c] = fma(v, xx, Rv[c]);
          }
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) R[c] += X0[c];  // back to absolute: the corner is exact in FP64
      double m[3];
      cross3(Ru, Rv, m);
      const double cw = sb.cw[gi][lane], c3 = cw * (1.0 / 3.0);
      acc[1] += c3 * (R[0] * m[0] + R[1] * m[1] + R[2] * m[2]);
      const double gg = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]), ig = 1.0 / gg;
      acc[0] += cw * gg;
      double n[3] = {m[0] * ig, m[1] * ig, m[2] * ig}, a1[3], a2[3], v1[3], v2[3];
      cross3(Rv, n, a1);  // dg/dRu
      cross3(n, Ru, a2);  // dg/dRv
      cross3(Rv, R, v1);  // d(R.m)/dRu
      cross3(R, Ru, v2);  // d(R.m)/dRv
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        acc[2 + k] += cw * (a1[k] * Ru[k] + a2[k] * Rv[k]) * ialpha[k];
        acc[5 + k] += c3 * (m[k] * R[k] + v1[k] * Ru[k] + v2[k] * Rv[k]) * ialpha[k];
      }
    }
    __syncwarp(hmask);
  }
  geo_finish(G, acc, red);
}

// ---- float-float (double-FP32) arithmetic for the precision form's volume.
// A value is hi + lo with |lo| <= ulp(hi)/2; the error-free transformations
// are Knuth's two-sum and the FMA two-product (Dekker's product with a fused
// multiply-add), so the arithmetic stays on the FP32 pipes and carries about
// 44 bits. Every product and sum inside them is rounded on its own (no
// contraction into an FMA), as the transformations require.
struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF ff_fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF ff_add(FF x, FF y) {
  float s, e;
  two_sum(x.hi, y.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(x.lo, y.lo));
  return ff_fast_two_sum(s, e);
}
__device__ __forceinline__ FF ff_mul(FF x, FF y) {
  const float p = __fmul_rn(x.hi, y.hi);
  float e = __fmaf_rn(x.hi, y.hi, -p);
  e = __fmaf_rn(x.hi, y.lo, e);
  e = __fmaf_rn(x.lo, y.hi, e);
  return ff_fast_two_sum(p, e);
}
// acc += b x, without renormalising acc (call ff_norm once at the end).
__device__ __forceinline__ void ff_acc(FF &acc, float bh, float bl, float xh, float xl) {
  const float p = __fmul_rn(bh, xh);
  float e = __fmaf_rn(bh, xh, -p);
  e = __fmaf_rn(bh, xl, e);
  e = __fmaf_rn(bl, xh, e);
  float s, t;
  two_sum(acc.hi, p, s, t);
  acc.hi = s;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(t, e));
}
__device__ __forceinline__ FF ff_norm(FF x) { return ff_fast_two_sum(x.hi, x.lo); }
__device__ __forceinline__ FF ff_of(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}

// The precision form's sums: V from float-float contractions of float-float
// local coordinates (formed from the FP32 hi/lo position pairs with error-free
// sums) and summed in float-float per thread; the area and the box-scale
// derivatives from the FP32 leading parts with Kahan sums. FP64 enters only in
// the per-block and final sums.
//
// One face per thread. Each thread keeps its face's
// float-float local coordinates in its own columns of shared memory
// (coordinate-major, control points padded to 16, the column 400 bytes, an
// odd number of 16-byte chunks, so a warp's 16-byte reads do not conflict),
// and walks the face's points; the value and derivative rows of the point
// (hi and lo) are the same for every thread of a warp that is on the same
// patch type, so they come out of shared memory as broadcasts. (A half-warp
// form, lanes = points with per-lane row reads, took 177.6 us on a 40,962-vertex
// vesicle against 154.5 us for this one, both issue-bound on the float-float
// arithmetic.)
namespace geo_tpf {
constexpr int kThreads = 128;
constexpr int kCp = 16;                  // control points, padded
constexpr int kCol = 3 * kCp * 2 + 4;    // floats of a thread's column: hi [3][16], lo [3][16], pad
struct Rows {
  float4 r[3][kGeoPt][6][kCp / 4];       // [group][point][w hi, w lo, u hi, u lo, v hi, v lo][control points in fours]
  float cw[3][kGeoPt];
  FF c3[3][kGeoPt];
};
constexpr size_t kDynBytes = sizeof(float) * kCol * kThreads;
}  // namespace geo_tpf

template <int NCP, int NPT>
__device__ __forceinline__ void geo_face_ff(const GeoArgs &G, const GeoGroup &g, const geo_tpf::Rows &rows, int gi,
                                            int lf, const FF alpha[3], const float ialpha[3], float *col, FF &accV,
                                            float ks[kGeoWords], float kc[kGeoWords]) {
  using namespace geo_tpf;
  auto kahan = [&](int q, float v) {
    const float y = v - kc[q], t = ks[q] + y;
    kc[q] = (t - ks[q]) - y;
    ks[q] = t;
  };
  // ---- local coordinates (float-float, relative to the corner, in their images, times alpha)
  const uint32_t *cp = g.cp + (size_t)lf * NCP;
  float ahi[3], alo[3];
  {
    const int v0 = (int)(__ldg(&cp[0]) & kVertexMask);
#pragma unroll
    for (int c = 0; c < 3; ++c) { ahi[c] = G.rhi[3 * (size_t)v0 + c]; alo[c] = G.rlo[3 * (size_t)v0 + c]; }
  }
  FF X0[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) X0[c] = ff_mul(alpha[c], FF{ahi[c], alo[c]});  // the corner carries no image
#pragma unroll
  for (int j = 0; j < kCp; ++j) {
    float xh[3] = {0.f, 0.f, 0.f}, xl[3] = {0.f, 0.f, 0.f};
    if (j < NCP) {
      const uint32_t packed = __ldg(&cp[j]);
      const int v = (int)(packed & kVertexMask), code = (int)(packed >> kVertexBits);
      const int img[3] = {code % 3 - 1, (code / 3) % 3 - 1, code / 9 - 1};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float hi = G.rhi[3 * (size_t)v + c], lo = G.rlo[3 * (size_t)v + c];
        float sh = 0.f, she = 0.f, shl = 0.f;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          float t, e;
          two_sum(sh, __fmul_rn((float)img[d], G.box_hi[d][c]), t, e);
          sh = t;
          she = __fadd_rn(she, e);
          shl = __fadd_rn(shl, __fmul_rn((float)img[d], G.box_lo[d][c]));
        }
        float s1, e1, s2, e2;
        two_sum(hi, sh, s1, e1);
        two_sum(s1, -ahi[c], s2, e2);
        const float res = __fadd_rn(__fadd_rn(e1, e2), __fadd_rn(__fsub_rn(lo, alo[c]), __fadd_rn(she, shl)));
        const FF x = ff_mul(alpha[c], ff_fast_two_sum(s2, res));
        xh[c] = x.hi;
        xl[c] = x.lo;
      }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      col[c * kCp + j] = xh[c];
      col[3 * kCp + c * kCp + j] = xl[c];
    }
  }
  // ---- the points
#pragma unroll 1
  for (int p = 0; p < NPT; ++p) {
    FF R[3] = {{0, 0}, {0, 0}, {0, 0}}, Ru[3] = {{0, 0}, {0, 0}, {0, 0}}, Rv[3] = {{0, 0}, {0, 0}, {0, 0}};
#pragma unroll 1  // rolled: the unrolled body (about 1,900 instructions) missed in the instruction cache
    for (int q = 0; q < (NCP + 3) / 4; ++q) {
      const float4 w4h = rows.r[gi][p][0][q], w4l = rows.r[gi][p][1][q], u4h = rows.r[gi][p][2][q],
                   u4l = rows.r[gi][p][3][q], v4h = rows.r[gi][p][4][q], v4l = rows.r[gi][p][5][q];
      const float wh[4] = {w4h.x, w4h.y, w4h.z, w4h.w}, wl[4] = {w4l.x, w4l.y, w4l.z, w4l.w};
      const float uh[4] = {u4h.x, u4h.y, u4h.z, u4h.w}, ul[4] = {u4l.x, u4l.y, u4l.z, u4l.w};
      const float vh[4] = {v4h.x, v4h.y, v4h.z, v4h.w}, vl[4] = {v4l.x, v4l.y, v4l.z, v4l.w};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float4 x4h = *reinterpret_cast<const float4 *>(&col[c * kCp + 4 * q]);
        const float4 x4l = *reinterpret_cast<const float4 *>(&col[3 * kCp + c * kCp + 4 * q]);
        const float xh[4] = {x4h.x, x4h.y, x4h.z, x4h.w}, xl[4] = {x4l.x, x4l.y, x4l.z, x4l.w};
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          if (4 * q + jj >= NCP) break;
          ff_acc(R[c], wh[jj], wl[jj], xh[jj], xl[jj]);
          ff_acc(Ru[c], uh[jj], ul[jj], xh[jj], xl[jj]);
          ff_acc(Rv[c], vh[jj], vl[jj], xh[jj], xl[jj]);
        }
      }
    }
    FF Ra[3], m[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      Ru[c] = ff_norm(Ru[c]);
      Rv[c] = ff_norm(Rv[c]);
      Ra[c] = ff_add(X0[c], ff_norm(R[c]));
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int a = (c + 1) % 3, b = (c + 2) % 3;
      const FF t = ff_mul(Ru[b], Rv[a]);
      m[c] = ff_add(ff_mul(Ru[a], Rv[b]), FF{-t.hi, -t.lo});
    }
    const FF dot = ff_add(ff_add(ff_mul(Ra[0], m[0]), ff_mul(Ra[1], m[1])), ff_mul(Ra[2], m[2]));
    accV = ff_add(accV, ff_mul(rows.c3[gi][p], dot));
    // area and box-scale derivatives from the leading parts
    const float Rf[3] = {Ra[0].hi, Ra[1].hi, Ra[2].hi}, Uf[3] = {Ru[0].hi, Ru[1].hi, Ru[2].hi},
                Vf[3] = {Rv[0].hi, Rv[1].hi, Rv[2].hi}, mf[3] = {m[0].hi, m[1].hi, m[2].hi};
    const float gg2 = mf[0] * mf[0] + mf[1] * mf[1] + mf[2] * mf[2];
    const float ig = rsqrtf(gg2), gg = gg2 * ig;
    const float cwf = rows.cw[gi][p], c3f = rows.c3[gi][p].hi;
    kahan(0, cwf * gg);
    float n[3] = {mf[0] * ig, mf[1] * ig, mf[2] * ig}, a1[3], a2[3], v1[3], v2[3];
    cross3(Vf, n, a1);
    cross3(n, Uf, a2);
    cross3(Vf, Rf, v1);
    cross3(Rf, Uf, v2);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      kahan(2 + k, cwf * (a1[k] * Uf[k] + a2[k] * Vf[k]) * ialpha[k]);
      kahan(5 + k, c3f * (mf[k] * Rf[k] + v1[k] * Uf[k] + v2[k] * Vf[k]) * ialpha[k]);
    }
  }
}

__global__ void __launch_bounds__(geo_tpf::kThreads, 3) geo_sums_ff_tpf_kernel(GeoArgs G) {
  using namespace geo_tpf;
  __shared__ Rows rows;
  __shared__ FF alpha_s[3];
  __shared__ float ialpha_s[3];
  extern __shared__ __align__(16) float geo_cols[];
  for (int gi = 0; gi < G.ngroups; ++gi) {  // rows hi/lo, control points padded with zeros
    const GeoGroup &g = G.g[gi];
    const int nrow = g.npt * 3 * g.ncp;
    float *r = &rows.r[gi][0][0][0].x;
    for (int i = threadIdx.x; i < g.npt * 6 * kCp; i += blockDim.x) {
      const int p = i / (6 * kCp), k = (i / kCp) % 6, x = i % kCp;  // k: row (w, u, v) * 2 + lo
      const int e = p * 3 * g.ncp + (k / 2) * g.ncp + x;
      r[((size_t)p * 6 + k) * kCp + x] = x < g.ncp ? g.tab[(k & 1) * nrow + e] : 0.f;
    }
    for (int p = threadIdx.x; p < g.npt; p += blockDim.x) {
      rows.cw[gi][p] = g.tab[2 * nrow + p];
      rows.c3[gi][p] = FF{g.tab[2 * nrow + g.npt + p], g.tab[2 * nrow + 2 * g.npt + p]};
    }
  }
  grid_dependency_wait();  // the state comes from the kernels before
  if (threadIdx.x < 3) {
    const double a = G.r[3 * (size_t)G.nv + threadIdx.x];
    alpha_s[threadIdx.x] = ff_of(a);
    ialpha_s[threadIdx.x] = 1.f / (float)a;
  }
  __syncthreads();
  const FF alpha[3] = {alpha_s[0], alpha_s[1], alpha_s[2]};
  const float ialpha[3] = {ialpha_s[0], ialpha_s[1], ialpha_s[2]};
  float *col = geo_cols + (size_t)kCol * threadIdx.x;
  FF accV = {0, 0};
  float ks[kGeoWords] = {0, 0, 0, 0, 0, 0, 0, 0}, kc[kGeoWords] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int f = blockIdx.x * kThreads + threadIdx.x; f < G.nfaces; f += gridDim.x * kThreads) {
    int lf;
    const int gi = geo_group(G, f, &lf);
    const GeoGroup &g = G.g[gi];
    if (g.ncp == 12) geo_face_ff<12, 15>(G, g, rows, gi, lf, alpha, ialpha, col, accV, ks, kc);
    else if (g.ncp == 11) geo_face_ff<11, 16>(G, g, rows, gi, lf, alpha, ialpha, col, accV, ks, kc);
    else geo_face_ff<13, 16>(G, g, rows, gi, lf, alpha, ialpha, col, accV, ks, kc);
  }
  double acc[kGeoWords];
#pragma unroll
  for (int q = 0; q < kGeoWords; ++q) acc[q] = (double)ks[q] - (double)kc[q];
  acc[1] = (double)accV.hi + (double)accV.lo;
  __syncthreads();  // every column is done with: the block sums reuse their space
  static_assert(kDynBytes >= sizeof(double) * kGeoWords * kThreads, "block sums must fit in the columns");
  geo_finish(G, acc, reinterpret_cast<double(*)[kThreads]>(geo_cols));
}

// partial[slot] += alpha * dE_r/dX for every (face, control point):
//   dE_r/dR  = c_V c/3 m,   dE_r/dRu = c_A c (Rv x n) + c_V c/3 (Rv x R),
//   dE_r/dRv = c_A c (n x Ru) + c_V c/3 (R x Ru),
// contracted with the w, u, v rows (lanes = points, then lanes = control points).
template <typename T>
__global__ void __launch_bounds__(kGeoThreads) geo_grad_kernel(GeoArgs G, T *__restrict__ partial) {
  grid_dependency_wait();  // the coefficients come from the sums kernel, the partials from the face launches
  const double cA64 = G.gterm[kGeoCA], cV64 = G.gterm[kGeoCV];
  if (cA64 == 0.0 && cV64 == 0.0) return;
  __shared__ GeoBasis<T> sb;
  __shared__ T Xs[kGeoHW][kMaxCpDev][3];
  __shared__ T Es[kGeoHW][kGeoPt][9];
  if constexpr (sizeof(T) == 4) {
    for (int gi = 0; gi < G.ngroups; ++gi) {
      const GeoGroup &g = G.g[gi];
      const int nrow = g.npt * 3 * g.ncp;
      for (int i = threadIdx.x; i < nrow; i += blockDim.x) sb.B[gi][i / (3 * g.ncp)][(i / g.ncp) % 3][i % g.ncp] = g.tab[i];
      for (int p = threadIdx.x; p < g.npt; p += blockDim.x) sb.cw[gi][p] = g.tab[2 * nrow + p];
    }
  } else {
    stage_geo_basis<T>(G, sb);
  }
  __syncthreads();
  const int hw = threadIdx.x >> 4, lane = threadIdx.x & 15;
  const unsigned hmask = (threadIdx.x & 16) ? 0xFFFF0000u : 0x0000FFFFu;
  const double a64[3] = {G.r[3 * (size_t)G.nv], G.r[3 * (size_t)G.nv + 1], G.r[3 * (size_t)G.nv + 2]};
  const T alpha[3] = {(T)a64[0], (T)a64[1], (T)a64[2]};
  const T cA = (T)cA64, cV = (T)cV64;
  for (int f = blockIdx.x * kGeoHW + hw; f < G.nfaces; f += gridDim.x * kGeoHW) {
    int lf;
    const int gi = geo_group(G, f, &lf);
    const GeoGroup &g = G.g[gi];
    {  // the next face's control-point and slot rows into L1 while this face runs
      const int fn = f + gridDim.x * kGeoHW;
      if (lane < 2 && fn < G.nfaces) {
        int lfn;
        const GeoGroup &h = G.g[geo_group(G, fn, &lfn)];
        const size_t at = (size_t)lfn * h.ncp + (lane ? h.ncp - 1 : 0);
        tpf::prefetch_l1(h.cp + at);
        tpf::prefetch_l1(h.dest + at);
      }
    }
    int dest = 0;
    T X0[3];
    if constexpr (sizeof(T) == 8) {
      double X[3] = {0, 0, 0};
      if (lane < g.ncp) geo_abs64(G, g, lf, lane, a64, X, &dest);
#pragma unroll
      for (int c = 0; c < 3; ++c) X0[c] = shfl_d(hmask, X[c], 0);
      if (lane < g.ncp)
#pragma unroll
        for (int c = 0; c < 3; ++c) Xs[hw][lane][c] = X[c] - X0[c];
    } else {
      // FP32 coordinates relative to the corner from the hi/lo pairs with
      // error-free sums, as the face pass forms them.
      float hi[3] = {0, 0, 0}, lo[3] = {0, 0, 0};
      int img[3] = {0, 0, 0};
      if (lane < g.ncp) {
        const uint32_t packed = __ldg(&g.cp[(size_t)lf * g.ncp + lane]);
        const int v = (int)(packed & kVertexMask), code = (int)(packed >> kVertexBits);
        img[0] = code % 3 - 1; img[1] = (code / 3) % 3 - 1; img[2] = code / 9 - 1;
#pragma unroll
        for (int c = 0; c < 3; ++c) { hi[c] = G.rhi[3 * (size_t)v + c]; lo[c] = G.rlo[3 * (size_t)v + c]; }
        dest = __ldg(&g.dest[(size_t)lf * g.ncp + lane]);
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float ahi = __shfl_sync(hmask, hi[c], 0, 16), alo = __shfl_sync(hmask, lo[c], 0, 16);
        float sh = 0.f, she = 0.f, shl = 0.f;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          float t, e;
          two_sum(sh, (float)img[d] * G.box_hi[d][c], t, e);
          sh = t;
          she += e;
          shl += (float)img[d] * G.box_lo[d][c];
        }
        float s1, e1, s2, e2;
        two_sum(hi[c], sh, s1, e1);
        two_sum(s1, -ahi, s2, e2);
        if (lane < g.ncp) Xs[hw][lane][c] = alpha[c] * (s2 + ((e1 + e2) + ((lo[c] - alo) + (she + shl))));
        X0[c] = alpha[c] * (ahi + alo);  // the corner carries no image (its shift is zero)
      }
    }
    // this face's partial slots, read now so that the read-modify-write at the
    // end does not wait on them (no other thread touches these slots)
    T old[3] = {0, 0, 0};
    if (lane < g.ncp)
#pragma unroll
      for (int k = 0; k < 3; ++k) old[k] = partial[3 * (size_t)dest + k];
    __syncwarp(hmask);
    if (lane < g.npt) {
      T R[3] = {0, 0, 0}, Ru[3] = {0, 0, 0}, Rv[3] = {0, 0, 0};
      const T *bw = sb.B[gi][lane][0], *bu = sb.B[gi][lane][1], *bv = sb.B[gi][lane][2];
#pragma unroll
      for (int x = 0; x < kMaxCpDev; ++x) {
        if (x < g.ncp) {
          const T w = bw[x], u = bu[x], v = bv[x];
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const T xx = Xs[hw][x][c];
            R[c] += w * xx;
            Ru[c] += u * xx;
            Rv[c] += v * xx;
          }
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) R[c] += X0[c];
      T m[3], n[3], a1[3], a2[3], v1[3], v2[3];
      cross3(Ru, Rv, m);
      const T ig = T(1) / sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
#pragma unroll
      for (int c = 0; c < 3; ++c) n[c] = m[c] * ig;
      cross3(Rv, n, a1);
      cross3(n, Ru, a2);
      cross3(Rv, R, v1);
      cross3(R, Ru, v2);
      const T cw = sb.cw[gi][lane], kA = cA * cw, kV = cV * cw * (T(1) / T(3));
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        Es[hw][lane][k] = kV * m[k];
        Es[hw][lane][3 + k] = kA * a1[k] + kV * v1[k];
        Es[hw][lane][6 + k] = kA * a2[k] + kV * v2[k];
      }
    }
    __syncwarp(hmask);
    if (lane < g.ncp) {
      T Gx[3] = {0, 0, 0};
      for (int p = 0; p < g.npt; ++p) {
        const T w = sb.B[gi][p][0][lane], u = sb.B[gi][p][1][lane], v = sb.B[gi][p][2][lane];
#pragma unroll
        for (int k = 0; k < 3; ++k) Gx[k] += w * Es[hw][p][k] + u * Es[hw][p][3 + k] + v * Es[hw][p][6 + k];
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) partial[3 * (size_t)dest + k] = old[k] + alpha[k] * Gx[k];
    }
    __syncwarp(hmask);
  }
}

// One warp per row; lanes stride the row's nonzeros (coalesced reads of the
// value/column streams), warp-shuffle sum in fixed order.
__global__ void spmv_kernel(int nrow, const int *__restrict__ row_ptr, const int *__restrict__ col,
                            const double *__restrict__ val, const double *__restrict__ scalev, double scale,
                            const double *__restrict__ alphas, const double *__restrict__ in, double *__restrict__ out,
                            int accumulate) {
  grid_dependency_wait();
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

// spmv_kernel on FP32 values and an FP32 copy of the input packed as one
// float4 per row {x, y, z, 0} (the precision form's inverse mass), so each
// nonzero gathers its input with one 16-byte load. kSpmvUnroll nonzeros per
// lane per round have their loads in flight together. Kahan-compensated FP32 sums
// per lane, the cross-lane sum and the scaling in FP64. Reads 8 bytes per
// nonzero instead of 12 and keeps the FP64 pipe out of the loop.
constexpr int kSpmvUnroll = 4;
// spmv32_kernel streams each row's values and columns, kSpmvUnroll windows of
// 32 nonzeros per warp iteration; a warp also asks L2 for the lines
// kSpmvAhead windows ahead of the ones it loads, so that its loads find them
// there (40,962-vertex M^-1, 415 M nonzeros: 546 -> about 475 us per apply).
constexpr int kSpmvAhead = 32;
__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }
template <typename C>  // column index type: int, or uint16_t for up to 65,536 columns
__global__ void spmv32_kernel(int nrow, const int *__restrict__ row_ptr, const C *__restrict__ col,
                              const float *__restrict__ val, const double *__restrict__ scalev, double scale,
                              const double *__restrict__ alphas, const float4 *__restrict__ in4,
                              double *__restrict__ out, int accumulate) {
  grid_dependency_wait();
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
    HalfWarpSums<float> acc;
    const int beg = row_ptr[i], end = row_ptr[i + 1];
    for (int w = 32 * lane; w < 32 * kSpmvAhead; w += 32 * 32) {  // the row's first windows
      if (w < end - beg) {
        prefetch_l2(&val[beg + w]);
        prefetch_l2(&col[beg + w]);
      }
    }
    for (int k0 = beg + lane; k0 < end; k0 += 32 * kSpmvUnroll) {
      if (lane < 2 * kSpmvUnroll) {  // lanes 0..3: value lines ahead; lanes 4..7: their columns
        const int w = k0 - lane, ahead = 32 * (kSpmvAhead + (lane % kSpmvUnroll));
        if (ahead < end - w)
          prefetch_l2(lane < kSpmvUnroll ? (const void *)&val[w + ahead] : (const void *)&col[w + ahead]);
      }
      float v[kSpmvUnroll];
      int j[kSpmvUnroll];
#pragma unroll
      for (int u = 0; u < kSpmvUnroll; ++u) {
        const int k = k0 + 32 * u;
        v[u] = k < end ? __ldcs(&val[k]) : 0.f;
        j[u] = k < end ? (int)__ldcs(&col[k]) : 0;
      }
      float4 x[kSpmvUnroll];
#pragma unroll
      for (int u = 0; u < kSpmvUnroll; ++u) x[u] = __ldg(&in4[j[u]]);
      // groups of four products summed by plain multiply-adds, each group
      // added to the compensated total
#pragma unroll
      for (int g = 0; g < kSpmvUnroll; g += 4) {
        float t0 = v[g] * x[g].x, t1 = v[g] * x[g].y, t2 = v[g] * x[g].z;
#pragma unroll
        for (int u = g + 1; u < g + 4; ++u) {
          t0 = fmaf(v[u], x[u].x, t0);
          t1 = fmaf(v[u], x[u].y, t1);
          t2 = fmaf(v[u], x[u].z, t2);
        }
        acc.add(0, t0);
        acc.add(1, t1);
        acc.add(2, t2);
      }
    }
    double s[3] = {acc.get(0), acc.get(1), acc.get(2)};
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1)
#pragma unroll
      for (int c = 0; c < 3; ++c) s[c] += __shfl_xor_sync(0xffffffffu, s[c], off);
    if (lane == 0) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        double o = s[c] * f[c];
        if (scalev) o *= scalev[(size_t)c * nrow + i];
        if (accumulate) out[3 * (size_t)i + c] += o;
        else out[3 * (size_t)i + c] = o;
      }
    }
  }
}

// Rows of three doubles to float4 {x, y, z, 0}.
__global__ void to_f32x4_kernel(int n, const double *__restrict__ in, float4 *__restrict__ out) {
  grid_dependency_wait();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = make_float4((float)in[3 * (size_t)i], (float)in[3 * (size_t)i + 1], (float)in[3 * (size_t)i + 2], 0.f);
}

}  // namespace dev

static int grid_for(int n, int per_block) {
  int g = (n + per_block - 1) / per_block;
  return g < 1 ? 1 : g;
}

// A value fixed per device and computed once on it (thread-safe: meshes may
// be made on several threads). cudaFuncSetAttribute applies to the current
// device only, and the persistent grids follow each device's SM count, so
// neither may be shared between the devices of one process.
constexpr int kMaxDevices = 64;
// Launch with programmatic stream serialization: the kernel may be scheduled
// while the kernel before it on the stream drains, and waits for it in
// grid_dependency_wait (which it calls before reading that kernel's results).
template <typename... P, typename... A>
static cudaError_t launch_after(void (*kernel)(P...), int grid, int block, size_t smem, cudaStream_t s, A... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<P>(args)...);
}

struct PerDevice {
  std::once_flag once[kMaxDevices];
  int value[kMaxDevices] = {};
};
template <class F>
static int per_device(PerDevice &pd, F make) {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= kMaxDevices) return make();
  std::call_once(pd.once[dev], [&] { pd.value[dev] = make(); });
  return pd.value[dev];
}
// The dynamic shared memory limit above 48 KB that the tensor-core kernel
// opts into, once per device; returns the cudaError_t of the opt-in.
static cudaError_t tc_opt_in() {
  static PerDevice pd;
  return (cudaError_t)per_device(pd, [] {
    return (int)cudaFuncSetAttribute(dev::face_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)dev::tc::kSmemBytes);
  });
}
static int sm_count() {
  static PerDevice pd;
  return per_device(pd, [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
  });
}

template <typename T, int NCP, int NPT>
static int face_grid_size(int nfaces) {
  // Persistent grid: as many blocks as fit on the device at once (a fixed
  // number per device, so the face-to-block assignment and the sums' order are fixed).
  static PerDevice pd;
  const int cached = per_device(pd, [] {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::face_kernel<T, NCP, NPT>,
                                                  dev::FaceCfg<T>::threads, 0);
    return sm_count() * (per_sm > 0 ? per_sm : 1);
  });
  int need = grid_for(nfaces, dev::FaceCfg<T>::half_warps);
  return need < cached ? need : cached;
}

// The thread-per-face kernel's persistent grid (precision form, regular faces).
static int face_grid_size_tpf(int nfaces) {
  static PerDevice pd;
  const int cached = per_device(pd, [] {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::face_tpf_kernel, dev::tpf::kThreads,
                                                  dev::tpf::kSumBytes);
    return sm_count() * (per_sm > 0 ? per_sm : 1);
  });
  int need = grid_for(nfaces, dev::tpf::kThreads);
  return need < cached ? need : cached;
}

template <typename T>
int face_blocks(int nfaces, int ncp, int npt) {
  if (nfaces <= 0) return 0;
  if (sizeof(T) == 4 && ncp == 12 && npt == 15) return face_grid_size_tpf(nfaces);
  if (ncp == 12 && npt == 15) return face_grid_size<T, 12, 15>(nfaces);
  if (ncp == 11 && npt == 16) return face_grid_size<T, 11, 16>(nfaces);
  if (ncp == 13 && npt == 16) return face_grid_size<T, 13, 16>(nfaces);
  return 0;
}
template int face_blocks<double>(int, int, int);
template int face_blocks<float>(int, int, int);

template <typename T>
cudaError_t launch_faces(const dev::FaceLaunch &L, const int *dest, int ncp, int npt, const dev::SurfaceParams &P,
                         const double *r, const F32Pos &f, T *partial, double *blockpart, int *status, int grid,
                         const FinishArgs &fin, cudaStream_t s) {
  if (L.nfaces <= 0) return cudaSuccess;
  constexpr int NT = dev::FaceCfg<T>::threads;
  const float *rhi = f.hi, *rlo = f.lo, *dsp = f.dsp;
  if constexpr (sizeof(T) == 4) {
    if (!rhi || !rlo || !dsp) return cudaErrorInvalidValue;
    if (ncp == 12 && npt == 15)
      return launch_after(dev::face_tpf_kernel, grid, dev::tpf::kThreads, dev::tpf::kSumBytes, s, L, dest, P, r, rhi,
                          rlo, dsp, partial, blockpart, status, fin);
  }
  if (ncp == 12 && npt == 15)
    return launch_after(dev::face_kernel<T, 12, 15>, grid, NT, 0, s, L, dest, P, r, rhi, rlo, dsp, partial, blockpart,
                        status, fin);
  else if (ncp == 11 && npt == 16)
    dev::face_kernel<T, 11, 16><<<grid, NT, 0, s>>>(L, dest, P, r, rhi, rlo, dsp, partial, blockpart, status,
                                                           fin);
  else if (ncp == 13 && npt == 16)
    dev::face_kernel<T, 13, 16><<<grid, NT, 0, s>>>(L, dest, P, r, rhi, rlo, dsp, partial, blockpart, status,
                                                           fin);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}
template cudaError_t launch_faces<double>(const dev::FaceLaunch &, const int *, int, int, const dev::SurfaceParams &,
                                          const double *, const F32Pos &, double *, double *, int *, int,
                                          const FinishArgs &, cudaStream_t);
template cudaError_t launch_faces<float>(const dev::FaceLaunch &, const int *, int, int, const dev::SurfaceParams &,
                                         const double *, const F32Pos &, float *, double *, int *, int,
                                         const FinishArgs &, cudaStream_t);

cudaError_t launch_split_positions(int n, const double *r, const F32Pos &f, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (!f.hi || !f.lo || !f.r0 || !f.dsp) return cudaErrorInvalidValue;
  dev::split_positions_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, r, f.hi, f.lo, f.r0, f.dsp);
  return cudaGetLastError();
}

cudaError_t launch_status_merge(const int *src, int *dst, cudaStream_t s) {
  dev::status_merge_kernel<<<1, 1, 0, s>>>(src, dst);
  return cudaGetLastError();
}

cudaError_t launch_finish(const FinishArgs &F, const double *blockpart, cudaStream_t s) {
  dev::finish_kernel<<<1, 256, 0, s>>>(F, blockpart);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_gather(int nv, const T *partial, const int *off, double *g, cudaStream_t s) {
  if (nv <= 0) return cudaSuccess;
  dev::gather_kernel<T><<<grid_for(nv, 256), 256, 0, s>>>(nv, partial, off, g);
  return cudaGetLastError();
}
template cudaError_t launch_gather<double>(int, const double *, const int *, double *, cudaStream_t);
template cudaError_t launch_gather<float>(int, const float *, const int *, double *, cudaStream_t);

template <typename T>
cudaError_t launch_gather_step(int nv, const T *partial, const int *off, const StepArgs &a, const uint64_t *cnt,
                               double *r, double *p, const F32Pos &f, const int *status, cudaStream_t s) {
  return launch_after(dev::gather_step_kernel<T>, grid_for(nv, 256), 256, 0, s, nv, partial, off, a, cnt, r, p, f.hi,
                      f.lo, f.r0, f.dsp, status);
}
template cudaError_t launch_gather_step<double>(int, const double *, const int *, const StepArgs &, const uint64_t *,
                                                double *, double *, const F32Pos &, const int *, cudaStream_t);
template cudaError_t launch_gather_step<float>(int, const float *, const int *, const StepArgs &, const uint64_t *,
                                               double *, double *, const F32Pos &, const int *, cudaStream_t);

cudaError_t launch_kick(int nv, const StepArgs &a, const uint64_t *cnt, double *p, const double *g, const int *status,
                        cudaStream_t s) {
  return launch_after(dev::kick_kernel, grid_for(nv, 256), 256, 0, s, nv, a, cnt, p, g, status);
}
cudaError_t launch_drift(int nv, const StepArgs &a, double *r, double *p, const double *qdot, const F32Pos &f,
                         const int *status, cudaStream_t s) {
  return launch_after(dev::drift_kernel, grid_for(3 * nv, 256), 256, 0, s, nv, a, r, p, qdot, f.hi, f.lo, f.r0, f.dsp,
                      status);
}
cudaError_t launch_spmv32(int nrow, const int *row_ptr, const void *col, bool col16, const float *val,
                          const double *scalev, double scale, const double *alphas, const float4 *in, double *out,
                          int accumulate, cudaStream_t s) {
  if (nrow <= 0) return cudaSuccess;
  int warps_per_block = 8;
  int grid = grid_for(nrow, warps_per_block);
  if (grid > 152 * 16) grid = 152 * 16;
  // consecutive lanes take consecutive nonzeros, so runs of consecutive columns
  // gather the input with coalesced loads (a form with four nonzeros per lane,
  // 16-byte value loads, was slower: 0.80 against 0.55 ms at 40,962 rows)
  if (col16)
    return launch_after(dev::spmv32_kernel<uint16_t>, grid, 32 * warps_per_block, 0, s, nrow, row_ptr,
                        static_cast<const uint16_t *>(col), val, scalev, scale, alphas, in, out, accumulate);
  return launch_after(dev::spmv32_kernel<int>, grid, 32 * warps_per_block, 0, s, nrow, row_ptr,
                      static_cast<const int *>(col), val, scalev, scale, alphas, in, out, accumulate);
}

cudaError_t launch_to_f32x4(int n, const double *in, float4 *out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int g = grid_for(n, 256);
  return launch_after(dev::to_f32x4_kernel, g < 152 * 8 ? g : 152 * 8, 256, 0, s, n, in, out);
}

cudaError_t launch_spmv(int nrow, const int *row_ptr, const int *col, const double *val, const double *scalev,
                        double scale, const double *alphas, const double *in, double *out, int accumulate,
                        cudaStream_t s) {
  if (nrow <= 0) return cudaSuccess;
  int warps_per_block = 8;
  int grid = grid_for(nrow, warps_per_block);
  if (grid > 152 * 16) grid = 152 * 16;
  return launch_after(dev::spmv_kernel, grid, 32 * warps_per_block, 0, s, nrow, row_ptr, col, val, scalev, scale,
                      alphas, in, out, accumulate);
}

}  // namespace umcp

namespace umcp {

template <typename T>
int batch_face_blocks(int ncp, int npt) {
  if (sizeof(T) == 4 && ncp == 12 && npt == 15) {  // the batched thread-per-face kernel's own occupancy
    static PerDevice pd;
    return per_device(pd, [] {
      int per_sm = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::batch_face_tpf_kernel, dev::tpf::kThreads, 0);
      return sm_count() * (per_sm > 0 ? per_sm : 1);
    });
  }
  return face_blocks<T>(1 << 30, ncp, npt);  // device-filling persistent grid
}
template int batch_face_blocks<double>(int, int);
template int batch_face_blocks<float>(int, int);

template <typename T>
cudaError_t launch_batch_faces(const BatchJob *jobs, int group, const BatchTile *tiles, const int *counts,
                               const double *basis, const double *weight, int ncp, int npt, double dudv,
                               int irregular, double *tile_sums, int grid, int *next_tile, cudaStream_t s) {
  constexpr int NT = dev::FaceCfg<T>::threads;
  if constexpr (sizeof(T) == 4) {
    if (ncp == 12 && npt == 15) {
      if (!next_tile) return cudaErrorInvalidValue;
      return launch_after(dev::batch_face_tpf_kernel, grid, dev::tpf::kThreads, 0, s, jobs, group, tiles, counts,
                          basis, weight, dudv, tile_sums, next_tile);
    }
  }
  if (ncp == 12 && npt == 15)
    dev::batch_face_kernel<T, 12, 15><<<grid, NT, 0, s>>>(jobs, group, tiles, counts, basis, weight, dudv, irregular,
                                                          tile_sums);
  else if (ncp == 11 && npt == 16)
    dev::batch_face_kernel<T, 11, 16><<<grid, NT, 0, s>>>(jobs, group, tiles, counts, basis, weight, dudv, irregular,
                                                          tile_sums);
  else if (ncp == 13 && npt == 16)
    dev::batch_face_kernel<T, 13, 16><<<grid, NT, 0, s>>>(jobs, group, tiles, counts, basis, weight, dudv, irregular,
                                                          tile_sums);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}
template cudaError_t launch_batch_faces<double>(const BatchJob *, int, const BatchTile *, const int *,
                                                const double *, const double *, int, int, double, int, double *, int,
                                                int *, cudaStream_t);
template cudaError_t launch_batch_faces<float>(const BatchJob *, int, const BatchTile *, const int *, const double *,
                                               const double *, int, int, double, int, double *, int, int *,
                                               cudaStream_t);

cudaError_t launch_batch_reduce(const BatchJob *jobs, const int *counts, int max_jobs, const int *tile_off,
                                const int *tile_idx, const double *tile_sums, int *live, unsigned long long *prog,
                                cudaStream_t s) {
  return launch_after(dev::batch_reduce_kernel, grid_for(max_jobs * 32, 256), 256, 0, s, jobs, counts, tile_off,
                      tile_idx, tile_sums, live, prog);
}

template <typename T>
cudaError_t launch_batch_gather_step(const BatchJob *jobs, const BatchTile *vtiles, const int *counts,
                                     const int *live, int grid, cudaStream_t s) {
  return launch_after(dev::batch_gather_step_kernel<T>, grid, kVertexTile, 0, s, jobs, vtiles, counts, live);
}
template cudaError_t launch_batch_gather_step<double>(const BatchJob *, const BatchTile *, const int *, const int *,
                                                      int, cudaStream_t);
template cudaError_t launch_batch_gather_step<float>(const BatchJob *, const BatchTile *, const int *, const int *,
                                                     int, cudaStream_t);

cudaError_t launch_batch_start(const BatchJob *jobs, const BatchTile *vtiles, const int *counts, const int *start,
                               const unsigned long long *step0, int grid, cudaStream_t s) {
  dev::batch_start_kernel<<<grid, kVertexTile, 0, s>>>(jobs, vtiles, counts, start, step0);
  return cudaGetLastError();
}

cudaError_t launch_batch_unpack(const BatchJob *jobs, const BatchTile *vtiles, const int *counts,
                                const long long *off, const double *pack, int grid, cudaStream_t s) {
  dev::batch_unpack_kernel<<<grid, kVertexTile, 0, s>>>(jobs, vtiles, counts, off, pack);
  return cudaGetLastError();
}

cudaError_t launch_batch_pack(const BatchJob *jobs, const BatchTile *vtiles, const int *counts, const long long *off,
                              double *pack, double *E, int grid, cudaStream_t s) {
  dev::batch_pack_kernel<<<grid, kVertexTile, 0, s>>>(jobs, vtiles, counts, off, pack, E);
  return cudaGetLastError();
}

}  // namespace umcp

namespace umcp {

cudaError_t launch_geo_sums(const GeoArgs &G, bool alpha64, cudaStream_t s) {
  if (alpha64) return launch_after(dev::geo_sums_kernel, geo_blocks(G.nfaces), kGeoThreads, 0, s, G);
  // the thread-per-face form: a grid that depends on the face count only (the sums' order is fixed)
  const cudaError_t e = cudaFuncSetAttribute(dev::geo_sums_ff_tpf_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)dev::geo_tpf::kDynBytes);
  if (e != cudaSuccess) return e;
  const int per_block = dev::geo_tpf::kThreads, want = (G.nfaces + per_block - 1) / per_block;
  const int grid = want < 1 ? 1 : (want < geo_blocks(G.nfaces) ? want : geo_blocks(G.nfaces));
  return launch_after(dev::geo_sums_ff_tpf_kernel, grid, dev::geo_tpf::kThreads, dev::geo_tpf::kDynBytes, s, G);
}

template <typename T>
cudaError_t launch_geo_grad(const GeoArgs &G, T *partial, cudaStream_t s) {
  if (G.nfaces <= 0) return cudaSuccess;
  return launch_after(dev::geo_grad_kernel<T>, geo_blocks(G.nfaces), kGeoThreads, 0, s, G, partial);
}
template cudaError_t launch_geo_grad<double>(const GeoArgs &, double *, cudaStream_t);
template cudaError_t launch_geo_grad<float>(const GeoArgs &, float *, cudaStream_t);

}  // namespace umcp

namespace umcp {

int face_blocks_tc(int nfaces) {
  const int tiles = (nfaces + dev::tc::kFaces - 1) / dev::tc::kFaces;
  const int cap = 2 * sm_count();  // two CTAs per SM (shared memory and tensor memory)
  return tiles < 1 ? 1 : (tiles < cap ? tiles : cap);
}

cudaError_t launch_faces_tc(const dev::FaceLaunch &L, const int *dest, const dev::SurfaceParams &P, const double *r,
                            const float *rhi, const float *rlo, const float *dsp, float *partial, double *blockpart,
                            int *status, int grid, const FinishArgs &fin, cudaStream_t s) {
  if (!dsp) return cudaErrorInvalidValue;
  const cudaError_t e = tc_opt_in();
  if (e != cudaSuccess) return e;
  dev::face_tc_kernel<<<grid, dev::tc::kThreads, dev::tc::kSmemBytes, s>>>(L, dest, P, r, rhi, rlo, dsp, partial,
                                                                           blockpart, status, fin);
  return cudaGetLastError();
}

}  // namespace umcp
