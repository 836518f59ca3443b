// Device kernels of the membrane-surface hot path (sm_103a).
//
// face_tpf_kernel one thread per regular face (precision form): control
//                 points in thread-private shared memory, basis rows as
//                 warp-wide broadcasts, gradient sums in registers.
// face_kernel     one half-warp per face (FP64, and irregular faces): lanes
//                 are quadrature points while the five basis contractions,
//                 the pointwise energy and adjoint, and each point's
//                 contribution to every control point are formed; then lanes
//                 are control points while those contributions are summed.
//                 Both write per-face gradient partials and per-block energy
//                 sums; no float atomics.
// gather_kernel   per vertex, sums its face partials in a fixed order
//                 (slots interleaved by groups of 32 vertices), optionally
//                 fused with an integrator update.
// finish_kernel   fixed-order sum of the block partials.
//
// The energy model is the reference's surface::fenergy/ifenergy with
// FIXED_A and LOCAL_LIPID_ENERGY (src/interpLib.C:3426-3881); the gradient
// is its exact derivative (src/grad.C:65-942, 6445-7457), written here in
// closed form: with m = Ru x Rv, W = |m|^2, l = m.Suu, k = m.Suv, n = m.Svv,
//   H = c1 + c2 = -(l Rv.Rv - 2 k Ru.Rv + n Ru.Ru) / W^(3/2)
//   K = c1 c2   = (l n - k^2) / W^2 - SAFETY/4
// which the reference reaches through the shape-operator eigenvalues.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace umcp {
namespace dev {

constexpr int kMaxCpDev = 13;   // control points of the largest patch (valence 7 + 6)
constexpr int kVertexBits = 27;  // packed control point: vertex | image_code << 27
constexpr uint32_t kVertexMask = (1u << kVertexBits) - 1u;
constexpr double kSafety = 1e-12;  // SAFETY, src/interp.h:14

struct SurfaceParams {
  double kc, KA, kg, k_reg;
  double box[3][3];
  float box_hi[3][3], box_lo[3][3];  // box = hi + lo, for the precision form
  int nv;
};

// Per-mesh view for a face launch.
struct FaceLaunch {
  int nfaces;              // faces in this launch
  int block_base;          // first block-partial row of this launch
  const uint32_t *cp;      // [nfaces][ncp] packed control points
  const double *g0;        // [nfaces][npt] (plain path)
  const double *rr0;       // [nfaces][npt]
  const double *comp;      // [nfaces][3]: P2, Hbar, Pres
  const float *g0f, *rr0f, *compf;  // the same in FP32 (precision form)
  const double *basis;     // [npt][5][ncp rounded up to 4] rows u,v,uu,uv,vv (staged to shared)
  const double *weight;    // [npt]
  double dudv;
  int irregular;
};

// FP64 uses half the threads per block so its shared memory stays below the
// 48 KB static limit.
template <typename T>
struct FaceCfg {
  static constexpr int threads = (sizeof(T) == 8) ? 64 : 128;
  static constexpr int half_warps = threads / 16;
  static constexpr int min_blocks = (sizeof(T) == 8) ? 6 : 4;  // caps registers near 128 (FP32) / 168 (FP64)
};

// Where one face group's data and its mesh's state live.
struct FaceSrc {
  const uint32_t *cp;
  const double *g0, *rr0, *comp;
  const float *g0f, *rr0f, *compf;
  const int *dest;
  const double *r;
  const float *rhi, *rlo;
  const float *dsp;  // precision form: r - r0 per coordinate (displacement from the reference state)
  int nfaces;
};

template <typename T>
struct Vec3 {
  T x, y, z;
};
template <typename T>
__device__ __forceinline__ Vec3<T> cross(const Vec3<T> &a, const Vec3<T> &b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename T>
__device__ __forceinline__ T dot(const Vec3<T> &a, const Vec3<T> &b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}

// FP32 reciprocals for the pointwise step: the hardware estimates refined by
// one Newton step (y <- y (3 - x y^2) / 2 for 1/sqrt(x), y <- y (2 - x y) for
// 1/x), about 1 ulp, instead of the longer correctly rounded sequences.
__device__ __forceinline__ float rsqrt_nr(float x) {
  const float y = rsqrtf(x);
  return y * (1.5f - 0.5f * x * y * y);
}
__device__ __forceinline__ float rcp_nr(float x) {
  const float y = __fdividef(1.f, x);
  return y * (2.f - x * y);
}
// a / b: a division in FP64; a times the reciprocal ib already formed in FP32
__device__ __forceinline__ double qdiv(double a, double b, double) { return a / b; }
__device__ __forceinline__ float qdiv(float a, float, float ib) { return a * ib; }

// Pointwise energy and adjoint at one quadrature point. Returns energy parts
// (area, curvature, angle) and writes dE/d{Ru,Rv,Suu,Suv,Svv} into Kb, and
// the angle-term part of dE/d{Ru,Rv} into Kreg (needed only for the box-scale
// derivative on irregular faces, src/grad.C:7414-7421).
// KG_REG = false: the caller has kg == 0 and k_reg == 0, and the Gaussian
// curvature and angle terms (zeros then) are left out; results agree with the
// full form's to rounding (the compiler may fuse a product and sum that the
// full form keeps apart).
// dR (precision form): {Ru - Ru0, Rv - Rv0}, the tangents' change from the
// reference state, contracted from the control points' displacements. The
// area strain g - g0 is then formed without cancellation:
//   dm = m - m0 = (Ru - Ru0) x Rv0 + Ru x (Rv - Rv0),  W - W0 = dm . (2 m - dm),
//   g - g0 = (W - W0) / (g + g0)
// (exactly zero at the reference state). Subtracting g0 from an FP32 g would
// leave every tangent's rounding in the strain: at and near the reference
// state that rounding is the whole area force, on coarse patches up to 1e-5
// of the gradient.
// lkn, mo (optional): the scalars lb, kb, nb and the normal m with
// Kb[2] = lb m, Kb[3] = kb m, Kb[4] = nb m, for a caller that contracts the
// three second-derivative rows as one scalar per control point times m
// (inlined: the Kb[2..4] it does not read are never formed).
template <typename T, bool KG_REG = true>
__device__ __forceinline__ void point_adjoint(const Vec3<T> K[5], T w, T g0, T rr0, T dudv, T P2, T Hbar, T Pres,
                                              T kc, T KA, T kg, T k_reg, T *ea, T *ec, T *er, Vec3<T> Kb[5],
                                              Vec3<T> Kreg[2], const Vec3<T> *dR = nullptr, T *lkn = nullptr,
                                              Vec3<T> *mo = nullptr) {
  const Vec3<T> &Ru = K[0], &Rv = K[1], &Suu = K[2], &Suv = K[3], &Svv = K[4];
  Vec3<T> m = cross(Ru, Rv);
  T W = dot(m, m);
  T E11 = dot(Ru, Ru), E12 = dot(Ru, Rv), E22 = dot(Rv, Rv);
  T l = dot(m, Suu), k = dot(m, Suv), n = dot(m, Svv);
  // g = sqrt(W), 1/W, W^-3/2, sqrt(E11 E22) and the reciprocals of g, g0,
  // sqrt(E11 E22), E11, E22 (FP32: from two reciprocal square roots and one
  // reciprocal; FP64: divisions, ib unused)
  T g, iW, ig3, sEE = 0, ig = 0, ig0 = 0, isEE = 0, iE11 = 0, iE22 = 0;
  if constexpr (sizeof(T) == 4) {
    ig = rsqrt_nr(W);
    g = W * ig;
    iW = ig * ig;
    ig3 = iW * ig;
    if constexpr (KG_REG) {
      isEE = rsqrt_nr(E11 * E22);
      sEE = E11 * E22 * isEE;
      iE11 = E22 * isEE * isEE;
      iE22 = E11 * isEE * isEE;
    }
    ig0 = rcp_nr(g0);
  } else {
    g = sqrt(W);
    iW = T(1) / W;
    ig3 = iW / g;  // W^-3/2
    sEE = sqrt(E11 * E22);
  }
  T Tt = l * E22 - T(2) * k * E12 + n * E11;
  T H = -Tt * ig3;
  T dH = H - Hbar;
  T dg;
  if (dR) {
    const Vec3<T> &a = dR[0], &b = dR[1];
    const Vec3<T> rv0 = {Rv.x - b.x, Rv.y - b.y, Rv.z - b.z};
    const Vec3<T> c1 = cross(a, rv0), c2 = cross(Ru, b);
    const Vec3<T> dm = {c1.x + c2.x, c1.y + c2.y, c1.z + c2.z};
    const Vec3<T> s = {T(2) * m.x - dm.x, T(2) * m.y - dm.y, T(2) * m.z - dm.z};
    if constexpr (sizeof(T) == 4) dg = dot(dm, s) * rcp_nr(g + g0);
    else dg = dot(dm, s) / (g + g0);
  } else {
    dg = g - g0;
  }
  *ec = T(0.25) * kc * w * (P2 * dH * dH + Pres);
  *ea = qdiv(dudv * w * KA * dg * dg, g0, ig0);
  *er = T(0);
  // adjoints
  T Hb = T(0.5) * kc * w * P2 * dH;
  T gb = qdiv(T(2) * dudv * w * KA * dg, g0, ig0);
  T Tb = -Hb * ig3;
  T Wb = Hb * T(1.5) * Tt * ig3 * iW + qdiv(gb, T(2) * g, T(0.5) * ig);
  T lb = Tb * E22, kb = T(-2) * Tb * E12, nb = Tb * E11;
  T E11b = Tb * n, E12b = T(-2) * Tb * k, E22b = Tb * l;
  T rE11 = 0, rE12 = 0, rE22 = 0;
  if constexpr (KG_REG) {
    // Gaussian curvature (kg) and the angle regulariser (k_reg), in the
    // order the full expressions add them
    T Q = l * n - k * k;
    T Kg = Q * iW * iW - T(kSafety * 0.25);
    T val = qdiv(E12, sEE, isEE);
    T dv = val - rr0;
    *ec = *ec + dudv * g0 * w * kg * Kg;
    *er = k_reg * dv * dv;
    T Kb_ = dudv * g0 * w * kg;
    T vb = T(2) * k_reg * dv;
    T Qb = Kb_ * iW * iW;
    Wb = Hb * T(1.5) * Tt * ig3 * iW - T(2) * Kb_ * Q * iW * iW * iW + qdiv(gb, T(2) * g, T(0.5) * ig);
    lb = Tb * E22 + Qb * n;
    kb = T(-2) * Tb * E12 - T(2) * Qb * k;
    nb = Tb * E11 + Qb * l;
    rE11 = qdiv(T(-0.5) * vb * val, E11, iE11);
    rE12 = qdiv(vb, sEE, isEE);
    rE22 = qdiv(T(-0.5) * vb * val, E22, iE22);
    E11b = Tb * n + rE11;
    E12b = T(-2) * Tb * k + rE12;
    E22b = Tb * l + rE22;
  }
  if (lkn) {
    lkn[0] = lb;
    lkn[1] = kb;
    lkn[2] = nb;
  }
  if (mo) *mo = m;
  Kb[2] = {lb * m.x, lb * m.y, lb * m.z};
  Kb[3] = {kb * m.x, kb * m.y, kb * m.z};
  Kb[4] = {nb * m.x, nb * m.y, nb * m.z};
  Vec3<T> mb = {lb * Suu.x + kb * Suv.x + nb * Svv.x + T(2) * Wb * m.x,
                lb * Suu.y + kb * Suv.y + nb * Svv.y + T(2) * Wb * m.y,
                lb * Suu.z + kb * Suv.z + nb * Svv.z + T(2) * Wb * m.z};
  Vec3<T> a = cross(Rv, mb), b = cross(mb, Ru);
  Kb[0] = {T(2) * E11b * Ru.x + E12b * Rv.x + a.x, T(2) * E11b * Ru.y + E12b * Rv.y + a.y,
           T(2) * E11b * Ru.z + E12b * Rv.z + a.z};
  Kb[1] = {T(2) * E22b * Rv.x + E12b * Ru.x + b.x, T(2) * E22b * Rv.y + E12b * Ru.y + b.y,
           T(2) * E22b * Rv.z + E12b * Ru.z + b.z};
  Kreg[0] = {T(2) * rE11 * Ru.x + rE12 * Rv.x, T(2) * rE11 * Ru.y + rE12 * Rv.y, T(2) * rE11 * Ru.z + rE12 * Rv.z};
  Kreg[1] = {T(2) * rE22 * Rv.x + rE12 * Ru.x, T(2) * rE22 * Rv.y + rE12 * Ru.y, T(2) * rE22 * Rv.z + rE12 * Ru.z};
}

}  // namespace dev
}  // namespace umcp
