// Plan builder: basis rows, irregular-patch tables and reference state.
#include "plan.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <sstream>

#include "philox.h"

namespace umcp {

// ------------------------------------------------------------ box splines
//
// Stam's twelve quartic box-spline basis functions of a regular Loop patch,
// written in barycentric monomials u^a v^b w^c (w = 1-u-v), each divided by
// 12. The table is the published basis as the reference states it
// (src/interpLib.C:5845-5856, n1..n12); derivatives are taken analytically
// here rather than from expanded polynomials.
namespace {
struct Term { int coef, a, b, c; };
const std::vector<Term> kSpline[13] = {
    {},
    /*n1*/ {{1, 4, 0, 0}, {2, 3, 1, 0}},
    /*n2*/ {{1, 4, 0, 0}, {2, 3, 0, 1}},
    /*n3*/ {{1, 4, 0, 0}, {2, 3, 0, 1}, {6, 3, 1, 0}, {6, 2, 1, 1}, {12, 2, 2, 0}, {6, 1, 2, 1}, {6, 1, 3, 0}, {2, 0, 3, 1}, {1, 0, 4, 0}},
    /*n4*/ {{6, 4, 0, 0}, {24, 3, 0, 1}, {24, 2, 0, 2}, {8, 1, 0, 3}, {1, 0, 0, 4}, {24, 3, 1, 0}, {60, 2, 1, 1}, {36, 1, 1, 2},
            {6, 0, 1, 3}, {24, 2, 2, 0}, {36, 1, 2, 1}, {12, 0, 2, 2}, {8, 1, 3, 0}, {6, 0, 3, 1}, {1, 0, 4, 0}},
    /*n5*/ {{1, 4, 0, 0}, {6, 3, 0, 1}, {12, 2, 0, 2}, {6, 1, 0, 3}, {1, 0, 0, 4}, {2, 3, 1, 0}, {6, 2, 1, 1}, {6, 1, 1, 2}, {2, 0, 1, 3}},
    /*n6*/ {{2, 1, 3, 0}, {1, 0, 4, 0}},
    /*n7*/ {{1, 4, 0, 0}, {6, 3, 0, 1}, {12, 2, 0, 2}, {6, 1, 0, 3}, {1, 0, 0, 4}, {8, 3, 1, 0}, {36, 2, 1, 1}, {36, 1, 1, 2},
            {8, 0, 1, 3}, {24, 2, 2, 0}, {60, 1, 2, 1}, {24, 0, 2, 2}, {24, 1, 3, 0}, {24, 0, 3, 1}, {6, 0, 4, 0}},
    /*n8*/ {{1, 4, 0, 0}, {8, 3, 0, 1}, {24, 2, 0, 2}, {24, 1, 0, 3}, {6, 0, 0, 4}, {6, 3, 1, 0}, {36, 2, 1, 1}, {60, 1, 1, 2},
            {24, 0, 1, 3}, {12, 2, 2, 0}, {36, 1, 2, 1}, {24, 0, 2, 2}, {6, 1, 3, 0}, {8, 0, 3, 1}, {1, 0, 4, 0}},
    /*n9*/ {{2, 1, 0, 3}, {1, 0, 0, 4}},
    /*n10*/ {{2, 0, 3, 1}, {1, 0, 4, 0}},
    /*n11*/ {{2, 1, 0, 3}, {1, 0, 0, 4}, {6, 1, 1, 2}, {6, 0, 1, 3}, {6, 1, 2, 1}, {12, 0, 2, 2}, {2, 1, 3, 0}, {6, 0, 3, 1}, {1, 0, 4, 0}},
    /*n12*/ {{1, 0, 0, 4}, {2, 0, 1, 3}},
};
// Control point x of the reference's point_list uses spline n_perm[x]
// (ceff_map = {n8,n7,n4,n5,n9,n12,n11,n10,n6,n3,n1,n2}).
const int kPerm[12] = {8, 7, 4, 5, 9, 12, 11, 10, 6, 3, 1, 2};

double ipow(double x, int n) {
  double r = 1.0;
  for (int i = 0; i < n; ++i) r *= x;
  return r;
}

// d^(du+dv)/du^du dv^dv of u^a v^b w^c with w = 1-u-v.
double monomial_deriv(double u, double v, int a, int b, int c, int du, int dv) {
  if (a < 0 || b < 0 || c < 0) return 0.0;
  if (du > 0) {
    double s = 0.0;
    if (a > 0) s += a * monomial_deriv(u, v, a - 1, b, c, du - 1, dv);
    if (c > 0) s -= c * monomial_deriv(u, v, a, b, c - 1, du - 1, dv);
    return s;
  }
  if (dv > 0) {
    double s = 0.0;
    if (b > 0) s += b * monomial_deriv(u, v, a, b - 1, c, 0, dv - 1);
    if (c > 0) s -= c * monomial_deriv(u, v, a, b, c - 1, 0, dv - 1);
    return s;
  }
  return ipow(u, a) * ipow(v, b) * ipow(1.0 - u - v, c);
}
}  // namespace

void box_spline_rows(double u, double v, double out[kKinds][12]) {
  static const int kd[kKinds][2] = {{0, 0}, {1, 0}, {0, 1}, {2, 0}, {1, 1}, {0, 2}};
  for (int kind = 0; kind < kKinds; ++kind)
    for (int x = 0; x < 12; ++x) {
      double s = 0.0;
      for (const Term &t : kSpline[kPerm[x]]) s += t.coef * monomial_deriv(u, v, t.a, t.b, t.c, kd[kind][0], kd[kind][1]);
      out[kind][x] = s / 12.0;
    }
}

void box_spline_values(double u, double v, double out[12]) {
  const double w = 1.0 - u - v;
  double pu[5] = {1, 0, 0, 0, 0}, pv[5] = {1, 0, 0, 0, 0}, pw[5] = {1, 0, 0, 0, 0};
  for (int k = 1; k < 5; ++k) {
    pu[k] = pu[k - 1] * u;
    pv[k] = pv[k - 1] * v;
    pw[k] = pw[k - 1] * w;
  }
  for (int x = 0; x < 12; ++x) {
    double s = 0.0;
    for (const Term &t : kSpline[kPerm[x]]) s += t.coef * (pu[t.a] * pv[t.b] * pw[t.c]);
    out[x] = s / 12.0;
  }
}

// ------------------------------------------------------------ quadrature

double irregular_k(int valence) {
  // Subdominant-eigenvalue parameter per valence (src/interpLib.C:5560-5570).
  static const double kv[11] = {0, 0, 0, 0, 0.375, 4.52254248593737e-01, 0.5, 5.30872450464684e-01,
                                5.51776695296637e-01, 5.66511110779745e-01, 5.77254248593736e-01};
  return (valence >= 4 && valence <= 10) ? kv[valence] : 0.0;
}

namespace {
constexpr int kGL = 16;
struct GaussLegendre {
  double x[kGL], w[kGL];
  GaussLegendre() {
    for (int i = 0; i < kGL; ++i) {
      double z = std::cos(M_PI * (i + 0.75) / (kGL + 0.5)), dp = 1.0;
      for (int it = 0; it < 100; ++it) {
        double p0 = 1.0, p1 = z;
        for (int n = 2; n <= kGL; ++n) {
          double p2 = ((2.0 * n - 1.0) * z * p1 - (n - 1.0) * p0) / n;
          p0 = p1;
          p1 = p2;
        }
        dp = kGL * (z * p1 - p0) / (z * z - 1.0);
        double dz = p1 / dp;
        z -= dz;
        if (std::fabs(dz) < 1e-16) break;
      }
      double p0 = 1.0, p1 = z;
      for (int n = 2; n <= kGL; ++n) {
        double p2 = ((2.0 * n - 1.0) * z * p1 - (n - 1.0) * p0) / n;
        p0 = p1;
        p1 = p2;
      }
      dp = kGL * (z * p1 - p0) / (z * z - 1.0);
      x[i] = z;
      w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
  }
};
const GaussLegendre &gl() {
  static GaussLegendre g;
  return g;
}

// Integral of f over [lo,hi] split geometrically toward lo_sing (the point
// where the weight is singular): pieces [s + (hi-s)2^-(m+1), s + (hi-s)2^-m].
template <class F>
double graded_integral(F f, double lo, double hi, double sing) {
  const GaussLegendre &g = gl();
  double total = 0.0;
  double span = hi - sing;
  for (int m = 0; m < 400; ++m) {
    double b = sing + span * std::ldexp(1.0, -m), a = sing + span * std::ldexp(1.0, -(m + 1));
    bool last = false;
    if (a <= lo) { a = lo; last = true; }
    if (b <= a) break;
    double c = 0.5 * (a + b), h = 0.5 * (b - a), s = 0.0;
    for (int i = 0; i < kGL; ++i) s += g.w[i] * f(c + h * g.x[i]);
    total += s * h;
    if (last) break;
  }
  return total;
}

// Orthogonal-polynomial recurrence -> Jacobi matrix -> nodes/weights
// (Stieltjes procedure + Golub-Welsch, as src/gauss.C:96-306 does).
template <class Inner>
void gauss_from_inner(int n, Inner inner, double *x, double *w) {
  std::vector<double> a(n + 1, 0.0), b(n + 1, 0.0);
  double prev = 1.0, mu0 = 0.0;
  for (int i = 0; i <= n; ++i) {
    auto poly = [&](double t) {
      double pm1 = 0.0, p = 1.0;
      for (int q = 0; q < i; ++q) {
        double nx = (t - a[q]) * p - b[q] * pm1;
        pm1 = p;
        p = nx;
      }
      return p;
    };
    double num = inner([&](double t) { double p = poly(t); return t * p * p; });
    double den = inner([&](double t) { double p = poly(t); return p * p; });
    a[i] = num / den;
    b[i] = (i > 0) ? den / prev : 0.0;
    if (i == 0) mu0 = den;
    prev = den;
  }
  // Symmetric tridiagonal eigenproblem by cyclic Jacobi rotations.
  std::vector<double> J(n * n, 0.0), V(n * n, 0.0);
  for (int i = 0; i < n; ++i) {
    J[i * n + i] = a[i];
    V[i * n + i] = 1.0;
    if (i > 0) J[(i - 1) * n + i] = J[i * n + i - 1] = std::sqrt(b[i]);
  }
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += J[p * n + q] * J[p * n + q];
    if (off < 1e-40) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = J[p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        double theta = (J[q * n + q] - J[p * n + p]) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  // J <- J R
          double jkp = J[k * n + p], jkq = J[k * n + q];
          J[k * n + p] = c * jkp - s * jkq;
          J[k * n + q] = s * jkp + c * jkq;
        }
        for (int k = 0; k < n; ++k) {  // J <- R^T J
          double jpk = J[p * n + k], jqk = J[q * n + k];
          J[p * n + k] = c * jpk - s * jqk;
          J[q * n + k] = s * jpk + c * jqk;
        }
        for (int k = 0; k < n; ++k) {  // V <- V R
          double vkp = V[k * n + p], vkq = V[k * n + q];
          V[k * n + p] = c * vkp - s * vkq;
          V[k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<std::pair<double, double>> nw(n);
  for (int i = 0; i < n; ++i) {
    double nrm = 0.0;
    for (int k = 0; k < n; ++k) nrm += V[k * n + i] * V[k * n + i];
    nw[i] = {J[i * n + i], mu0 * V[i] * V[i] / nrm};
  }
  std::sort(nw.begin(), nw.end());
  for (int i = 0; i < n; ++i) { x[i] = nw[i].first; w[i] = nw[i].second; }
}
}  // namespace

void irregular_gauss_v(int n, double k, double *x, double *w) {
  // Weight on [0,1]: (1 - v^(p+1))/(p+1), p = 4(1 + log2 k) (eval_fn_v, src/gauss.C:63-94).
  double p1 = 5.0 + 4.0 * std::log2(k);
  auto weight = [p1](double v) { return (1.0 - std::pow(v, p1)) / p1; };
  auto inner = [&](auto g) { return graded_integral([&](double v) { return g(v) * weight(v); }, 0.0, 1.0, 0.0); };
  gauss_from_inner(n, inner, x, w);
}

void irregular_gauss_u(int n, double k, double v, double *x, double *w) {
  // Weight on [0,1-v]: (u+v)^p (eval_fn, src/gauss.C:27-61), singular at u = -v.
  double p = 4.0 * (1.0 + std::log2(k));
  auto inner = [&](auto g) {
    return graded_integral([&](double u) { return g(u) * std::pow(u + v, p); }, 0.0, 1.0 - v, -v);
  };
  gauss_from_inner(n, inner, x, w);
}

// ------------------------------------------------------------ patch bases

void build_regular_basis(PatchBasis *b) {
  static const double pts[kRegPts][2] = {{0.1, 0.1}, {0.3, 0.1}, {0.5, 0.1}, {0.7, 0.1}, {0.9, 0.1},
                                         {0.1, 0.3}, {0.3, 0.3}, {0.5, 0.3}, {0.7, 0.3}, {0.1, 0.5},
                                         {0.3, 0.5}, {0.5, 0.5}, {0.1, 0.7}, {0.3, 0.7}, {0.1, 0.9}};
  b->valence = 6;
  b->ncp = 12;
  b->npt = kRegPts;
  b->row.assign((size_t)kKinds * kRegPts * 12, 0.0);
  b->weight.assign(kRegPts, 1.0 / 15);
  b->u.resize(kRegPts);
  b->v.resize(kRegPts);
  for (int p = 0; p < kRegPts; ++p) {
    double s[kKinds][12];
    box_spline_rows(pts[p][0], pts[p][1], s);
    b->u[p] = pts[p][0];
    b->v[p] = pts[p][1];
    for (int kind = 0; kind < kKinds; ++kind)
      for (int x = 0; x < 12; ++x) b->row[((size_t)kind * kRegPts + p) * 12 + x] = s[kind][x];
  }
}

// Subdivision matrix on the extended one-ring of an irregular vertex
// (rows: the val+12 child points, columns: the val+6 parent points), with
// the labelling of src/interpLib.C:5011-5161.
static std::vector<double> subdivision_matrix(int val) {
  const int N = val + 6, R = val + 12;
  std::vector<double> A((size_t)R * N, 0.0);
  auto set = [&](int r, int c, double x) { A[(size_t)r * N + c] = x; };
  const double w = 3.0 / (8.0 * val), w6 = 3.0 / 48.0, e3 = 3.0 / 8.0, e1 = 1.0 / 8.0;
  set(0, 0, 1.0 - val * w);
  for (int p = 1; p <= val; ++p) set(0, p, w);
  for (int p = 1; p <= val; ++p) {  // edge points around the irregular vertex
    int prev = (p == 1) ? val : p - 1, next = (p == val) ? 1 : p + 1;
    set(p, 0, e3); set(p, p, e3); set(p, prev, e1); set(p, next, e1);
  }
  set(val + 1, 1, e3); set(val + 1, val, e3); set(val + 1, 0, e1); set(val + 1, val + 1, e1);
  set(val + 2, 1, 1.0 - 6 * w6);
  for (int c : {0, val, val + 1, val + 2, val + 3, 2}) set(val + 2, c, w6);
  set(val + 3, 1, e3); set(val + 3, 2, e3); set(val + 3, 0, e1); set(val + 3, val + 3, e1);
  set(val + 4, 2, 1.0 - 6 * w6);
  for (int c : {0, 1, val + 3, val + 4, val + 5, 3}) set(val + 4, c, w6);
  set(val + 5, 2, e3); set(val + 5, 3, e3); set(val + 5, 0, e1); set(val + 5, val + 5, e1);
  set(val + 6, 1, e3); set(val + 6, val + 1, e3); set(val + 6, val + 2, e1); set(val + 6, val, e1);
  set(val + 7, 1, e3); set(val + 7, val + 2, e3); set(val + 7, val + 3, e1); set(val + 7, val + 1, e1);
  set(val + 8, 1, e3); set(val + 8, val + 3, e3); set(val + 8, 2, e1); set(val + 8, val + 2, e1);
  set(val + 9, 2, e3); set(val + 9, val + 3, e3); set(val + 9, 1, e1); set(val + 9, val + 4, e1);
  set(val + 10, 2, e3); set(val + 10, val + 4, e3); set(val + 10, val + 5, e1); set(val + 10, val + 3, e1);
  set(val + 11, 2, e3); set(val + 11, val + 5, e3); set(val + 11, 3, e1); set(val + 11, val + 4, e1);
  return A;
}

IrregularMap::IrregularMap(int val) : val_(val), n_(val + 6), atot_(subdivision_matrix(val)) {
  powers_.assign(1, std::vector<double>((size_t)n_ * n_, 0.0));
  for (int i = 0; i < n_; ++i) powers_[0][(size_t)i * n_ + i] = 1.0;
}

// Powers of the square block A (the first val+6 rows of Atot), A^0 = I.
const std::vector<double> &IrregularMap::power(int e) {
  const int N = n_;
  while ((int)powers_.size() <= e) {
    const std::vector<double> &P = powers_.back();
    std::vector<double> Q((size_t)N * N, 0.0);
    for (int i = 0; i < N; ++i)
      for (int l = 0; l < N; ++l) {
        double a = atot_[(size_t)i * N + l];
        if (a == 0.0) continue;
        for (int j = 0; j < N; ++j) Q[(size_t)i * N + j] += a * P[(size_t)l * N + j];
      }
    powers_.push_back(Q);
  }
  return powers_[e];
}

void IrregularMap::at(double *u, double *v, double *scale_out, double cmap[12][kMaxCp]) {
  const int val = val_, N = n_;
  double fu = *u, fv = *v;
  // Sub-triangle selection in the domain ring containing (fu,fv)
  // (src/interpLib.C:5648-5730, src/irr_kernel.C:474-541).
  double f_domain = -std::log10(fu + fv) / std::log10(2.0);
  if (fu + fv >= 1.0 - 1e-9) f_domain = 1;
  const int domain = (int)std::lround(std::ceil(f_domain));
  const double pow2 = std::pow(2.0, domain - 1.0);
  double scale = pow2;
  fu *= pow2;
  fv *= pow2;
  int pc[12];
  if (fu > 0.5) {
    fv = 2 * fv; fu = 2.0 * fu - 1.0; scale *= 2;
    int c[12] = {2, val + 3, val + 4, val + 5, 3, 0, 1, val + 2, val + 8, val + 9, val + 10, val + 11};
    std::memcpy(pc, c, sizeof pc);
  } else if (fv > 0.5) {
    fu = 2 * fu; fv = 2.0 * fv - 1.0; scale *= 2;
    int c[12] = {1, val + 2, val + 3, 2, 0, val, val + 1, val + 6, val + 7, val + 8, val + 9, val + 4};
    std::memcpy(pc, c, sizeof pc);
  } else {
    fv = 1 - 2 * fv; fu = 1 - 2 * fu; scale *= -2;
    int c[12] = {val + 3, 2, 1, val + 2, val + 8, val + 9, val + 4, val + 5, 3, 0, val, val + 1};
    std::memcpy(pc, c, sizeof pc);
  }
  const std::vector<double> &Ap = power(domain - 1);
  // cmap[y][x] = (Atot * A^(domain-1))[pc[y]][x]
  for (int y = 0; y < 12; ++y)
    for (int x = 0; x < N; ++x) {
      double s = 0.0;
      for (int l = 0; l < N; ++l) s += atot_[(size_t)pc[y] * N + l] * Ap[(size_t)l * N + x];
      cmap[y][x] = s;
    }
  *u = fu;
  *v = fv;
  *scale_out = scale;
}

std::string build_irregular_basis(int val, PatchBasis *b) {
  if (val != 5 && val != 7) return "irregular valence must be 5 or 7";
  const int N = val + 6;
  const double k = irregular_k(val);
  b->valence = val;
  b->ncp = N;
  b->npt = kIrrPts;
  b->row.assign((size_t)kKinds * kIrrPts * N, 0.0);
  b->weight.assign(kIrrPts, 0.0);
  b->u.assign(kIrrPts, 0.0);
  b->v.assign(kIrrPts, 0.0);
  IrregularMap map(val);

  const int n = 4;
  double vx[n], vw[n];
  irregular_gauss_v(n, k, vx, vw);
  const double p1 = 5.0 + 4.0 * std::log2(k), p = p1 - 1.0;
  int pt = 0;
  for (int iv = 0; iv < n; ++iv) {
    const double fv0 = vx[iv];
    const double v_factor = (1.0 - std::pow(fv0, p1)) / p1;
    const double v_weight = vw[iv] / v_factor;
    double ux[n], uw[n];
    irregular_gauss_u(n, k, fv0, ux, uw);
    for (int iu = 0; iu < n; ++iu, ++pt) {
      double fu = ux[iu], fv = fv0;
      const double u_weight = uw[iu] * std::pow(fu + fv, -p);
      b->weight[pt] = v_weight * u_weight;
      b->u[pt] = fu;
      b->v[pt] = fv;
      double scale, cmap[12][kMaxCp];
      map.at(&fu, &fv, &scale, cmap);
      double sp[kKinds][12];
      box_spline_rows(fu, fv, sp);
      const double ks[kKinds] = {1.0, scale, scale, scale * scale, scale * scale, scale * scale};
      for (int kind = 0; kind < kKinds; ++kind)
        for (int x = 0; x < N; ++x) {
          double s = 0.0;
          for (int y = 0; y < 12; ++y) s += cmap[y][x] * sp[kind][y] * ks[kind];
          b->row[((size_t)kind * kIrrPts + pt) * N + x] = s;
        }
    }
  }
  return "";
}

// ------------------------------------------------------------ subdivision

void subdivision_stencils(double S[4][12][12]) {
  // Refinability of the box splines: the patch over a child triangle is
  // itself a box-spline patch, so its control points C_k = S_k P are the
  // exact least-squares fit of the parent patch on the child. Child frames
  // (origin, u' corner, v' corner) in parent coordinates, in the order the
  // reference numbers its children (src/fast_mm.C fast_sub6_0..3): the corner
  // children share the parent's orientation, the centre one is turned 180
  // degrees.
  static const double frame[4][3][2] = {{{0, 0}, {0.5, 0}, {0, 0.5}},
                                        {{0.5, 0}, {1, 0}, {0.5, 0.5}},
                                        {{0, 0.5}, {0.5, 0.5}, {0, 1}},
                                        {{0.5, 0.5}, {0, 0.5}, {0.5, 0}}};
  const int ns = 28;  // sample points: a triangular grid strictly inside the child
  double sp[ns][2];
  int q = 0;
  for (int i = 1; i <= 7 && q < ns; ++i)
    for (int j = 1; i + j <= 8 && q < ns; ++j) sp[q][0] = i / 9.0, sp[q][1] = j / 9.0, ++q;
  for (int k = 0; k < 4; ++k) {
    const double *P0 = frame[k][0], *P1 = frame[k][1], *P2 = frame[k][2];
    // normal equations (Bc^T Bc) S = Bc^T Bp
    double A[12][12] = {}, R[12][12] = {};
    for (int t = 0; t < q; ++t) {
      double bc[12], bp[12];
      const double a = sp[t][0], b = sp[t][1];
      box_spline_values(a, b, bc);
      box_spline_values(P0[0] + a * (P1[0] - P0[0]) + b * (P2[0] - P0[0]),
                        P0[1] + a * (P1[1] - P0[1]) + b * (P2[1] - P0[1]), bp);
      for (int x = 0; x < 12; ++x)
        for (int y = 0; y < 12; ++y) {
          A[x][y] += bc[x] * bc[y];
          R[x][y] += bc[x] * bp[y];
        }
    }
    // Gauss-Jordan with partial pivoting on [A | R]
    for (int c = 0; c < 12; ++c) {
      int piv = c;
      for (int r = c + 1; r < 12; ++r)
        if (std::fabs(A[r][c]) > std::fabs(A[piv][c])) piv = r;
      for (int y = 0; y < 12; ++y) {
        std::swap(A[c][y], A[piv][y]);
        std::swap(R[c][y], R[piv][y]);
      }
      const double d = A[c][c];
      for (int y = 0; y < 12; ++y) { A[c][y] /= d; R[c][y] /= d; }
      for (int r = 0; r < 12; ++r) {
        if (r == c || A[r][c] == 0.0) continue;
        const double f = A[r][c];
        for (int y = 0; y < 12; ++y) { A[r][y] -= f * A[c][y]; R[r][y] -= f * R[c][y]; }
      }
    }
    // Loop subdivision weights are multiples of 1/16: round the fit to them.
    for (int x = 0; x < 12; ++x)
      for (int y = 0; y < 12; ++y) S[k][x][y] = std::nearbyint(R[x][y] * 16.0) / 16.0;
  }
}

// ------------------------------------------------------------ limit points

int limit_point_coeffs(const Face &f, double u, double v, IrregularMap *maps[8], double *coef) {
  const int N = f.ncp;
  for (int x = 0; x < N; ++x) coef[x] = 0.0;
  if (f.valence == 6) {
    box_spline_values(u, v, coef);
    return N;
  }
  if (!(std::isfinite(-std::log10(u + v))) && u < 1e-10 && v < 1e-10) {
    // The extraordinary vertex itself: half the vertex plus half the mean of
    // its ring (src/uv_map.C:32-61); the ring is control points 1..val.
    coef[0] = 0.5;
    for (int e = 1; e <= f.valence; ++e) coef[e] = 1.0 / (2.0 * f.valence);
    return N;
  }
  double fu = u, fv = v, scale, cmap[12][kMaxCp];
  maps[f.valence]->at(&fu, &fv, &scale, cmap);
  double sp[12];
  box_spline_values(fu, fv, sp);
  for (int x = 0; x < N; ++x) {
    double s = 0.0;
    for (int y = 0; y < 12; ++y) s += cmap[y][x] * sp[y];
    coef[x] = s;
  }
  return N;
}

int limit_point_rows(const Face &f, double u, double v, IrregularMap *maps[8], double *w, double *du, double *dv) {
  const int N = f.ncp;
  for (int x = 0; x < N; ++x) w[x] = du[x] = dv[x] = 0.0;
  double sp[kKinds][12];
  if (f.valence == 6) {
    box_spline_rows(u, v, sp);
    for (int x = 0; x < 12; ++x) { w[x] = sp[0][x]; du[x] = sp[1][x]; dv[x] = sp[2][x]; }
    return N;
  }
  if (!(std::isfinite(-std::log10(u + v))) && u < 1e-10 && v < 1e-10) {
    limit_point_coeffs(f, u, v, maps, w);
    for (int x = 0; x < N; ++x) du[x] = dv[x] = std::nan("");  // no tangent frame at the vertex itself
    return N;
  }
  double fu = u, fv = v, scale, cmap[12][kMaxCp];
  maps[f.valence]->at(&fu, &fv, &scale, cmap);
  box_spline_rows(fu, fv, sp);
  for (int x = 0; x < N; ++x) {
    double a = 0, b = 0, c = 0;
    for (int y = 0; y < 12; ++y) {
      a += cmap[y][x] * sp[0][y];
      b += cmap[y][x] * sp[1][y];
      c += cmap[y][x] * sp[2][y];
    }
    w[x] = a;
    du[x] = scale * b;
    dv[x] = scale * c;
  }
  return N;
}

MassPoints mass_points(const Plan &p, double mass_scale, int plim) {
  // Mass per point (src/hd.C:442-452): a lipid mass of 760.09 g/mol (POPC)
  // times mass_scale, spread over area0 at 65.35 A^2 per lipid and two
  // leaflets. area0 is surface::area's: 0.5 g0 w over the regular faces'
  // points plus g0 w over the irregular ones' (src/interpLib.C:4413-4601).
  double area0 = 0.0;
  for (size_t f = 0; f < p.reg_faces.size(); ++f)
    for (int q = 0; q < kRegPts; ++q) area0 += 0.5 * p.reg_g0[f * kRegPts + q] * p.regular.weight[q];
  for (size_t f = 0; f < p.irr_faces.size(); ++f)
    for (int q = 0; q < kIrrPts; ++q)
      area0 += p.irr_g0[f * kIrrPts + q] * p.irregular[p.irr_faces[f].valence].weight[q];
  const int ppf = (plim + 1) * (plim + 2) / 2;
  const double amu_per_kg = 1.0 / 1.661e-27;
  const double mass_per_lipid = mass_scale * 1000 * 760.09 / 6.022e23 / 1000;
  const size_t nfaces = p.reg_faces.size() + p.irr_faces.size();
  MassPoints out;
  out.area0 = area0;
  out.mass_per_point = amu_per_kg * 2 * area0 / (double)nfaces / ppf * mass_per_lipid / 65.35;
  out.points = (long long)ppf * (long long)nfaces;
  return out;
}

void face_mass_block(int valence, int ncp, int plim, double m, double *B) {
  IrregularMap map5(5), map7(7);
  IrregularMap *maps[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, &map5, nullptr, &map7};
  Face f{};
  f.valence = valence;
  f.ncp = ncp;
  for (int a = 0; a < ncp * ncp; ++a) B[a] = 0.0;
  double c[kMaxCp];
  for (int fi = 0; fi <= plim; ++fi)
    for (int fj = 0; fj <= plim - fi; ++fj) {
      limit_point_coeffs(f, fi / (double)plim, fj / (double)plim, maps, c);
      for (int a = 0; a < ncp; ++a)
        for (int b = 0; b < ncp; ++b) B[a * ncp + b] += c[a] * c[b] * m;
    }
}

// ------------------------------------------------------------ lipids

namespace {
struct BuiltinLipid { const char *name; double c0, apl; };
// Built-in lipid library (src/lipid_composition.C:18-32): name, c0 (1/A), APL (A^2).
const BuiltinLipid kLibrary[] = {
    {"ZERO", 0, 68.3}, {"POPC", -1.0 / 87.3, 68.3}, {"DOPE", -1.0 / 29.4, 63.4}, {"POPE", -1.0 / 29.4, 58.8},
    {"DOPC", -1.0 / 87.3, 69.7}, {"CHOL", -1.0 / 27.2, 31.0}, {"CHL1", -1.0 / 27.2, 31.0}, {"DOG", -1.0 / 11.5, 59.0},
    {"DOPS", 1.0 / 144.0, 71.6}, {"CER180", 0, 59.0}, {"SSM", 0, 59.0}, {"PSM", 0, 59.0}};

bool iequal(const std::string &a, const std::string &b) {
  if (a.size() != b.size()) return false;
  for (size_t i = 0; i < a.size(); ++i)
    if (tolower((unsigned char)a[i]) != tolower((unsigned char)b[i])) return false;
  return true;
}
}  // namespace

std::string parse_lipids(const std::string &text, std::vector<Lipid> *lipids) {
  std::vector<Lipid> lib;
  for (const BuiltinLipid &b : kLibrary) lib.push_back({b.name, b.c0, b.apl, 0, 0});
  std::vector<Lipid> types;
  std::istringstream in(text);
  std::string line;
  std::vector<std::string> rows;
  while (std::getline(in, line)) rows.push_back(line);
  // pass 0: library directives; pass 1: leaflet directives.
  for (int pass = 0; pass < 2; ++pass)
    for (const std::string &row : rows) {
      std::istringstream ls(row);
      std::string w0, cmd, name;
      if (!(ls >> w0) || !iequal(w0, "lipid") || !(ls >> cmd)) continue;
      if (pass == 0 && iequal(cmd, "library")) {
        double apl, c0;
        if (!(ls >> name >> apl >> c0)) return "expected 'lipid library NAME APL c0'";
        bool found = false;
        for (Lipid &l : lib)
          if (iequal(l.name, name)) { l.c0 = c0; l.apl = apl; found = true; }
        if (!found) lib.push_back({name, c0, apl, 0, 0});
      } else if (pass == 1 && (iequal(cmd, "inner") || iequal(cmd, "outer"))) {
        double parts;
        if (!(ls >> name >> parts)) return "expected 'lipid inner|outer NAME parts'";
        const Lipid *src = nullptr;
        for (const Lipid &l : lib)
          if (iequal(l.name, name)) src = &l;
        if (!src) return "lipid '" + name + "' is not in the library";
        Lipid *t = nullptr;
        for (Lipid &l : types)
          if (iequal(l.name, name)) t = &l;
        if (!t) { types.push_back({src->name, src->c0, src->apl, 0, 0}); t = &types.back(); }
        if (iequal(cmd, "inner")) t->inner_parts += parts; else t->outer_parts += parts;
      }
    }
  if (types.empty()) types.push_back({kLibrary[0].name, kLibrary[0].c0, kLibrary[0].apl, 0, 0});
  double po = 0, pi = 0;
  for (const Lipid &t : types) { po += t.outer_parts; pi += t.inner_parts; }
  if (po == 0) types[0].outer_parts = 1;
  if (pi == 0) types[0].inner_parts = 1;
  *lipids = types;
  return "";
}

void composition_coeffs(const double *outer, const double *inner, const std::vector<Lipid> &lipids,
                        double *P2, double *Hbar, double *Pres) {
  double so = 0, si = 0, soc = 0, sic = 0;
  for (size_t x = 0; x < lipids.size(); ++x) {
    so += outer[x]; si += inner[x];
    soc += outer[x] * lipids[x].c0; sic += inner[x] * lipids[x].c0;
  }
  double p2 = so + si;
  double hb = (p2 > 0) ? (soc - sic) / p2 : 0.0;
  double res = 0.0;
  for (size_t x = 0; x < lipids.size(); ++x) {
    double d_o = lipids[x].c0 - hb, d_i = lipids[x].c0 + hb;
    res += outer[x] * d_o * d_o + inner[x] * d_i * d_i;
  }
  *P2 = p2; *Hbar = hb; *Pres = res;
}

// ------------------------------------------------------------ reference state

// Whole-lipid fill of one face's leaflets until each exceeds the face area less
// half an average lipid (src/interpLib.C:3124-3195). With one lipid type per
// leaflet the fill is deterministic; with mixtures the type of each added
// lipid is drawn from a Philox stream keyed by the face (the reference's
// draws come from the C library rand()).
static void fill_face(double area, const std::vector<Lipid> &lipids, uint64_t face_key, double *outer, double *inner) {
  const size_t nt = lipids.size();
  std::vector<double> fo(nt), fi(nt);
  double so = 0, si = 0;
  for (size_t x = 0; x < nt; ++x) { fo[x] = lipids[x].outer_parts; fi[x] = lipids[x].inner_parts; so += fo[x]; si += fi[x]; }
  for (size_t x = 0; x < nt; ++x) { fo[x] /= so; fi[x] /= si; }
  for (size_t x = 1; x < nt; ++x) { fo[x] += fo[x - 1]; fi[x] += fi[x - 1]; }
  for (size_t x = 0; x < nt; ++x) outer[x] = inner[x] = 0.0;
  double ai = 0, ao = 0;
  const double half_lipid = 0.5 * 65.0;
  for (uint32_t draw = 0;; ++draw) {
    bool idone = (ai > 0 && ai > area - half_lipid), odone = (ao > 0 && ao > area - half_lipid);
    if (idone && odone) break;
    philox_out o = philox4x32_10((uint32_t)face_key, (uint32_t)(face_key >> 32), draw, 0x6c697064u, 0x1234u, 0x5678u);
    double rn_i = (nt > 1) ? philox_u53(o.v[0], o.v[1]) : 0.0, rn_o = (nt > 1) ? philox_u53(o.v[2], o.v[3]) : 0.0;
    for (size_t x = 0; x < nt; ++x) {
      if (rn_i < fi[x] && !idone) { inner[x] += lipids[x].apl; idone = true; ai += lipids[x].apl; }
      if (rn_o < fo[x] && !odone) { outer[x] += lipids[x].apl; odone = true; ao += lipids[x].apl; }
    }
  }
}

template <class FaceList>
static void reference_points(const Mesh &m, const double *r, const FaceList &faces, const PatchBasis *bases,
                             bool regular, std::vector<double> *g0, std::vector<double> *rr0,
                             std::vector<double> *area) {
  const int npt = regular ? kRegPts : kIrrPts;
  g0->assign(faces.size() * npt, 0.0);
  rr0->assign(faces.size() * npt, 0.0);
  area->assign(faces.size(), 0.0);
  for (size_t f = 0; f < faces.size(); ++f) {
    const Face &F = faces[f];
    const PatchBasis &B = regular ? bases[0] : bases[F.valence];
    double X[kMaxCp][3];
    for (int x = 0; x < F.ncp; ++x)
      for (int c = 0; c < 3; ++c)
        X[x][c] = r[3 * F.cp[x] + c] + F.img[x][0] * m.box[0][c] + F.img[x][1] * m.box[1][c] + F.img[x][2] * m.box[2][c];
    double A = 0.0;
    for (int p = 0; p < npt; ++p) {
      double Ru[3] = {0, 0, 0}, Rv[3] = {0, 0, 0};
      for (int x = 0; x < F.ncp; ++x)
        for (int c = 0; c < 3; ++c) {
          Ru[c] += B.at(1, p, x) * X[x][c];
          Rv[c] += B.at(2, p, x) * X[x][c];
        }
      double uu = Ru[0] * Ru[0] + Ru[1] * Ru[1] + Ru[2] * Ru[2];
      double uv = Ru[0] * Rv[0] + Ru[1] * Rv[1] + Ru[2] * Rv[2];
      double vv = Rv[0] * Rv[0] + Rv[1] * Rv[1] + Rv[2] * Rv[2];
      double g = std::sqrt(uu * vv - uv * uv);
      (*g0)[f * npt + p] = g;
      (*rr0)[f * npt + p] = uv / std::sqrt(uu * vv);
      A += g * (regular ? 0.5 : 1.0) * B.weight[p];
    }
    (*area)[f] = A;
  }
}

void set_reference_state(const Mesh &m, const double *r, Plan *p) {
  p->ref_r.assign(r, r + 3 * (size_t)m.nv);
  std::vector<double> reg_area, irr_area;
  reference_points(m, r, p->reg_faces, &p->regular, true, &p->reg_g0, &p->reg_RuRv0, &reg_area);
  reference_points(m, r, p->irr_faces, p->irregular, false, &p->irr_g0, &p->irr_RuRv0, &irr_area);
  const int nt = p->ntypes;
  p->reg_outer.assign(p->reg_faces.size() * nt, 0.0);
  p->reg_inner.assign(p->reg_faces.size() * nt, 0.0);
  p->irr_outer.assign(p->irr_faces.size() * nt, 0.0);
  p->irr_inner.assign(p->irr_faces.size() * nt, 0.0);
  for (size_t f = 0; f < p->reg_faces.size(); ++f)
    fill_face(reg_area[f], p->lipids, f, &p->reg_outer[f * nt], &p->reg_inner[f * nt]);
  for (size_t f = 0; f < p->irr_faces.size(); ++f)
    fill_face(irr_area[f], p->lipids, (1ull << 40) + f, &p->irr_outer[f * nt], &p->irr_inner[f * nt]);
}

std::string build_plan(const Mesh &m, const std::vector<Lipid> &lipids, Plan *p) {
  *p = Plan();
  std::string err = enumerate_faces(m, &p->reg_faces, &p->irr_faces);
  if (!err.empty()) return err;
  build_regular_basis(&p->regular);
  for (const Face &f : p->irr_faces)
    if (p->irregular[f.valence].row.empty()) {
      err = build_irregular_basis(f.valence, &p->irregular[f.valence]);
      if (!err.empty()) return err;
    }
  p->lipids = lipids.empty() ? std::vector<Lipid>{{"ZERO", 0.0, 68.3, 1, 1}} : lipids;
  p->ntypes = (int)p->lipids.size();
  set_reference_state(m, m.r.data(), p);
  return "";
}

}  // namespace umcp
