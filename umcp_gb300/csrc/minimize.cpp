// Energy minimization of a mesh over its vertex positions: the reference's
// L-BFGS (src/l-bfgs.C) as Simulation::minimize drives it for a membrane
// without particles (src/minimize.C:489-560), on the engine's energy and
// gradient. A caller of the C ABI, as minimize.C is a caller of
// surface::energy / surface::grad.
//
// The reference optimises p = {alpha, r, alpha copy} with the alpha entries'
// gradient set to zero (src/minimize.C:321-333), so alpha never moves and
// its entries add exact zeros to every dot product; the iteration here runs
// over the 3 nv position coordinates alone and is the same iteration. The
// vector algebra (a few dot products and updates per stored pair) runs on
// the host in FP64 in the reference's order, so the iterates follow the
// reference's; each energy and gradient is one evaluation on the device.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/umcp_gpu.h"

namespace umcp {
umcp_status set_error(umcp_status s, const std::string &msg);  // umcp_last_error's text (api.cu)
}
using umcp::set_error;

namespace {

constexpr double kEnergyError = 1e37;  // ENERGY_ERROR, src/l-bfgs.h:3

class Minimizer {
 public:
  Minimizer(umcp_mesh *m, int n, int hist, double max_move, const double *alpha)
      : m_(m), n_(n), hist_(hist), max_move_(max_move), s_((size_t)hist * n), y_((size_t)hist * n), rho_(hist),
        a_(hist), rot_(hist), x_(n), last_x_(n), last_g_(n), q_(n), z_(n), trial_((size_t)n + 3), full_((size_t)n + 3) {
    for (int i = 0; i < hist; ++i) rot_[i] = i;
    memcpy(&trial_[n], alpha, 3 * sizeof(double));
    memcpy(&full_[n], alpha, 3 * sizeof(double));
  }
  std::vector<double> &x() { return x_; }
  int evaluations() const { return evals_; }

  // One iteration (l_bfgs_iteration, src/l-bfgs.C:97-208). Returns 0 when the
  // newest curvature pair vanishes (the reference stops there), -1 on an
  // evaluation error, 1 otherwise.
  int iterate(umcp_status *err) {
    double e0 = 0;
    if ((*err = energy_grad(x_.data(), &e0, q_.data())) != UMCP_OK) return -1;
    // the newest pair goes to the slot the oldest held
    const int newest = rot_[hist_ - 1];
    for (int i = hist_ - 1; i > 0; --i) rot_[i] = rot_[i - 1];
    rot_[0] = newest;
    if (cur_ > 0) {
      double *y = &y_[(size_t)rot_[0] * n_], *s = &s_[(size_t)rot_[0] * n_];
      for (int j = 0; j < n_; ++j) {
        y[j] = q_[j] - last_g_[j];
        s[j] = x_[j] - last_x_[j];
      }
      double dp = 0;
      for (int j = 0; j < n_; ++j) dp += y[j] * s[j];
      if (fabs(dp) < 1e-40) return 0;
      rho_[rot_[0]] = 1.0 / dp;
    }
    last_x_ = x_;
    last_g_ = q_;
    for (int i = 0; i < cur_; ++i) {  // newest to oldest
      const double *s = &s_[(size_t)rot_[i] * n_], *y = &y_[(size_t)rot_[i] * n_];
      double a = 0;
      for (int j = 0; j < n_; ++j) a += s[j] * q_[j];
      a *= rho_[rot_[i]];
      for (int j = 0; j < n_; ++j) q_[j] -= a * y[j];
      a_[rot_[i]] = a;
    }
    double h0 = 1.0;
    if (cur_ > 0) {
      const double *s = &s_[(size_t)rot_[0] * n_], *y = &y_[(size_t)rot_[0] * n_];
      double den = 0, num = 0;
      for (int j = 0; j < n_; ++j) den += y[j] * y[j];
      for (int j = 0; j < n_; ++j) num += y[j] * s[j];
      h0 = num / den;
    }
    for (int j = 0; j < n_; ++j) z_[j] = h0 * q_[j];
    for (int i = cur_ - 1; i >= 0; --i) {  // oldest to newest
      const double *s = &s_[(size_t)rot_[i] * n_], *y = &y_[(size_t)rot_[i] * n_];
      double b = 0;
      for (int j = 0; j < n_; ++j) b += y[j] * z_[j];
      b *= rho_[rot_[i]];
      for (int j = 0; j < n_; ++j) z_[j] += s[j] * (a_[rot_[i]] - b);
    }
    if ((*err = line_search(e0)) != UMCP_OK) return -1;
    cur_ = std::min(cur_ + 1, hist_);
    return 1;
  }

  umcp_status energy_at(const double *x, double *e) {
    memcpy(full_.data(), x, (size_t)n_ * sizeof(double));
    return energy(full_.data(), e);
  }

 private:
  // Energy of a full state; a non-finite energy reads as +infinity (the
  // reference's line search backs off from such steps).
  umcp_status energy(const double *r, double *e) {
    ++evals_;
    umcp_status st = umcp_energy(m_, r, e, nullptr);
    if (st == UMCP_ERR_NONFINITE || !std::isfinite(*e)) {
      *e = HUGE_VAL;
      return UMCP_OK;
    }
    return st;
  }
  umcp_status energy_grad(const double *x, double *e, double *g) {
    ++evals_;
    memcpy(full_.data(), x, (size_t)n_ * sizeof(double));
    std::vector<double> gf((size_t)n_ + 3, 0.0);
    umcp_status st = umcp_energy_grad(m_, full_.data(), e, gf.data());
    if (st != UMCP_OK) return st;
    memcpy(g, gf.data(), (size_t)n_ * sizeof(double));  // alpha's gradient is not used
    return UMCP_OK;
  }
  // E(x - t z)
  umcp_status eval(double t, double *e) {
    for (int j = 0; j < n_; ++j) trial_[j] = x_[j] - z_[j] * t;
    return energy(trial_.data(), e);
  }
  void step(double t) {
    for (int j = 0; j < n_; ++j) x_[j] -= t * z_[j];
  }

  // do_linesearch (src/l-bfgs.C:225-404) along -z from x, E(x) = e0.
  umcp_status line_search(double e0) {
    umcp_status st;
    double max_t = 0.01;
    if (max_move_ > 0) {
      double mm = 0;
      for (int j = 0; j < n_; ++j) mm = std::max(mm, fabs(z_[j]));
      max_t = fabs(max_move_ / mm);
    }
    double t_low = 0, f_low = e0, t_high = max_t, f_high = 0;
    if ((st = eval(t_high, &f_high)) != UMCP_OK) return st;
    if (f_high < f_low) {
      step(t_high);
      return UMCP_OK;
    }
    int iter = 0, n_cat = 300;
    const int n_max = 20;
    if (f_low < kEnergyError) {
      while (f_high >= kEnergyError && iter < n_cat) {
        t_high /= 2;
        if ((st = eval(t_high, &f_high)) != UMCP_OK) return st;
        n_cat++;
      }
      while (f_high < f_low && iter < n_cat) {
        t_high *= 1.5;
        if ((st = eval(t_high, &f_high)) != UMCP_OK) return st;
        n_cat++;
      }
    }
    if (f_high < f_low) {
      step(t_high);
      return UMCP_OK;
    }
    int citer = 0;
    while (f_high < f_low && citer < n_cat) {
      t_high *= 2;
      if ((st = eval(t_high, &f_high)) != UMCP_OK) return st;
      citer++;
    }
    if (t_high > max_t) {
      t_high = max_t;
      if ((st = eval(t_high, &f_high)) != UMCP_OK) return st;
    }
    double t_mid = (t_high + t_low) / 2, f_mid = 0;
    if ((st = eval(t_mid, &f_mid)) != UMCP_OK) return st;
    while (f_mid > f_low && citer < n_cat) {
      t_mid = (t_mid + t_low) / 2;
      if ((st = eval(t_mid, &f_mid)) != UMCP_OK) return st;
      citer++;
    }
    if (f_mid > f_high) return UMCP_OK;  // no bracket: the reference leaves x where it is
    while (iter < n_max) {
      double t_try = (t_mid + t_low) / 2, f_try = 0;
      if ((st = eval(t_try, &f_try)) != UMCP_OK) return st;
      if (f_try < f_mid) {
        t_high = t_mid; f_high = f_mid;
        t_mid = t_try; f_mid = f_try;
      } else {
        t_low = t_try; f_low = f_try;
      }
      t_try = (t_mid + t_high) / 2;
      if ((st = eval(t_try, &f_try)) != UMCP_OK) return st;
      if (f_try < f_mid) {
        t_low = t_mid; f_low = f_mid;
        t_mid = t_try; f_mid = f_try;
      } else {
        t_high = t_try; f_high = f_try;
      }
      iter += 1;
    }
    step(t_mid);
    return UMCP_OK;
  }

  umcp_mesh *m_;
  int n_, hist_;
  double max_move_;
  std::vector<double> s_, y_, rho_, a_;
  std::vector<int> rot_;  // rot_[k]: storage slot of the k-th newest pair
  int cur_ = 0;            // pairs stored
  int evals_ = 0;
  std::vector<double> x_, last_x_, last_g_, q_, z_;
  std::vector<double> trial_, full_;  // positions + alpha (fixed) for evaluations
};

}  // namespace

extern "C" umcp_status umcp_minimize(umcp_mesh *mesh, const umcp_minimize_opts *opts, double *energies,
                                     umcp_minimize_info *info) {
  if (!mesh) return set_error(UMCP_ERR_INVALID, "null mesh");
  umcp_minimize_opts o{100, 0, 1.0};
  if (opts) o = *opts;
  if (o.max_iterations < 0 || o.history < 0) return set_error(UMCP_ERR_INVALID, "negative minimize option");
  umcp_mesh_info mi{};
  umcp_status st = umcp_mesh_info_get(mesh, &mi);
  if (st != UMCP_OK) return st;
  const int nv = mi.nv, n = 3 * nv;
  // the reference stores min(iterations, parameters) pairs; its parameter
  // vector also holds alpha twice (3 nv + 6 entries)
  const int hist = o.history > 0 ? o.history : std::max(1, std::min(o.max_iterations, n + 6));
  std::vector<double> r((size_t)n + 3), p((size_t)n);
  st = umcp_state_get(mesh, r.data(), p.data());
  if (st != UMCP_OK) return st;
  Minimizer mz(mesh, n, hist, o.max_move, &r[n]);
  memcpy(mz.x().data(), r.data(), (size_t)n * sizeof(double));
  // the reference skips the iterations when the initial gradient vanishes
  double e = 0;
  {
    std::vector<double> g((size_t)n + 3, 0.0);
    if ((st = umcp_energy_grad(mesh, r.data(), &e, g.data())) != UMCP_OK) return st;
    double mag = 0;
    for (int j = 0; j < n; ++j) mag += g[j] * g[j];
    if (energies) energies[0] = e;
    if (info) {
      memset(info, 0, sizeof(*info));
      info->energy_initial = e;
    }
    if (!(mag > 1e-20)) o.max_iterations = 0;
  }
  int it = 0;
  for (; it < o.max_iterations; ++it) {
    const int k = mz.iterate(&st);
    if (k < 0) return st;
    if (k == 0) break;
    if ((st = mz.energy_at(mz.x().data(), &e)) != UMCP_OK) return st;
    if (energies) energies[it + 1] = e;
  }
  // the minimized positions become the resident state (alpha unchanged, momenta kept)
  memcpy(r.data(), mz.x().data(), (size_t)n * sizeof(double));
  if ((st = umcp_state_set(mesh, r.data(), p.data())) != UMCP_OK) return st;
  if (info) {
    std::vector<double> g((size_t)n + 3, 0.0);
    double ef = 0;
    if ((st = umcp_energy_grad(mesh, r.data(), &ef, g.data())) != UMCP_OK) return st;
    double ss = 0;
    for (int j = 0; j < n; ++j) ss += g[j] * g[j];
    info->iterations = it;
    info->evaluations = mz.evaluations() + 2;
    info->energy_final = ef;
    info->grad_rms = sqrt(ss / (n > 0 ? n : 1));
  }
  return UMCP_OK;
}
