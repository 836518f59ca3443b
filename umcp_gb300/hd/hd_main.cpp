// hd_gb300: the membrane-only dynamics run of the reference's hd program
// (main in src/hd.C) on the GB300 engine, through the public C ABI.
//
//   hd_gb300 input.inp [key=value ...]
//
// Keywords (src/input.C; case-insensitive, later ones win, command-line
// key=value pairs last):
//   mesh FILE          the .mesh file                      (required)
//   jobname NAME       output prefix (NAME.save)           (default "job")
//   load FILE          restart file to start from          (src/restart.C format)
//   nsteps|nouter N    outer iterations, one t: line each  (default 10000)
//   o_lim|ninner N     steps per outer iteration           (default 10000)
//   time_step S        seconds (default 1e-3 (2 sqrt(65/pi))^2 / (4 diffc))
//   diffc D            A^2/s, sets only that default       (default 1e10)
//   gamma_langevin G   friction, per AKMA time unit        (default 0.001)
//   do_ld yes|no, do_bd_membrane yes|no                    (Langevin, mass-weighted BD)
//   seed N             (default: the clock's microseconds)
//   T K, kc, KA, kg, k_reg, lipid ... lines                (as the reference)
//   nequil N           the temperature average (AV_TEMP) restarts at outer
//                      iteration N (src/hd.C:2142-2147; default nsteps / 10)
// (the defaults are the reference's, src/input.C:16-310)
//   nmin N             N energy minimizations before the dynamics (the
//                      reference's L-BFGS, src/hd.C:805-840, src/minimize.C:489)
//   kv, restrain_volume_inside|outside
//                      the minimizer's leaflet-volume restraint
//                      (src/minimize.C:90-112): accepted while it is off;
//                      with nmin > 0, kv > 0 and restrain_volume_inside or
//                      _outside on, the run stops with an error (that term
//                      is not built)
//   planar_topology    accepted; the reference reads it only for the SRD
//                      solvent (src/hd.C:123, 625), which is not built
// Additions of this engine (no reference keyword):
//   do_bd_overdamped D overdamped BD with diffusion coefficient D (A^2/s)
//   precision fp64|fp32, mass yes|no (M^-1 from the limit surface for
//   do_ld/do_bd_membrane, default yes, as hd.C always builds it),
//   K_area, K_volume   global area/volume restraints (targets: the start state)
//   ignore_unsupported yes   warn about unsupported keywords instead of stopping
// Any other keyword of the reference (particles, collisions, output and
// analysis options, ...) stops the run with an error naming it: the driver
// runs the membrane path only and does not drop input it cannot honour. So
// does a run with neither do_ld nor do_bd_membrane (the reference's plain
// Hamiltonian dynamics with its nequil friction switch, not built here).
//
// Output per outer iteration, as the reference prints it (src/hd.C:1896-1899):
//   t: <ns> ns o: <o> T: <kinetic> V: <potential> T+V: ... TEMP: ... MEM_TEMP: ...
//   AV_TEMP ... VR: <angle term> VMEM: <membrane energy> VP: 0 steps/s: <rate>
// with T = p.M^-1 p / 2 of the state at the line and TEMP = 2T/(3nv-3)/k_B.
// An energy rise above 1e5 kcal/mol in one step stops the run as the
// reference's bail-out does (src/hd.C:1280-1300), writing NAME_crash0.save
// with the state before the failing iteration. NAME.save is written at the end.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>
#include <sys/time.h>

#include <cmath>
#include <map>
#include <string>
#include <vector>

#include "../../include/umcp_gpu.h"

namespace {

double now_s() {
  timeval tv;
  gettimeofday(&tv, nullptr);
  return tv.tv_sec + 1e-6 * tv.tv_usec;
}

std::string lower(std::string s) {
  for (char &c : s) c = (char)tolower((unsigned char)c);
  return s;
}

bool yes(const std::string &v) { return lower(v) == "yes" || v == "1" || lower(v) == "true" || lower(v) == "on"; }

// Keywords this driver honours (lower case); "lipid" lines go to the lipid parser.
const char *const kHandled[] = {"mesh", "jobname", "load", "nsteps", "nouter", "o_lim", "ninner", "time_step",
                                "gamma_langevin", "do_ld", "do_bd_membrane", "do_bd_overdamped", "seed", "t", "kc",
                                "ka", "kg", "k_reg", "lipid", "precision", "mass", "k_area", "k_volume", "nequil",
                                "nmin", "kv", "restrain_volume_inside", "restrain_volume_outside", "planar_topology",
                                "diffc", "ignore_unsupported"};

int die(const char *what) {
  fprintf(stderr, "hd_gb300: %s: %s\n", what, umcp_last_error());
  return 1;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s input.inp [key=value ...]\n", argv[0]);
    return 2;
  }
  FILE *fin = fopen(argv[1], "r");
  if (!fin) {
    fprintf(stderr, "hd_gb300: cannot open %s\n", argv[1]);
    return 1;
  }
  std::string text, line;
  std::map<std::string, std::string> kv;
  char buf[4096];
  auto take = [&](const std::string &l) {
    std::string s = l.substr(0, l.find('#'));
    char key[256], val[4096];
    if (sscanf(s.c_str(), "%255s %4095[^\n]", key, val) == 2) kv[lower(key)] = val;
    text += s + "\n";
  };
  while (fgets(buf, sizeof buf, fin)) take(buf);
  fclose(fin);
  for (int i = 2; i < argc; ++i) {
    std::string a = argv[i];
    size_t eq = a.find('=');
    if (eq == std::string::npos) continue;
    take(a.substr(0, eq) + " " + a.substr(eq + 1));
  }
  auto get = [&](const char *k, const char *def) { return kv.count(k) ? kv[k] : std::string(def); };
  auto getn = [&](std::initializer_list<const char *> ks, const char *def) {
    for (const char *k : ks)
      if (kv.count(k)) return kv[k];
    return std::string(def);
  };
  if (!kv.count("mesh")) {
    fprintf(stderr, "hd_gb300: no mesh keyword\n");
    return 1;
  }
  {
    std::string unsupported;
    for (const auto &e : kv) {
      bool ok = false;
      for (const char *h : kHandled) ok = ok || e.first == h;
      if (!ok) unsupported += (unsupported.empty() ? "" : ", ") + e.first;
    }
    if (!unsupported.empty()) {
      fprintf(stderr, "hd_gb300: keywords outside the membrane path, not built here: %s\n", unsupported.c_str());
      if (!yes(get("ignore_unsupported", "no"))) return 2;
    }
  }
  if (!yes(get("do_ld", "no")) && !yes(get("do_bd_membrane", "no")) && !kv.count("do_bd_overdamped")) {
    fprintf(stderr, "hd_gb300: set do_ld yes, do_bd_membrane yes or do_bd_overdamped D: the reference's plain "
                    "Hamiltonian dynamics (friction only after nequil, no noise) is not built\n");
    return 2;
  }
  const int nmin = atoi(get("nmin", "0").c_str());
  if (nmin > 0 && atof(get("kv", "0").c_str()) > 0 &&
      (yes(get("restrain_volume_inside", "no")) || yes(get("restrain_volume_outside", "no")))) {
    fprintf(stderr, "hd_gb300: the minimizer's leaflet-volume restraint (kv with restrain_volume_inside/outside, "
                    "src/minimize.C:90-112) is not built\n");
    return 2;
  }
  const std::string mesh_path = kv["mesh"], job = get("jobname", "job");
  const int nouter = atoi(getn({"nsteps", "nouter"}, "10000").c_str());
  const int ninner = atoi(getn({"o_lim", "ninner"}, "10000").c_str());
  const int nequil = kv.count("nequil") ? atoi(kv["nequil"].c_str()) : (int)(nouter * 0.1);
  const double diffc = atof(get("diffc", "1e10").c_str());
  const double lipid_d = 2.0 * std::sqrt(65.0 / M_PI);
  const double time_step = kv.count("time_step") ? atof(kv["time_step"].c_str()) : 1e-3 * lipid_d * lipid_d / (4.0 * diffc);
  int seed = kv.count("seed") ? atoi(kv["seed"].c_str()) : (int)(std::fmod(now_s(), 1.0) * 1e6);

  umcp_params prm;
  umcp_params_default(&prm);
  std::vector<char> lipid_buf(text.size() + 1);
  if (umcp_params_from_input(text.c_str(), &prm, lipid_buf.data(), lipid_buf.size()) != UMCP_OK)
    return die("input");
  prm.precision = lower(get("precision", "fp64")) == "fp32" ? UMCP_FP32_CENTRED : UMCP_FP64;

  umcp_integrator it{};
  it.time_step = time_step;
  it.seed = (uint64_t)seed;
  it.gamma = atof(get("gamma_langevin", "0.001").c_str());
  it.divergence_threshold = 1e5;
  if (kv.count("do_bd_overdamped")) {
    it.kind = UMCP_OVERDAMPED_BD;
    it.D = atof(kv["do_bd_overdamped"].c_str());
  } else if (yes(get("do_bd_membrane", "no"))) {
    it.kind = UMCP_BD_MEMBRANE;
  } else {
    it.kind = UMCP_LANGEVIN;  // do_ld, and the reference's default dynamics
  }
  const bool use_mass = it.kind != UMCP_OVERDAMPED_BD && yes(get("mass", "yes"));
  it.use_mass = use_mass ? 1 : 0;

  umcp_ctx *ctx;
  umcp_plan *plan;
  umcp_mesh *mesh;
  if (umcp_ctx_create(0, &ctx) != UMCP_OK) return die("device");
  if (umcp_plan_from_file(mesh_path.c_str(), &prm, &plan) != UMCP_OK) return die("mesh");
  if (umcp_mesh_create(ctx, plan, &prm, &mesh) != UMCP_OK) return die("upload");
  umcp_mesh_info info;
  umcp_mesh_info_get(mesh, &info);
  const int nv = info.nv;
  printf("hd_gb300: %d vertices, %d faces, %s, %s\n", nv, info.n_faces,
         prm.precision == UMCP_FP64 ? "FP64" : "FP32 precision form",
         it.kind == UMCP_LANGEVIN ? "Langevin" : it.kind == UMCP_BD_MEMBRANE ? "BD (membrane)" : "overdamped BD");
  if (use_mass) {
    umcp_mass_info mi;
    double t0 = now_s();
    if (umcp_mass_build(mesh, plan, nullptr, &mi) != UMCP_OK) return die("effective mass");
    printf("effective mass: %lld points, %.4le amu each, M^-1 %s, built in %.2lf s\n", mi.points, mi.mass_per_point,
           mi.dense ? "dense" : "sparse", now_s() - t0);
  }
  if (kv.count("load")) {
    int s2 = -1;
    if (umcp_restart_read(mesh, kv["load"].c_str(), &s2) != UMCP_OK) {
      fprintf(stderr, "hd_gb300: cannot read restart %s\n", kv["load"].c_str());
      return 1;
    }
    if (s2 > 0) it.seed = (uint64_t)(seed = s2);
    printf("Loaded %s\n", kv["load"].c_str());
  }
  const double K_area = atof(get("k_area", "0").c_str()), K_volume = atof(get("k_volume", "0").c_str());
  if (K_area > 0 || K_volume > 0) {
    umcp_restraints rs{K_area, -1.0, K_volume, -1.0};
    if (umcp_restraints_set(mesh, &rs) != UMCP_OK) return die("restraints");
  }

  for (int k = 0; k < nmin; ++k) {
    umcp_minimize_info mi;
    if (umcp_minimize(mesh, nullptr, nullptr, &mi) != UMCP_OK) return die("minimize");
    printf("minimization %d: %d iterations, energy %.10le -> %.10le\n", k, mi.iterations, mi.energy_initial,
           mi.energy_final);
  }

  std::vector<double> r(3 * (size_t)nv + 3), p(3 * (size_t)nv), q(3 * (size_t)nv), e((size_t)std::max(ninner, 1));
  double av_temp = 0, rate = 0;
  int n_temp = 0;
  const std::string crash = job + "_crash0.save";
  for (int o = 0; o < nouter; ++o) {
    // the line's state: energy terms, kinetic energy p.M^-1 p / 2
    double V = 0, terms[3] = {0, 0, 0};
    umcp_state_get(mesh, r.data(), p.data());
    if (umcp_energy(mesh, r.data(), &V, terms) != UMCP_OK) return die("energy");
    double T = 0;
    if (use_mass) {
      std::fill(q.begin(), q.end(), 0.0);
      if (umcp_mass_apply(mesh, p.data(), q.data(), nullptr, 1.0, nullptr) != UMCP_OK) return die("mass apply");
      for (size_t i = 0; i < p.size(); ++i) T += 0.5 * p[i] * q[i];
    } else {
      for (size_t i = 0; i < p.size(); ++i) T += 0.5 * p[i] * p[i];
    }
    const double temp = 2 * T / (3.0 * nv - 3.0) / (5.92186663194e-01 / 298.0);
    if (o == nequil) av_temp = 0, n_temp = 0;  // the average restarts after equilibration
    av_temp += temp;
    ++n_temp;
    printf("t: %le ns o: %d T: %.8le V: %.12le T+V: %.14le TEMP: %le MEM_TEMP: %le AV_TEMP %le VR: %.3le VMEM: %le VP: %le",
           o * (double)ninner * time_step * 1e9, o, T, V, T + V, temp, temp, av_temp / n_temp, terms[2], V, 0.0);
    if (rate > 0) printf(" steps/s: %le", rate);
    printf("\n");
    fflush(stdout);
    umcp_restart_write(mesh, crash.c_str(), seed);  // the state before this iteration
    const double t0 = now_s();
    umcp_status st = umcp_run(mesh, &it, (uint64_t)o * (uint64_t)ninner, ninner, e.data());
    rate = ninner / (now_s() - t0 + 1e-10);
    if (st == UMCP_ERR_DIVERGED || st == UMCP_ERR_NONFINITE) {
      printf("System unstable at iteration %d: %s, bailing (state before the iteration in %s).\n", o,
             umcp_last_error(), crash.c_str());
      return 1;
    }
    if (st != UMCP_OK) return die("run");
  }
  remove(crash.c_str());
  double V = 0;
  umcp_state_get(mesh, r.data(), nullptr);
  umcp_energy(mesh, r.data(), &V, nullptr);
  printf("Energy at save: %.14le\n", V);
  const std::string save = job + ".save";
  if (umcp_restart_write(mesh, save.c_str(), seed) != UMCP_OK) return die("save");
  umcp_mesh_destroy(mesh);
  umcp_plan_destroy(plan);
  umcp_ctx_destroy(ctx);
  return 0;
}
