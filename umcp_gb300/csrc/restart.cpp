// Restart files in the reference's save format (Simulation::saveRestart /
// loadRestart, src/restart.C:7-168), for one surface without particles:
//   alpha_x alpha_y alpha_z
//   x y z px py pz          one line per vertex, then one for the box scales
//   seed N
// Numbers are written with %lf as the reference writes them; lines with three
// numbers (no momenta) and lines after the surface's (particle records) are
// accepted on reading.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/umcp_gpu.h"

extern "C" umcp_status umcp_restart_write(umcp_mesh *mesh, const char *path, int seed) {
  if (!mesh || !path) return UMCP_ERR_INVALID;
  umcp_mesh_info info;
  umcp_status st = umcp_mesh_info_get(mesh, &info);
  if (st != UMCP_OK) return st;
  const int nv = info.nv;
  std::vector<double> r(3 * (size_t)nv + 3), p(3 * (size_t)nv + 3, 0.0);
  if ((st = umcp_state_get(mesh, r.data(), p.data())) != UMCP_OK) return st;
  FILE *f = fopen(path, "w");
  if (!f) return UMCP_ERR_IO;
  fprintf(f, "%lf %lf %lf\n", r[3 * nv], r[3 * nv + 1], r[3 * nv + 2]);
  for (int v = 0; v < nv + 1; ++v)
    fprintf(f, "%lf %lf %lf %lf %lf %lf\n", r[3 * v], r[3 * v + 1], r[3 * v + 2], p[3 * v], p[3 * v + 1], p[3 * v + 2]);
  fprintf(f, "seed %d\n", seed);
  return fclose(f) == 0 ? UMCP_OK : UMCP_ERR_IO;
}

extern "C" umcp_status umcp_restart_read(umcp_mesh *mesh, const char *path, int *seed) {
  if (!mesh || !path) return UMCP_ERR_INVALID;
  umcp_mesh_info info;
  umcp_status st = umcp_mesh_info_get(mesh, &info);
  if (st != UMCP_OK) return st;
  const int nv = info.nv;
  FILE *f = fopen(path, "r");
  if (!f) return UMCP_ERR_IO;
  std::vector<double> r(3 * (size_t)nv + 3, 0.0), p(3 * (size_t)nv + 3, 0.0);
  char line[4096];
  double a[3];
  bool ok = fgets(line, sizeof line, f) && sscanf(line, "%lf %lf %lf", &a[0], &a[1], &a[2]) == 3;
  for (int v = 0; ok && v < nv + 1; ++v) {
    double x[6];
    ok = fgets(line, sizeof line, f) != nullptr;
    if (!ok) break;
    const int n = sscanf(line, "%lf %lf %lf %lf %lf %lf", &x[0], &x[1], &x[2], &x[3], &x[4], &x[5]);
    if (n != 3 && n != 6) { ok = false; break; }
    for (int c = 0; c < 3; ++c) {
      r[3 * (size_t)v + c] = x[c];
      if (n == 6) p[3 * (size_t)v + c] = x[3 + c];
    }
  }
  // The box scales: the first line is the simulation's alpha, which the
  // reference loads into the surface state as well.
  if (ok) for (int c = 0; c < 3; ++c) r[3 * (size_t)nv + c] = a[c];
  int sd = -1;
  while (ok && fgets(line, sizeof line, f))
    if (sscanf(line, "seed %d", &sd) == 1) break;
  fclose(f);
  if (!ok) return UMCP_ERR_IO;
  if (seed) *seed = sd;
  p.resize(3 * (size_t)nv);
  return umcp_state_set(mesh, r.data(), p.data());
}
