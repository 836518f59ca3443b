// Limit-surface points of a mesh's resident state: surface::evaluateRNRM
// (src/interpLib.C:7936-8020) on every face at the lattice (u, v) = (i/p,
// j/p), i + j <= p, and the reference's limit-surface writer
// (surface::writeLimitingSurface, src/write_structures.C:660-715, which takes
// p = 1: each face's three corners). One thread per (face, point), FP64. The
// weight rows of a lattice point depend only on the patch type (the box
// spline on regular faces; the irregular map of the corner's valence on the
// others), so the host forms one table per patch type.
#include <stdio.h>

#include <string>
#include <vector>

#include "engine.h"
#include "plan.h"

using namespace umcp;

namespace {

// R[o] = alpha (sum_x w_x X_x), N[o] = unit (X_u x X_v) from the tangents
// before the box scaling (as the reference forms it), o = the face's plan
// index times npts plus the point.
__global__ void limit_points_kernel(int nfaces, int ncp, int npts, const uint32_t *__restrict__ cp,
                                    const int *__restrict__ face_index, const double *__restrict__ rows,
                                    const double *__restrict__ r, dev::SurfaceParams P, double *__restrict__ R,
                                    double *__restrict__ N) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nfaces * npts) return;
  const int f = (int)(t / npts), q = (int)(t % npts);
  const double *w = rows + (size_t)q * 3 * ncp, *du = w + ncp, *dv = du + ncp;
  double X[3] = {0, 0, 0}, Xu[3] = {0, 0, 0}, Xv[3] = {0, 0, 0};
  for (int x = 0; x < ncp; ++x) {
    const uint32_t packed = cp[(size_t)f * ncp + x];
    const int v = (int)(packed & dev::kVertexMask), code = (int)(packed >> dev::kVertexBits);
    const int img[3] = {code % 3 - 1, (code / 3) % 3 - 1, code / 9 - 1};
    for (int c = 0; c < 3; ++c) {
      const double pos = r[3 * (size_t)v + c] + img[0] * P.box[0][c] + img[1] * P.box[1][c] + img[2] * P.box[2][c];
      X[c] += w[x] * pos;
      Xu[c] += du[x] * pos;
      Xv[c] += dv[x] * pos;
    }
  }
  const size_t o = (size_t)face_index[f] * npts + q;
  for (int c = 0; c < 3; ++c) R[3 * o + c] = r[3 * (size_t)P.nv + c] * X[c];
  if (N) {
    const double m[3] = {Xu[1] * Xv[2] - Xu[2] * Xv[1], Xu[2] * Xv[0] - Xu[0] * Xv[2], Xu[0] * Xv[1] - Xu[1] * Xv[0]};
    const double l = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
    for (int c = 0; c < 3; ++c) N[3 * o + c] = m[c] / l;
  }
}

umcp_status fail(umcp_status s, const std::string &m) { return set_error(s, m); }

}  // namespace

extern "C" umcp_status umcp_limit_points(umcp_mesh *m, int plim, double *R, double *N) {
  if (!m || !R || plim < 1 || plim > 1000) return fail(UMCP_ERR_INVALID, "bad argument");
  UMCP_CUDA(cudaSetDevice(m->ctx->device));
  cudaStream_t s = m->ctx->stream;
  const int npts = (plim + 1) * (plim + 2) / 2;
  const size_t nout = (size_t)m->nfaces * npts * 3;
  DevBuf dR, dN, drows, didx;
  UMCP_CUDA(dR.alloc(nout * sizeof(double)));
  if (N) UMCP_CUDA(dN.alloc(nout * sizeof(double)));
  IrregularMap m5(5), m7(7);
  IrregularMap *maps[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, &m5, nullptr, &m7};
  for (auto &Gp : m->groups) {
    const Group &G = *Gp;
    if (!G.nfaces) continue;
    Face F{};
    F.valence = G.valence;
    F.ncp = G.ncp;
    std::vector<double> rows((size_t)npts * 3 * G.ncp);
    int q = 0;
    for (int fi = 0; fi <= plim; ++fi)
      for (int fj = 0; fj <= plim - fi; ++fj, ++q) {
        double *w = &rows[(size_t)q * 3 * G.ncp];
        limit_point_rows(F, fi / (double)plim, fj / (double)plim, maps, w, w + G.ncp, w + 2 * G.ncp);
      }
    UMCP_CUDA(upload(drows, rows));
    UMCP_CUDA(upload(didx, G.face_index));
    const long long nthreads = (long long)G.nfaces * npts;
    limit_points_kernel<<<(unsigned)((nthreads + 255) / 256), 256, 0, s>>>(
        G.nfaces, G.ncp, npts, G.cp.as<uint32_t>(), didx.as<int>(), drows.as<double>(), m->r.as<double>(), m->P,
        dR.as<double>(), N ? dN.as<double>() : nullptr);
    UMCP_CUDA(cudaGetLastError());
    UMCP_CUDA(cudaStreamSynchronize(s));  // the tables above are freed at the next group
  }
  UMCP_CUDA(cudaMemcpyAsync(R, dR.p, nout * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (N) UMCP_CUDA(cudaMemcpyAsync(N, dN.p, nout * sizeof(double), cudaMemcpyDeviceToHost, s));
  UMCP_CUDA(cudaStreamSynchronize(s));
  return UMCP_OK;
}

extern "C" umcp_status umcp_write_limiting_surface(umcp_mesh *m, const char *path) {
  if (!m || !path) return fail(UMCP_ERR_INVALID, "null argument");
  std::vector<double> R((size_t)m->nfaces * 3 * 3);
  umcp_status st = umcp_limit_points(m, 1, R.data(), nullptr);
  if (st != UMCP_OK) return st;
  FILE *f = fopen(path, "w");
  if (!f) return fail(UMCP_ERR_IO, std::string("cannot write ") + path);
  fprintf(f, "%d\n", 3 * m->nfaces);
  fprintf(f, "limiting surface\n");
  for (size_t p = 0; p < R.size() / 3; ++p) fprintf(f, "C %lf %lf %lf\n", R[3 * p], R[3 * p + 1], R[3 * p + 2]);
  fclose(f);
  return UMCP_OK;
}
