// C ABI of the membrane-surface engine (include/umcp_gpu.h): host plans,
// device-resident meshes, energy/gradient, effective-mass apply and runs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/umcp_gpu.h"
#include "launch.h"
#include "mesh.h"
#include "plan.h"
#include "engine.h"

using namespace umcp;

static constexpr double kAkmaTime = 1.0 / (0.04888 * 1e-12);  // AKMA_TIME, src/units.h:5

// ------------------------------------------------------------------ errors

static thread_local std::string g_last_error;

umcp_status umcp::set_error(umcp_status s, const std::string &msg) {
  g_last_error = msg;
  return s;
}

static umcp_status fail(umcp_status s, const std::string &msg) { return umcp::set_error(s, msg); }

extern "C" const char *umcp_last_error(void) { return g_last_error.c_str(); }

extern "C" const char *umcp_status_string(umcp_status s) {
  switch (s) {
    case UMCP_OK: return "ok";
    case UMCP_ERR_INVALID: return "invalid argument";
    case UMCP_ERR_IO: return "i/o error";
    case UMCP_ERR_CUDA: return "cuda error";
    case UMCP_ERR_NONFINITE: return "non-finite energy";
    case UMCP_ERR_TIMEOUT: return "device wait timed out";
    case UMCP_ERR_NOMEM: return "out of device memory";
    case UMCP_ERR_UNSUPPORTED: return "unsupported";
    case UMCP_ERR_DIVERGED: return "diverged";
  }
  return "unknown";
}

// ------------------------------------------------------------------ params

extern "C" umcp_status umcp_params_default(umcp_params *p) {
  if (!p) return fail(UMCP_ERR_INVALID, "null params");
  p->kc = 14.0;      // src/input.C:66
  p->KA = 0.215;     // src/input.C:64,309-310 (KA -1 resolves to 0.215)
  p->kg = 0.0;       // src/input.C:67
  p->k_reg = 0.0;    // src/interpLib.C:87
  p->temperature = 298.0;  // src/input.C:71
  p->precision = UMCP_FP64;
  p->lipid_directives = nullptr;
  p->face_kernel = 0;
  return UMCP_OK;
}

extern "C" umcp_status umcp_params_from_input(const char *text, umcp_params *p, char *lipid_buf, size_t lipid_len) {
  if (!text || !p) return fail(UMCP_ERR_INVALID, "null argument");
  std::istringstream in(text);
  std::string line, lipids;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    std::string key;
    if (!(ls >> key)) continue;
    std::string lk = key;
    for (char &c : lk) c = (char)tolower((unsigned char)c);
    if (lk == "lipid") { lipids += line + "\n"; continue; }
    double v;
    if (!(ls >> v)) continue;
    if (lk == "kc") p->kc = v;
    else if (lk == "ka") p->KA = (v < 0) ? 0.215 : v;
    else if (lk == "kg") p->kg = v;
    else if (lk == "t") p->temperature = v;
    else if (lk == "k_reg") p->k_reg = v;
  }
  if (lipid_buf && lipid_len) {
    if (lipids.size() + 1 > lipid_len) return fail(UMCP_ERR_INVALID, "lipid buffer too small");
    memcpy(lipid_buf, lipids.c_str(), lipids.size() + 1);
    p->lipid_directives = lipid_buf;
  }
  return UMCP_OK;
}

// ------------------------------------------------------------------ mesh generators

extern "C" umcp_status umcp_mesh_generate_icosphere(int level, double R, double sigma, uint64_t seed, const char *path) {
  if (level < 1 || level > 9 || !(R > 0) || sigma < 0 || !path)
    return fail(UMCP_ERR_INVALID, "icosphere needs 1 <= level <= 9, R > 0, sigma >= 0");
  Mesh m;
  generate_icosphere(level, R, sigma, seed, &m);
  std::string e = write_mesh(path, m);
  return e.empty() ? UMCP_OK : fail(UMCP_ERR_IO, e);
}

extern "C" umcp_status umcp_mesh_generate_planar(int nx, int ny, double a, double kc_kT, uint64_t seed, const char *path) {
  if (nx < 4 || ny < 4 || !(a > 0) || !(kc_kT > 0) || !path)
    return fail(UMCP_ERR_INVALID, "planar mesh needs nx, ny >= 4, a > 0, kc > 0");
  Mesh m;
  generate_planar(nx, ny, a, kc_kT, seed, &m);
  std::string e = write_mesh(path, m);
  return e.empty() ? UMCP_OK : fail(UMCP_ERR_IO, e);
}

// ------------------------------------------------------------------ plans

struct umcp_plan {
  Mesh mesh;
  Plan plan;
};

extern "C" umcp_status umcp_plan_from_file(const char *mesh_path, const umcp_params *p, umcp_plan **out) {
  if (!mesh_path || !out) return fail(UMCP_ERR_INVALID, "null argument");
  auto pl = std::make_unique<umcp_plan>();
  std::string e = read_mesh(mesh_path, &pl->mesh);
  if (!e.empty()) return fail(e.find("cannot open") == 0 ? UMCP_ERR_IO : UMCP_ERR_INVALID, e);
  e = orient(&pl->mesh);
  if (!e.empty()) return fail(UMCP_ERR_INVALID, e);
  std::vector<Lipid> lipids;
  e = parse_lipids((p && p->lipid_directives) ? p->lipid_directives : "", &lipids);
  if (!e.empty()) return fail(UMCP_ERR_INVALID, e);
  e = build_plan(pl->mesh, lipids, &pl->plan);
  if (!e.empty()) return fail(UMCP_ERR_INVALID, e);
  *out = pl.release();
  return UMCP_OK;
}

const Plan &umcp::plan_of(const umcp_plan *p) { return p->plan; }

extern "C" umcp_status umcp_plan_point_coeffs(const umcp_plan *plan, int face, double u, double v, int *ids,
                                              double *coef, int *n) {
  if (!plan || !ids || !coef || !n) return fail(UMCP_ERR_INVALID, "null argument");
  const Plan &P = plan->plan;
  const int nreg = (int)P.reg_faces.size(), nirr = (int)P.irr_faces.size();
  if (face < 0 || face >= nreg + nirr) return fail(UMCP_ERR_INVALID, "face index out of range");
  if (!(u >= -1e-4 && v >= -1e-4 && u + v <= 1.0 + 1e-4)) return fail(UMCP_ERR_INVALID, "(u,v) outside the face");
  const Face &F = face < nreg ? P.reg_faces[face] : P.irr_faces[face - nreg];
  IrregularMap m5(5), m7(7);
  IrregularMap *maps[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, &m5, nullptr, &m7};
  *n = limit_point_coeffs(F, u, v, maps, coef);
  for (int x = 0; x < *n; ++x) ids[x] = F.cp[x];
  return UMCP_OK;
}

extern "C" umcp_status umcp_plan_evaluate(const umcp_plan *plan, const double *r, int n, const int *faces,
                                          const double *uv, double *R, double *N) {
  if (!plan || !r || n < 0 || (n > 0 && (!faces || !uv || !R))) return fail(UMCP_ERR_INVALID, "bad argument");
  const Plan &P = plan->plan;
  const Mesh &ME = plan->mesh;
  const int nreg = (int)P.reg_faces.size(), nirr = (int)P.irr_faces.size(), nv = ME.nv;
  IrregularMap m5(5), m7(7);
  IrregularMap *maps[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, &m5, nullptr, &m7};
  for (int q = 0; q < n; ++q) {
    const int face = faces[q];
    const double u = uv[2 * q], v = uv[2 * q + 1];
    if (face < 0 || face >= nreg + nirr) return fail(UMCP_ERR_INVALID, "face index out of range");
    if (!(u >= -1e-4 && v >= -1e-4 && u + v <= 1.0 + 1e-4)) return fail(UMCP_ERR_INVALID, "(u,v) outside the face");
    const Face &F = face < nreg ? P.reg_faces[face] : P.irr_faces[face - nreg];
    double w[kMaxCp], du[kMaxCp], dv[kMaxCp];
    limit_point_rows(F, u, v, maps, w, du, dv);
    double X[3] = {0, 0, 0}, Xu[3] = {0, 0, 0}, Xv[3] = {0, 0, 0};
    for (int x = 0; x < F.ncp; ++x)
      for (int c = 0; c < 3; ++c) {
        const double pos = r[3 * (size_t)F.cp[x] + c] + F.img[x][0] * ME.box[0][c] + F.img[x][1] * ME.box[1][c] +
                           F.img[x][2] * ME.box[2][c];
        X[c] += w[x] * pos;
        Xu[c] += du[x] * pos;
        Xv[c] += dv[x] * pos;
      }
    for (int c = 0; c < 3; ++c) R[3 * (size_t)q + c] = r[3 * (size_t)nv + c] * X[c];
    if (N) {
      // from the tangents before the box scaling, as the reference forms it
      const double *a = Xu, *b = Xv;
      double m[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
      const double l = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
      for (int c = 0; c < 3; ++c) N[3 * (size_t)q + c] = m[c] / l;
    }
  }
  return UMCP_OK;
}

extern "C" umcp_status umcp_plan_set_reference(umcp_plan *plan, const double *r) {
  if (!plan || !r) return fail(UMCP_ERR_INVALID, "null argument");
  set_reference_state(plan->mesh, r, &plan->plan);
  return UMCP_OK;
}

extern "C" umcp_status umcp_plan_info_get(const umcp_plan *plan, umcp_plan_info *info) {
  if (!plan || !info) return fail(UMCP_ERR_INVALID, "null argument");
  info->nv = plan->mesh.nv;
  info->n_regular = (int)plan->plan.reg_faces.size();
  info->n_irregular = (int)plan->plan.irr_faces.size();
  info->n_lipid_types = plan->plan.ntypes;
  for (int d = 0; d < 3; ++d)
    for (int c = 0; c < 3; ++c) info->box[3 * d + c] = plan->mesh.box[d][c];
  return UMCP_OK;
}

extern "C" umcp_status umcp_plan_positions(const umcp_plan *plan, double *r) {
  if (!plan || !r) return fail(UMCP_ERR_INVALID, "null argument");
  std::copy(plan->mesh.r.begin(), plan->mesh.r.end(), r);
  r[3 * plan->mesh.nv] = r[3 * plan->mesh.nv + 1] = r[3 * plan->mesh.nv + 2] = 1.0;
  return UMCP_OK;
}

extern "C" umcp_status umcp_plan_rings(const umcp_plan *plan, int *valence, int *ring) {
  if (!plan) return fail(UMCP_ERR_INVALID, "null argument");
  if (valence) std::copy(plan->mesh.valence.begin(), plan->mesh.valence.end(), valence);
  if (ring) std::copy(plan->mesh.nbr.begin(), plan->mesh.nbr.end(), ring);
  return UMCP_OK;
}

extern "C" umcp_status umcp_plan_faces(const umcp_plan *plan, int kind, int *cp, int8_t *img, int *valence, double *g0,
                                       double *rr0, double *outer, double *inner) {
  if (!plan || (kind != 0 && kind != 1)) return fail(UMCP_ERR_INVALID, "bad plan or kind");
  const Plan &P = plan->plan;
  const std::vector<Face> &F = kind ? P.irr_faces : P.reg_faces;
  const int npt = kind ? kIrrPts : kRegPts;
  for (size_t f = 0; f < F.size(); ++f) {
    for (int x = 0; x < 13; ++x) {
      if (cp) cp[f * 13 + x] = (x < F[f].ncp) ? F[f].cp[x] : -1;
      for (int c = 0; c < 3; ++c)
        if (img) img[(f * 13 + x) * 3 + c] = (x < F[f].ncp) ? F[f].img[x][c] : 0;
    }
    if (valence) valence[f] = F[f].valence;
  }
  const std::vector<double> &G0 = kind ? P.irr_g0 : P.reg_g0, &RR = kind ? P.irr_RuRv0 : P.reg_RuRv0;
  if (g0) std::copy(G0.begin(), G0.end(), g0);
  if (rr0) std::copy(RR.begin(), RR.end(), rr0);
  (void)npt;
  const std::vector<double> &O = kind ? P.irr_outer : P.reg_outer, &I = kind ? P.irr_inner : P.reg_inner;
  if (outer) std::copy(O.begin(), O.end(), outer);
  if (inner) std::copy(I.begin(), I.end(), inner);
  return UMCP_OK;
}

extern "C" umcp_status umcp_plan_basis(const umcp_plan *plan, int valence, double *rows, double *weight, double *u,
                                       double *v) {
  if (!plan) return fail(UMCP_ERR_INVALID, "null plan");
  PatchBasis tmp;
  const PatchBasis *B = nullptr;
  if (valence == 6) B = &plan->plan.regular;
  else if (valence == 5 || valence == 7) {
    B = &plan->plan.irregular[valence];
    if (B->row.empty()) {
      std::string e = build_irregular_basis(valence, &tmp);
      if (!e.empty()) return fail(UMCP_ERR_INVALID, e);
      B = &tmp;
    }
  } else
    return fail(UMCP_ERR_INVALID, "valence must be 5, 6 or 7");
  if (rows) std::copy(B->row.begin(), B->row.end(), rows);
  if (weight) std::copy(B->weight.begin(), B->weight.end(), weight);
  if (u) std::copy(B->u.begin(), B->u.end(), u);
  if (v) std::copy(B->v.begin(), B->v.end(), v);
  return UMCP_OK;
}

extern "C" umcp_status umcp_plan_lipids(const umcp_plan *plan, double *c0, double *apl) {
  if (!plan) return fail(UMCP_ERR_INVALID, "null plan");
  for (size_t x = 0; x < plan->plan.lipids.size(); ++x) {
    if (c0) c0[x] = plan->plan.lipids[x].c0;
    if (apl) apl[x] = plan->plan.lipids[x].apl;
  }
  return UMCP_OK;
}

extern "C" void umcp_plan_destroy(umcp_plan *plan) { delete plan; }

// ------------------------------------------------------------------ device context


extern "C" umcp_status umcp_ctx_create(int device, umcp_ctx **out) {
  if (!out) return fail(UMCP_ERR_INVALID, "null out");
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return fail(UMCP_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
  if (device < 0 || device >= n) return fail(UMCP_ERR_INVALID, "device index out of range");
  UMCP_CUDA(cudaSetDevice(device));
  auto c = std::make_unique<umcp_ctx>();
  c->device = device;
  UMCP_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  UMCP_CUDA(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
  UMCP_CUDA(cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming));
  UMCP_CUDA(cudaEventCreateWithFlags(&c->join, cudaEventDisableTiming));
  *out = c.release();
  return UMCP_OK;
}

extern "C" void umcp_ctx_destroy(umcp_ctx *ctx) {
  if (ctx) ctx_release(ctx);  // the stream goes when the last mesh or batch on it does
}

extern "C" umcp_status umcp_ctx_stream(umcp_ctx *ctx, void **stream) {
  if (!ctx || !stream) return fail(UMCP_ERR_INVALID, "null argument");
  *stream = (void *)ctx->stream;
  return UMCP_OK;
}

extern "C" umcp_status umcp_ctx_mem_info(umcp_ctx *ctx, size_t *free_bytes, size_t *total_bytes) {
  if (!ctx) return fail(UMCP_ERR_INVALID, "null ctx");
  UMCP_CUDA(cudaSetDevice(ctx->device));
  size_t f = 0, t = 0;
  UMCP_CUDA(cudaMemGetInfo(&f, &t));
  if (free_bytes) *free_bytes = f;
  if (total_bytes) *total_bytes = t;
  return UMCP_OK;
}

extern "C" umcp_status umcp_ctx_synchronize(umcp_ctx *ctx) {
  if (!ctx) return fail(UMCP_ERR_INVALID, "null ctx");
  UMCP_CUDA(cudaStreamSynchronize(ctx->stream));
  return UMCP_OK;
}

// ------------------------------------------------------------------ device mesh


static void fill_params(umcp_mesh *m, const umcp_params *p) {
  m->kT = (5.92186663194E-01 / 298.0) * p->temperature;
  m->P.kc = p->kc;
  m->P.KA = p->KA;
  m->P.kg = p->kg;
  m->P.k_reg = p->k_reg;
}

namespace {
// The pinned host staging of the host-pointer calls (state in and out, run
// counters), allocated at the first such call: meshes run only from the
// device (batches, servers) never pay for page-locking.
cudaError_t ensure_pinned(umcp_mesh *m) {
  if (m->h_pinned) return cudaSuccess;
  const size_t nst = 3 * (size_t)m->nv + 3;
  const size_t a = (nst * sizeof(double) + 63) & ~(size_t)63, b = (3 * (size_t)m->nv * sizeof(double) + 63) & ~(size_t)63;
  cudaError_t e = cudaMallocHost(&m->h_pinned, a + b + 2 * sizeof(uint64_t));
  if (e != cudaSuccess) return e;
  unsigned char *h = (unsigned char *)m->h_pinned;
  m->h_stage = (double *)h;
  m->h_stage2 = (double *)(h + a);
  m->h_cnt = (uint64_t *)(h + a + b);
  return cudaSuccess;
}

// The device buffers a mesh makes at creation, carved out of one allocation
// (one cudaMalloc, one host-to-device copy and one memset per mesh instead
// of some forty calls; a server admits meshes one after another). Sections,
// in order: contents staged from the host, zero-initialised, uninitialised.
class MeshArena {
 public:
  template <class T>
  void stage(umcp::DevBuf &b, const std::vector<T> &h) {
    const size_t at = align(host_.size()), n = h.size() * sizeof(T);
    host_.resize(at + n);
    if (n) memcpy(host_.data() + at, h.data(), n);
    parts_.push_back({&b, 0, at, n});
  }
  void zeroed(umcp::DevBuf &b, size_t n) { parts_.push_back({&b, 1, 0, n}); }
  void uninit(umcp::DevBuf &b, size_t n) { parts_.push_back({&b, 2, 0, n}); }
  cudaError_t commit(umcp::DevBuf &store) {
    size_t off[3] = {0, align(host_.size()), 0};
    size_t zero_end = off[1];
    for (Part &q : parts_)
      if (q.section == 1) { q.at = zero_end; zero_end = align(zero_end + q.n); }
    size_t end = zero_end;
    for (Part &q : parts_)
      if (q.section == 2) { q.at = end; end = align(end + q.n); }
    cudaError_t e = store.alloc(std::max<size_t>(end, 1));
    if (e != cudaSuccess) return e;
    unsigned char *base = store.as<unsigned char>();
    for (Part &q : parts_) q.buf->view(base + q.at, q.n);
    if (!host_.empty()) e = cudaMemcpy(base, host_.data(), host_.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && zero_end > off[1]) e = cudaMemset(base + off[1], 0, zero_end - off[1]);
    return e;
  }

 private:
  struct Part {
    umcp::DevBuf *buf;
    int section;
    size_t at, n;
  };
  static size_t align(size_t x) { return (x + 255) & ~(size_t)255; }
  std::vector<unsigned char> host_;
  std::vector<Part> parts_;
};
}  // namespace

extern "C" umcp_status umcp_mesh_create(umcp_ctx *ctx, const umcp_plan *plan, const umcp_params *prm, umcp_mesh **out) {
  if (!ctx || !plan || !out) return fail(UMCP_ERR_INVALID, "null argument");
  umcp_params defaults;
  umcp_params_default(&defaults);
  if (!prm) prm = &defaults;
  if (prm->precision != UMCP_FP64 && prm->precision != UMCP_FP32_CENTRED)
    return fail(UMCP_ERR_INVALID, "unknown precision");
  UMCP_CUDA(cudaSetDevice(ctx->device));
  auto m = std::make_unique<umcp_mesh>();
  m->ctx = ctx;
  m->precision = prm->precision;
  const Plan &PL = plan->plan;
  const Mesh &ME = plan->mesh;
  m->nv = ME.nv;
  m->P.nv = ME.nv;
  for (int d = 0; d < 3; ++d)
    for (int c = 0; c < 3; ++c) {
      m->P.box[d][c] = ME.box[d][c];
      m->P.box_hi[d][c] = (float)ME.box[d][c];
      m->P.box_lo[d][c] = (float)(ME.box[d][c] - (double)m->P.box_hi[d][c]);
    }
  fill_params(m.get(), prm);

  // Face groups: regular, then irregular by valence (5, 7).
  struct Src { const PatchBasis *B; std::vector<int> idx; bool irr; };
  std::vector<Src> srcs;
  {
    Src s{&PL.regular, {}, false};
    for (size_t f = 0; f < PL.reg_faces.size(); ++f) s.idx.push_back((int)f);
    srcs.push_back(s);
    for (int val : {5, 7}) {
      Src t{&PL.irregular[val], {}, true};
      for (size_t f = 0; f < PL.irr_faces.size(); ++f)
        if (PL.irr_faces[f].valence == val) t.idx.push_back((int)f);
      if (!t.idx.empty()) srcs.push_back(t);
    }
  }
  const int nt = PL.ntypes;
  MeshArena arena;
  std::vector<int> slot_vertex;  // vertex of every (face, control point) slot, in slot order
  std::vector<int> counts(ME.nv, 0);
  int face_base = 0, slot_base = 0, block_base = 0, block_rows = 0;
  for (const Src &s : srcs) {
    auto G = std::make_unique<Group>();
    const PatchBasis &B = *s.B;
    G->ncp = B.ncp;
    G->npt = B.npt;
    G->nfaces = (int)s.idx.size();
    G->slot_base = slot_base;
    G->irregular = s.irr;
    G->valence = B.valence;
    G->dudv = s.irr ? 1.0 : 0.5;
    for (int f : s.idx) G->face_index.push_back(s.irr ? (int)PL.reg_faces.size() + f : f);
    std::vector<uint32_t> cp((size_t)G->nfaces * G->ncp);
    std::vector<double> g0((size_t)G->nfaces * G->npt), rr0((size_t)G->nfaces * G->npt), comp((size_t)G->nfaces * 3);
    for (int q = 0; q < G->nfaces; ++q) {
      int f = s.idx[q];
      const Face &F = s.irr ? PL.irr_faces[f] : PL.reg_faces[f];
      for (int x = 0; x < G->ncp; ++x) {
        cp[(size_t)q * G->ncp + x] = pack_cp(F.cp[x], F.img[x]);
        slot_vertex.push_back(F.cp[x]);
        ++counts[F.cp[x]];
      }
      const std::vector<double> &G0 = s.irr ? PL.irr_g0 : PL.reg_g0, &RR = s.irr ? PL.irr_RuRv0 : PL.reg_RuRv0;
      for (int p = 0; p < G->npt; ++p) {
        g0[(size_t)q * G->npt + p] = G0[(size_t)f * G->npt + p];
        rr0[(size_t)q * G->npt + p] = RR[(size_t)f * G->npt + p];
      }
      const double *O = &(s.irr ? PL.irr_outer : PL.reg_outer)[(size_t)f * nt];
      const double *I = &(s.irr ? PL.irr_inner : PL.reg_inner)[(size_t)f * nt];
      composition_coeffs(O, I, PL.lipids, &comp[3 * q], &comp[3 * q + 1], &comp[3 * q + 2]);
    }
    // basis rows u,v,uu,uv,vv as [pt][kind][cp], cp padded with zeros to a multiple of 4
    const int ncpp = (G->ncp + 3) / 4 * 4;
    std::vector<double> basis((size_t)G->npt * 5 * ncpp, 0.0);
    for (int p = 0; p < G->npt; ++p)
      for (int k = 0; k < 5; ++k)
        for (int x = 0; x < G->ncp; ++x) basis[((size_t)p * 5 + k) * ncpp + x] = B.at(k + 1, p, x);
    G->tc = prm->precision == UMCP_FP32_CENTRED && prm->face_kernel == 1 && G->ncp == 12 && G->npt == 15;
    G->nblocks = group_blocks(prm->precision, G->tc, G->ncp, G->npt, G->nfaces);
    G->block_base = block_base;
    block_base += G->nblocks;
    block_rows += group_block_rows(prm->precision, G->ncp, G->npt, G->nfaces);
    arena.stage(G->cp, cp);
    arena.stage(G->basis, basis);
    if (prm->precision == UMCP_FP32_CENTRED) {  // the precision form's kernels read only the FP32 copies
      arena.stage(G->g0f, std::vector<float>(g0.begin(), g0.end()));
      arena.stage(G->rr0f, std::vector<float>(rr0.begin(), rr0.end()));
      arena.stage(G->compf, std::vector<float>(comp.begin(), comp.end()));
    } else {
      arena.stage(G->g0, g0);
      arena.stage(G->rr0, rr0);
      arena.stage(G->comp, comp);
    }
    arena.stage(G->weight, B.weight);
    {
      std::vector<double> bw((size_t)G->npt * G->ncp);
      for (int p = 0; p < G->npt; ++p)
        for (int x = 0; x < G->ncp; ++x) bw[(size_t)p * G->ncp + x] = B.at(0, p, x);
      arena.stage(G->basis_w, bw);
    }
    face_base += G->nfaces;
    slot_base += G->nfaces * G->ncp;
    m->groups.push_back(std::move(G));
  }
  m->nfaces = face_base;
  m->nslots = slot_base;
  // Destination of every (face, control point) slot in the interleaved
  // numbering: the k-th slot of vertex v at loc[2 v] + 32 k, in ascending
  // order of (face, control point), which is the order the gather sums them.
  std::vector<int> off, dest(slot_base, -1), kth(ME.nv, 0);
  m->nslot_cap = (int)interleave_slots(counts, &off);
  for (int q = 0; q < slot_base; ++q) {
    const int v = slot_vertex[q];
    dest[q] = off[2 * (size_t)v] + 32 * kth[v]++;
  }
  for (auto &G : m->groups) {
    std::vector<int> d(dest.begin() + G->slot_base, dest.begin() + G->slot_base + (size_t)G->nfaces * G->ncp);
    arena.stage(G->dest, d);
  }
  arena.stage(m->off, off);
  m->nblocks = block_base;
  arena.zeroed(m->blockpart, (size_t)(block_rows > 0 ? block_rows : 1) * 6 * sizeof(double));
  const size_t elem = (m->precision == UMCP_FP64) ? sizeof(double) : sizeof(float);
  arena.uninit(m->partial, (size_t)m->nslot_cap * 3 * elem);
  const size_t nst = 3 * (size_t)ME.nv + 3;
  // Initial state: the plan's positions, alpha = 1.
  std::vector<double> r0(nst);
  std::copy(ME.r.begin(), ME.r.end(), r0.begin());
  r0[3 * ME.nv] = r0[3 * ME.nv + 1] = r0[3 * ME.nv + 2] = 1.0;
  arena.stage(m->r, r0);
  arena.uninit(m->g, nst * sizeof(double));
  arena.zeroed(m->p, 3 * (size_t)ME.nv * sizeof(double));
  arena.uninit(m->qdot, 3 * (size_t)ME.nv * sizeof(double));
  arena.uninit(m->E, sizeof(double));
  arena.uninit(m->parts, 3 * sizeof(double));
  arena.zeroed(m->status, sizeof(int));
  arena.uninit(m->cnt, 2 * sizeof(uint64_t));
  arena.uninit(m->r_eval, nst * sizeof(double));
  arena.zeroed(m->done, sizeof(unsigned));
  arena.uninit(m->alphas, 3 * sizeof(double));
  if (m->precision == UMCP_FP32_CENTRED) {
    arena.uninit(m->rhi, 3 * (size_t)ME.nv * sizeof(float));
    arena.uninit(m->rlo, 3 * (size_t)ME.nv * sizeof(float));
    arena.stage(m->r0, PL.ref_r);  // the state the reference metric g0 was taken at
    arena.uninit(m->dsp, 3 * (size_t)ME.nv * sizeof(float));
  }
  UMCP_CUDA(arena.commit(m->arena));
  if (m->precision == UMCP_FP32_CENTRED) {
    // On the legacy stream, which does not wait for (or stall) work queued on
    // the context's non-blocking stream, e.g. a batch a server is running.
    UMCP_CUDA(launch_split_positions(3 * ME.nv, m->r.as<double>(), m->f32pos(), 0));
    UMCP_CUDA(cudaStreamSynchronize(0));
    m->split_valid = true;
  }
  *out = m.release();
  ctx_retain(ctx);
  return UMCP_OK;
}

extern "C" void umcp_mesh_destroy(umcp_mesh *mesh) {
  if (!mesh) return;
  cudaSetDevice(mesh->ctx->device);
  cudaStreamSynchronize(mesh->ctx->stream);
  if (mesh->batch) batch_forget_mesh(mesh->batch, mesh);
  umcp_ctx *ctx = mesh->ctx;
  delete mesh;
  ctx_release(ctx);
}

extern "C" umcp_status umcp_mesh_set_params(umcp_mesh *mesh, const umcp_params *p) {
  if (!mesh || !p) return fail(UMCP_ERR_INVALID, "null argument");
  fill_params(mesh, p);
  mesh->drop_graphs();
  if (mesh->batch) batch_mesh_changed(mesh->batch);  // its job entry holds the parameters
  return UMCP_OK;
}

// Slot numbering of the gradient partials. Vertices go in groups of 32 (one
// warp of the gather); slot k of vertex 32 g + t is base_g + 32 k + t, and
// base_g advances by 32 times the group's largest slot count. A warp's gather
// then reads 32 consecutive slots per k instead of 32 strided runs. Fills
// loc[2 v] = base_g + t and loc[2 v + 1] = count of v; returns the slots to
// allocate (the padding slots are neither written nor read).
size_t umcp::interleave_slots(const std::vector<int> &counts, std::vector<int> *loc) {
  const size_t nv = counts.size();
  loc->assign(2 * nv, 0);
  size_t base = 0;
  for (size_t g0 = 0; g0 < nv; g0 += 32) {
    const size_t g1 = std::min(nv, g0 + 32);
    int most = 0;
    for (size_t v = g0; v < g1; ++v) most = std::max(most, counts[v]);
    for (size_t v = g0; v < g1; ++v) {
      (*loc)[2 * v] = (int)(base + (v - g0));
      (*loc)[2 * v + 1] = counts[v];
    }
    base += 32 * (size_t)most;
  }
  return base;
}

int umcp::group_blocks(int precision, bool tc, int ncp, int npt, int nfaces) {
  if (tc) return face_blocks_tc(nfaces);
  return precision == UMCP_FP64 ? face_blocks<double>(nfaces, ncp, npt) : face_blocks<float>(nfaces, ncp, npt);
}

int umcp::group_block_rows(int precision, int ncp, int npt, int nfaces) {
  int b = group_blocks(precision, false, ncp, npt, nfaces);
  if (precision == UMCP_FP32_CENTRED && ncp == 12 && npt == 15) b = std::max(b, face_blocks_tc(nfaces));
  return b;
}

// Arguments of the area/volume kernels for state d_r.
static GeoArgs geo_args(umcp_mesh *m, const double *d_r) {
  GeoArgs G{};
  int base = 0;
  for (auto &Gp : m->groups) {
    GeoGroup &g = G.g[G.ngroups++];
    g.cp = Gp->cp.as<uint32_t>();
    g.dest = Gp->dest.as<int>();
    g.basis = Gp->basis.as<double>();
    g.basis_w = Gp->basis_w.as<double>();
    g.weight = Gp->weight.as<double>();
    g.tab = Gp->geo_tab.as<float>();
    g.ncp = Gp->ncp;
    g.npt = Gp->npt;
    g.ncpp = (Gp->ncp + 3) / 4 * 4;
    g.nfaces = Gp->nfaces;
    g.face_base = base;
    g.dudv = Gp->dudv;
    base += Gp->nfaces;
  }
  G.nfaces = base;
  G.nv = m->nv;
  G.r = d_r;
  G.rhi = m->rhi.as<float>();
  G.rlo = m->rlo.as<float>();
  for (int d = 0; d < 3; ++d)
    for (int c = 0; c < 3; ++c) {
      G.box[d][c] = m->P.box[d][c];
      G.box_hi[d][c] = m->P.box_hi[d][c];
      G.box_lo[d][c] = m->P.box_lo[d][c];
    }
  G.KA = m->rs.KA;
  G.A0 = m->rs.A0;
  G.KV = m->rs.KV;
  G.V0 = m->rs.V0;
  G.block = m->geo_block.as<double>();
  G.gterm = m->gterm.as<double>();
  G.done = m->geo_done.as<unsigned>();
  return G;
}

// Face launches of an evaluation at d_r. With restraints on, the area and
// volume sums run first (the face pass's finish adds their energy) and their
// gradient is added into the partial slots after it. The irregular groups run
// on the ctx's side stream beside the regular group; every block of every
// launch counts toward the finish (FinishArgs::nblk), so whichever block is
// the last of all sums the block partials.
template <typename T>
static cudaError_t queue_faces(umcp_mesh *m, const double *d_r, const FinishArgs *fin_in) {
  cudaStream_t s = m->ctx->stream;
  FinishArgs none{};
  FinishArgs fin_geo{};
  const FinishArgs *fin = fin_in;
  const bool geo = m->rs.on && fin_in;
  GeoArgs GA{};
  if (geo) {
    GA = geo_args(m, d_r);
    cudaError_t e = launch_geo_sums(GA, m->precision == UMCP_FP64, s);
    if (e != cudaSuccess) return e;
    fin_geo = *fin_in;
    fin_geo.gterm = m->gterm.as<double>();
    fin = &fin_geo;
  }
  const bool fork = m->groups.size() > 1;
  if (fork) {
    cudaError_t e = cudaEventRecord(m->ctx->fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(m->ctx->side, m->ctx->fork, 0);
    if (e != cudaSuccess) return e;
  }
  for (size_t gi = 0; gi < m->groups.size(); ++gi) {
    auto &G = m->groups[gi];
    const cudaStream_t on = (fork && gi > 0) ? m->ctx->side : s;
    dev::FaceLaunch L;
    L.nfaces = G->nfaces;
    L.block_base = G->block_base;
    L.cp = G->cp.as<uint32_t>();
    L.g0 = G->g0.as<double>();
    L.rr0 = G->rr0.as<double>();
    L.comp = G->comp.as<double>();
    L.g0f = G->g0f.as<float>();
    L.rr0f = G->rr0f.as<float>();
    L.compf = G->compf.as<float>();
    L.basis = G->basis.as<double>();
    L.weight = G->weight.as<double>();
    L.dudv = G->dudv;
    L.irregular = G->irregular;
    cudaError_t e;
    if constexpr (sizeof(T) == 4) {
      if (G->tc)
        e = launch_faces_tc(L, G->dest.as<int>(), m->P, d_r, m->rhi.as<float>(), m->rlo.as<float>(),
                            m->dsp.as<float>(), m->partial.as<float>(), m->blockpart.as<double>(), m->status.as<int>(), G->nblocks,
                            fin ? *fin : none, on);
      else
        e = launch_faces<T>(L, G->dest.as<int>(), G->ncp, G->npt, m->P, d_r, m->f32pos(), m->partial.as<T>(), m->blockpart.as<double>(), m->status.as<int>(), G->nblocks,
                            fin ? *fin : none, on);
    } else {
      e = launch_faces<T>(L, G->dest.as<int>(), G->ncp, G->npt, m->P, d_r, m->f32pos(), m->partial.as<T>(), m->blockpart.as<double>(), m->status.as<int>(), G->nblocks,
                          fin ? *fin : none, on);
    }
    if (e != cudaSuccess) return e;
  }
  if (fork) {
    cudaError_t e = cudaEventRecord(m->ctx->join, m->ctx->side);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, m->ctx->join, 0);
    if (e != cudaSuccess) return e;
  }
  if (geo) return launch_geo_grad<T>(GA, m->partial.as<T>(), s);
  return cudaSuccess;
}

// Energy and gradient of state d_r: E -> d_E (parts -> d_parts), gradient
// ADDED into d_g (3*nv+3) when d_g is given.
template <typename T>
static cudaError_t queue_energy_grad(umcp_mesh *m, const double *d_r, double *d_E, double *d_parts, double *d_g,
                                     bool faces_only) {
  cudaStream_t s = m->ctx->stream;
  cudaError_t e = cudaSuccess;
  if (faces_only) {
    if (sizeof(T) == 4 && !m->split_valid)
      e = launch_split_positions(3 * m->nv, m->r.as<double>(), m->f32pos(), s);
    m->split_valid = true;
    return e == cudaSuccess ? queue_faces<T>(m, m->r.as<double>(), nullptr) : e;
  }
  if (sizeof(T) == 4) {
    e = launch_split_positions(3 * m->nv, d_r, m->f32pos(), s);
    m->split_valid = (d_r == m->r.as<double>());
  }
  if (e != cudaSuccess) return e;
  FinishArgs fin{m->nblocks, d_E, d_parts, d_g ? d_g + 3 * m->nv : nullptr, nullptr, nullptr, 0.0,
                 m->status.as<int>(), m->done.as<unsigned>()};
  e = queue_faces<T>(m, d_r, &fin);
  if (e != cudaSuccess) return e;
  if (d_g) e = launch_gather<T>(m->nv, m->partial.as<T>(), m->off.as<int>(), d_g, s);
  return e;
}

static cudaError_t queue_eg(umcp_mesh *m, const double *d_r, double *d_E, double *d_parts, double *d_g,
                            bool faces_only = false) {
  return (m->precision == UMCP_FP64) ? queue_energy_grad<double>(m, d_r, d_E, d_parts, d_g, faces_only)
                                     : queue_energy_grad<float>(m, d_r, d_E, d_parts, d_g, faces_only);
}

static umcp_status check_status(umcp_mesh *m) {
  int st = 0;
  UMCP_CUDA(cudaMemcpyAsync(&st, m->status.p, sizeof(int), cudaMemcpyDeviceToHost, m->ctx->stream));
  UMCP_CUDA(cudaStreamSynchronize(m->ctx->stream));
  if (st & kStatusNonFinite) return fail(UMCP_ERR_NONFINITE, "non-finite energy (the reference stops with \"nan en.\")");
  if (st & kStatusDiverged) return fail(UMCP_ERR_DIVERGED, "energy rose above the divergence threshold");
  if (st & kStatusTimeout) return fail(UMCP_ERR_TIMEOUT, "a tensor-core wait in the face pass gave up");
  return UMCP_OK;
}

static umcp_status host_energy_grad(umcp_mesh *m, const double *r, double *E, double *terms, double *g) {
  if (!m || !r) return fail(UMCP_ERR_INVALID, "null argument");
  UMCP_CUDA(cudaSetDevice(m->ctx->device));
  UMCP_CUDA(ensure_pinned(m));
  cudaStream_t s = m->ctx->stream;
  const size_t nst = 3 * (size_t)m->nv + 3;
  memcpy(m->h_stage, r, nst * sizeof(double));
  UMCP_CUDA(cudaMemcpyAsync(m->r_eval.p, m->h_stage, nst * sizeof(double), cudaMemcpyHostToDevice, s));
  UMCP_CUDA(cudaMemsetAsync(m->status.p, 0, sizeof(int), s));
  if (g) UMCP_CUDA(cudaMemsetAsync(m->g.p, 0, nst * sizeof(double), s));
  UMCP_CUDA(queue_eg(m, m->r_eval.as<double>(), m->E.as<double>(), m->parts.as<double>(),
                     g ? m->g.as<double>() : nullptr));
  double e_parts[4];
  UMCP_CUDA(cudaMemcpyAsync(&e_parts[0], m->E.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  UMCP_CUDA(cudaMemcpyAsync(&e_parts[1], m->parts.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (g) UMCP_CUDA(cudaMemcpyAsync(m->h_stage, m->g.p, nst * sizeof(double), cudaMemcpyDeviceToHost, s));
  umcp_status st = check_status(m);  // synchronizes
  if (E) *E = e_parts[0];
  if (terms) { terms[0] = e_parts[1]; terms[1] = e_parts[2]; terms[2] = e_parts[3]; }
  if (g)
    for (size_t i = 0; i < nst; ++i) g[i] += m->h_stage[i];
  return st;
}

extern "C" umcp_status umcp_energy(umcp_mesh *mesh, const double *r, double *E, double *terms) {
  return host_energy_grad(mesh, r, E, terms, nullptr);
}
extern "C" umcp_status umcp_grad(umcp_mesh *mesh, const double *r, double *g) {
  if (!g) return fail(UMCP_ERR_INVALID, "null gradient");
  return host_energy_grad(mesh, r, nullptr, nullptr, g);
}
extern "C" umcp_status umcp_energy_grad(umcp_mesh *mesh, const double *r, double *E, double *g) {
  return host_energy_grad(mesh, r, E, nullptr, g);
}

extern "C" umcp_status umcp_face_pass(umcp_mesh *m) {
  if (!m) return fail(UMCP_ERR_INVALID, "null mesh");
  UMCP_CUDA(cudaSetDevice(m->ctx->device));
  UMCP_CUDA(queue_eg(m, m->r.as<double>(), m->E.as<double>(), m->parts.as<double>(), nullptr, /*faces_only=*/true));
  return UMCP_OK;
}

extern "C" umcp_status umcp_mesh_info_get(const umcp_mesh *m, umcp_mesh_info *info) {
  if (!m || !info) return fail(UMCP_ERR_INVALID, "null argument");
  info->nv = m->nv;
  info->n_faces = m->nfaces;
  int npts = 0;
  for (auto &G : m->groups) npts += G->nfaces * G->npt;
  info->n_points = npts;
  info->n_slots = m->nslots;
  const int groups = (int)m->groups.size();
  // face kernels (the last one also sums the energy) + fused gather/update;
  // the mass path replaces the fused kernel with memset + gather + kick + spmv + drift.
  info->kernels_per_step = groups + 1;
  info->kernels_per_step_mass = groups + 5;
  info->precision = m->precision;
  info->device_bytes = (long long)m->device_bytes();
  // bytes umcp_mesh_create copied in: face tables, bases, slot offsets, positions
  long long h2d = (long long)(m->off.bytes + (3 * (size_t)m->nv + 3) * sizeof(double));
  for (auto &G : m->groups)
    for (const DevBuf *x : {&G->cp, &G->g0, &G->rr0, &G->comp, &G->basis, &G->weight, &G->dest, &G->g0f, &G->rr0f,
                            &G->compf, &G->basis_w})
      h2d += (long long)x->bytes;
  info->h2d_bytes = h2d;
  info->mass_form = !m->mrows ? 0 : m->mass_dense ? 1 : 2;
  return UMCP_OK;
}

// Device bytes umcp_mesh_create allocates for a plan, plus the energy record
// of a run of n_energies steps: the same sizes, buffer by buffer.
extern "C" umcp_status umcp_plan_device_bytes(const umcp_plan *plan, umcp_ctx *ctx, int precision,
                                              int64_t n_energies, size_t *bytes) {
  if (!plan || !ctx || !bytes || n_energies < 0) return fail(UMCP_ERR_INVALID, "bad argument");
  if (precision != UMCP_FP64 && precision != UMCP_FP32_CENTRED) return fail(UMCP_ERR_INVALID, "unknown precision");
  UMCP_CUDA(cudaSetDevice(ctx->device));
  const Plan &PL = plan->plan;
  const size_t nv = (size_t)plan->mesh.nv, nst = 3 * nv + 3;
  const bool f32 = precision == UMCP_FP32_CENTRED;
  size_t b = 0;
  int nblocks = 0;
  std::vector<int> counts(nv, 0), loc;
  for (const Face &F : PL.reg_faces)
    for (int x = 0; x < PL.regular.ncp; ++x) ++counts[F.cp[x]];
  for (const Face &F : PL.irr_faces)
    for (int x = 0; x < PL.irregular[F.valence].ncp; ++x) ++counts[F.cp[x]];
  const size_t slots = interleave_slots(counts, &loc);
  auto group = [&](const PatchBasis &B, size_t nf) {
    const size_t ncpp = (size_t)(B.ncp + 3) / 4 * 4;
    b += nf * B.ncp * 4 + (size_t)B.npt * 5 * ncpp * 8 + B.weight.size() * 8 + nf * B.ncp * 4 +
         (size_t)B.npt * B.ncp * 8;
    const size_t es = f32 ? 4 : 8;  // g0, reference angles and composition in the form's own type
    b += 2 * nf * B.npt * es + nf * 3 * es;
    nblocks += group_block_rows(precision, B.ncp, B.npt, (int)nf);
  };
  group(PL.regular, PL.reg_faces.size());
  for (int val : {5, 7}) {
    size_t nf = 0;
    for (const Face &F : PL.irr_faces) nf += F.valence == val;
    if (nf) group(PL.irregular[val], nf);
  }
  b += 2 * nv * 4;                                    // slot locations
  b += (size_t)std::max(nblocks, 1) * 6 * 8;          // blockpart
  b += slots * 3 * (f32 ? 4 : 8);                     // partial
  b += 3 * nst * 8 + 2 * 3 * nv * 8;                  // r, g, r_eval; p, qdot
  b += 8 + 3 * 8 + 4 + 2 * 8 + 4 + 3 * 8;             // E, parts, status, cnt, done, alphas
  if (f32) b += 3 * 3 * nv * 4 + 3 * nv * 8;          // rhi, rlo, dsp; r0
  b += (size_t)n_energies * 8;                        // energy record
  *bytes = b;
  return UMCP_OK;
}

extern "C" umcp_status umcp_energy_grad_device(umcp_mesh *m, const double *d_r, double *d_E, double *d_g) {
  if (!m || !d_r) return fail(UMCP_ERR_INVALID, "null argument");
  UMCP_CUDA(cudaSetDevice(m->ctx->device));
  UMCP_CUDA(queue_eg(m, d_r, d_E ? d_E : m->E.as<double>(), m->parts.as<double>(), d_g));
  return UMCP_OK;
}

// ------------------------------------------------------------------ effective mass

extern "C" umcp_status umcp_mass_set(umcp_mesh *m, int nrow, const int *row_ptr, const int *col, const double *val) {
  if (!m || !row_ptr || !col || !val || nrow != m->nv) return fail(UMCP_ERR_INVALID, "mass matrix must have nv rows");
  int nnz = row_ptr[nrow];
  for (int i = 0; i < nrow; ++i)
    if (row_ptr[i + 1] < row_ptr[i]) return fail(UMCP_ERR_INVALID, "row_ptr not monotone");
  for (int k = 0; k < nnz; ++k)
    if (col[k] < 0 || col[k] >= m->nv) return fail(UMCP_ERR_INVALID, "column index out of range");
  UMCP_CUDA(cudaSetDevice(m->ctx->device));
  UMCP_CUDA(upload(m->mrow, std::vector<int>(row_ptr, row_ptr + nrow + 1)));
  m->mass_f32 = m->precision == UMCP_FP32_CENTRED;  // the precision form applies M^-1 in FP32
  m->mcol16 = m->mass_f32 && nrow <= 65536;         // and stores its columns in 16 bits when they fit
  if (m->mcol16) UMCP_CUDA(upload(m->mcol, std::vector<uint16_t>(col, col + nnz)));
  else UMCP_CUDA(upload(m->mcol, std::vector<int>(col, col + nnz)));
  if (m->mass_f32) UMCP_CUDA(upload(m->mval, std::vector<float>(val, val + nnz)));
  else UMCP_CUDA(upload(m->mval, std::vector<double>(val, val + nnz)));
  UMCP_CUDA(m->min32.alloc(m->mass_f32 ? (size_t)nrow * sizeof(float4) : 0));
  UMCP_CUDA(m->mdense.alloc(0));
  m->mass_dense = false;
  m->mrows = nrow;
  m->drop_graphs();
  return UMCP_OK;
}

extern "C" umcp_status umcp_mass_apply_device(umcp_mesh *m, const double *d_in, double *d_out, const double *d_scalev,
                                              double scale, const double *alphas) {
  if (!m || !d_in || !d_out) return fail(UMCP_ERR_INVALID, "null argument");
  if (!m->mrows) return fail(UMCP_ERR_INVALID, "no mass matrix installed");
  UMCP_CUDA(cudaSetDevice(m->ctx->device));
  double a[3] = {1, 1, 1};
  if (alphas) { a[0] = alphas[0]; a[1] = alphas[1]; a[2] = alphas[2]; }
  UMCP_CUDA(cudaMemcpyAsync(m->alphas.p, a, sizeof a, cudaMemcpyHostToDevice, m->ctx->stream));
  UMCP_CUDA(queue_mass_apply(m, d_scalev, scale, m->alphas.as<double>(), d_in, d_out, 1, m->ctx->stream));
  UMCP_CUDA(cudaStreamSynchronize(m->ctx->stream));
  return UMCP_OK;
}

extern "C" umcp_status umcp_mass_apply(umcp_mesh *m, const double *in, double *out, const double *scalev, double scale,
                                       const double *alphas) {
  if (!m || !in || !out) return fail(UMCP_ERR_INVALID, "null argument");
  if (!m->mrows) return fail(UMCP_ERR_INVALID, "no mass matrix installed");
  UMCP_CUDA(cudaSetDevice(m->ctx->device));
  cudaStream_t s = m->ctx->stream;
  const size_t n3 = 3 * (size_t)m->nv;
  DevBuf din, dout, dsc;
  UMCP_CUDA(din.alloc(n3 * sizeof(double)));
  UMCP_CUDA(dout.alloc(n3 * sizeof(double)));
  UMCP_CUDA(cudaMemcpyAsync(din.p, in, n3 * sizeof(double), cudaMemcpyHostToDevice, s));
  UMCP_CUDA(cudaMemcpyAsync(dout.p, out, n3 * sizeof(double), cudaMemcpyHostToDevice, s));
  if (scalev) {
    UMCP_CUDA(dsc.alloc(n3 * sizeof(double)));
    UMCP_CUDA(cudaMemcpyAsync(dsc.p, scalev, n3 * sizeof(double), cudaMemcpyHostToDevice, s));
  }
  double a[3] = {1, 1, 1};
  if (alphas) { a[0] = alphas[0]; a[1] = alphas[1]; a[2] = alphas[2]; }
  UMCP_CUDA(cudaMemcpyAsync(m->alphas.p, a, sizeof a, cudaMemcpyHostToDevice, s));
  UMCP_CUDA(queue_mass_apply(m, scalev ? dsc.as<double>() : nullptr, scale, m->alphas.as<double>(),
                             din.as<double>(), dout.as<double>(), 1, s));
  UMCP_CUDA(cudaMemcpyAsync(out, dout.p, n3 * sizeof(double), cudaMemcpyDeviceToHost, s));
  UMCP_CUDA(cudaStreamSynchronize(s));
  return UMCP_OK;
}

// ------------------------------------------------------------------ dynamics


extern "C" umcp_status umcp_state_set(umcp_mesh *m, const double *r, const double *p) {
  if (!m) return fail(UMCP_ERR_INVALID, "null mesh");
  UMCP_CUDA(cudaSetDevice(m->ctx->device));
  const size_t nst = 3 * (size_t)m->nv + 3;
  if (r) UMCP_CUDA(cudaMemcpyAsync(m->r.p, r, nst * sizeof(double), cudaMemcpyHostToDevice, m->ctx->stream));
  if (r && m->precision == UMCP_FP32_CENTRED) {
    UMCP_CUDA(launch_split_positions(3 * m->nv, m->r.as<double>(), m->f32pos(), m->ctx->stream));
    m->split_valid = true;
  }
  if (p) UMCP_CUDA(cudaMemcpyAsync(m->p.p, p, (nst - 3) * sizeof(double), cudaMemcpyHostToDevice, m->ctx->stream));
  else UMCP_CUDA(cudaMemsetAsync(m->p.p, 0, (nst - 3) * sizeof(double), m->ctx->stream));
  UMCP_CUDA(cudaStreamSynchronize(m->ctx->stream));
  return UMCP_OK;
}

extern "C" umcp_status umcp_state_get(umcp_mesh *m, double *r, double *p) {
  if (!m) return fail(UMCP_ERR_INVALID, "null mesh");
  UMCP_CUDA(cudaSetDevice(m->ctx->device));
  const size_t nst = 3 * (size_t)m->nv + 3;
  if (r) UMCP_CUDA(cudaMemcpyAsync(r, m->r.p, nst * sizeof(double), cudaMemcpyDeviceToHost, m->ctx->stream));
  if (p) UMCP_CUDA(cudaMemcpyAsync(p, m->p.p, (nst - 3) * sizeof(double), cudaMemcpyDeviceToHost, m->ctx->stream));
  UMCP_CUDA(cudaStreamSynchronize(m->ctx->stream));
  return UMCP_OK;
}

extern "C" umcp_status umcp_restraints_set(umcp_mesh *m, const umcp_restraints *rs) {
  if (!m) return fail(UMCP_ERR_INVALID, "null mesh");
  if (m->batch) return fail(UMCP_ERR_INVALID, "remove the mesh from its batch first");
  UMCP_CUDA(cudaSetDevice(m->ctx->device));
  cudaStream_t s = m->ctx->stream;
  UMCP_CUDA(cudaStreamSynchronize(s));  // captured steps hold the previous setting
  m->drop_graphs();
  if (!rs || (rs->K_area == 0.0 && rs->K_volume == 0.0)) {
    m->rs = umcp_mesh::Restraints{};
    return UMCP_OK;
  }
  if (rs->K_area < 0 || rs->K_volume < 0) return fail(UMCP_ERR_INVALID, "restraint constants must be >= 0");
  if (rs->K_volume != 0.0)
    for (auto &G : m->groups) {
      std::vector<uint32_t> cp((size_t)G->nfaces * G->ncp);
      if (!cp.empty())
        UMCP_CUDA(cudaMemcpy(cp.data(), G->cp.p, cp.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
      const uint32_t home = (uint32_t)13 << dev::kVertexBits;  // image code of (0,0,0)
      for (uint32_t c : cp)
        if ((c & ~dev::kVertexMask) != home)
          return fail(UMCP_ERR_INVALID, "a volume restraint needs a closed surface (this mesh is periodic)");
    }
  if (m->precision == UMCP_FP32_CENTRED)
    for (auto &G : m->groups) {
      if (G->geo_tab.p || G->nfaces == 0) continue;
      // FP32 tables of the restraint kernels: the value and first-derivative
      // rows split as hi + lo, and the point weights
      const int ncp = G->ncp, npt = G->npt, ncpp = (ncp + 3) / 4 * 4;
      std::vector<double> basis((size_t)npt * 5 * ncpp), bw((size_t)npt * ncp), w(npt);
      UMCP_CUDA(cudaMemcpy(basis.data(), G->basis.p, basis.size() * sizeof(double), cudaMemcpyDeviceToHost));
      UMCP_CUDA(cudaMemcpy(bw.data(), G->basis_w.p, bw.size() * sizeof(double), cudaMemcpyDeviceToHost));
      UMCP_CUDA(cudaMemcpy(w.data(), G->weight.p, w.size() * sizeof(double), cudaMemcpyDeviceToHost));
      std::vector<float> tab(geo_tab_floats(ncp, npt));
      const size_t nrow = (size_t)npt * 3 * ncp;
      for (int p = 0; p < npt; ++p)
        for (int k = 0; k < 3; ++k)
          for (int x = 0; x < ncp; ++x) {
            const double b = k == 0 ? bw[(size_t)p * ncp + x] : basis[((size_t)p * 5 + (k - 1)) * ncpp + x];
            const size_t i = ((size_t)p * 3 + k) * ncp + x;
            tab[i] = (float)b;
            tab[nrow + i] = (float)(b - (double)tab[i]);
          }
      for (int p = 0; p < npt; ++p) {
        const double cw = G->dudv * w[p], c3 = cw / 3.0;
        tab[2 * nrow + p] = (float)cw;
        tab[2 * nrow + npt + p] = (float)c3;
        tab[2 * nrow + 2 * npt + p] = (float)(c3 - (double)(float)c3);
      }
      UMCP_CUDA(upload(G->geo_tab, tab));
    }
  if (!m->gterm.p) {
    int nblk = geo_blocks(m->nfaces);
    UMCP_CUDA(m->geo_block.alloc((size_t)nblk * kGeoWords * sizeof(double)));
    UMCP_CUDA(m->gterm.alloc(kGeoWords * sizeof(double)));
    UMCP_CUDA(m->geo_done.alloc(sizeof(unsigned)));
    UMCP_CUDA(cudaMemset(m->geo_done.p, 0, sizeof(unsigned)));
  }
  umcp_mesh::Restraints R;
  R.on = true;
  R.KA = rs->K_area;
  R.KV = rs->K_volume;
  R.A0 = rs->area0;
  R.V0 = rs->volume0;
  if (R.A0 < 0 || R.V0 < 0) {
    // targets from the resident state: one sums pass with the constants off
    m->rs = umcp_mesh::Restraints{true, 0, 1, 0, 0};
    // the precision form's sums read the hi/lo pairs, which may hold the last evaluated state
    if (m->precision == UMCP_FP32_CENTRED && !m->split_valid)
      UMCP_CUDA(launch_split_positions(3 * m->nv, m->r.as<double>(), m->f32pos(), s));
    m->split_valid = true;
    UMCP_CUDA(launch_geo_sums(geo_args(m, m->r.as<double>()), m->precision == UMCP_FP64, s));
    double gt[kGeoWords];
    UMCP_CUDA(cudaMemcpyAsync(gt, m->gterm.p, sizeof gt, cudaMemcpyDeviceToHost, s));
    UMCP_CUDA(cudaStreamSynchronize(s));
    if (R.A0 < 0) R.A0 = gt[kGeoA];
    if (R.V0 < 0) R.V0 = gt[kGeoV];
  }
  if (!(R.A0 > 0) && R.KA != 0) return fail(UMCP_ERR_INVALID, "area restraint needs area0 > 0");
  m->rs = R;
  return UMCP_OK;
}

extern "C" umcp_status umcp_restraints_get(umcp_mesh *m, double *area, double *volume, double *energy) {
  if (!m) return fail(UMCP_ERR_INVALID, "null mesh");
  if (!m->rs.on) return fail(UMCP_ERR_INVALID, "no restraints set");
  UMCP_CUDA(cudaSetDevice(m->ctx->device));
  double gt[kGeoWords];
  UMCP_CUDA(cudaMemcpyAsync(gt, m->gterm.p, sizeof gt, cudaMemcpyDeviceToHost, m->ctx->stream));
  UMCP_CUDA(cudaStreamSynchronize(m->ctx->stream));
  if (area) *area = gt[kGeoA];
  if (volume) *volume = gt[kGeoV];
  if (energy) *energy = gt[kGeoE];
  return UMCP_OK;
}

extern "C" umcp_status umcp_mesh_energies(umcp_mesh *m, double *energies, int64_t n) {
  if (!m || (n > 0 && !energies) || n < 0) return fail(UMCP_ERR_INVALID, "bad argument");
  if ((size_t)n > m->energies_cap) return fail(UMCP_ERR_INVALID, "more energies asked for than the run records");
  UMCP_CUDA(cudaSetDevice(m->ctx->device));
  if (n > 0)
    UMCP_CUDA(cudaMemcpyAsync(energies, m->energies.p, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost,
                              m->ctx->stream));
  UMCP_CUDA(cudaStreamSynchronize(m->ctx->stream));
  return UMCP_OK;
}

umcp_status umcp::make_step_args(const umcp_mesh *m, const umcp_integrator *it, StepArgs *a) {
  if (it->kind < 0 || it->kind > 2) return fail(UMCP_ERR_INVALID, "unknown integrator kind");
  if (!(it->time_step > 0)) return fail(UMCP_ERR_INVALID, "time_step must be positive");
  if (it->use_mass && !m->mrows) return fail(UMCP_ERR_INVALID, "use_mass set but no mass matrix installed");
  if (it->kind == 0 && !(it->D > 0)) return fail(UMCP_ERR_INVALID, "overdamped BD needs D > 0");
  if (it->kind != 0 && !(it->gamma > 0)) return fail(UMCP_ERR_INVALID, "leapfrog integrators need gamma > 0");
  *a = StepArgs{};
  a->kind = it->kind;
  a->seed = it->seed;
  a->stream = it->stream;
  a->gamma = it->gamma;
  a->AK = kAkmaTime * it->time_step;
  if (it->kind == 0) {
    a->mob_dt = it->D * it->time_step / m->kT;
    a->sigma = std::sqrt(2.0 * it->D * it->time_step);
    a->mob_dt_f = (float)a->mob_dt;
    a->sigma_f = (float)a->sigma;
  } else {
    a->sigma = std::sqrt(2.0 * it->gamma * m->kT * a->AK);
  }
  return UMCP_OK;
}

// One step on the resident state: energy and gradient at r(t), then the update.
template <typename T>
static cudaError_t queue_step_t(umcp_mesh *m, const StepArgs &a, int use_mass, double threshold) {
  cudaStream_t s = m->ctx->stream;
  FinishArgs fin{m->nblocks, m->E.as<double>(), m->parts.as<double>(), nullptr, m->energies.as<double>(),
                 m->cnt.as<uint64_t>(), threshold, m->status.as<int>(), m->done.as<unsigned>()};
  cudaError_t e = queue_faces<T>(m, m->r.as<double>(), &fin);
  if (e != cudaSuccess) return e;
  if (a.kind == 0 || !use_mass)
    return launch_gather_step<T>(m->nv, m->partial.as<T>(), m->off.as<int>(), a, m->cnt.as<uint64_t>(),
                                 m->r.as<double>(), m->p.as<double>(), m->f32pos(), m->status.as<int>(), s);
  e = cudaMemsetAsync(m->g.p, 0, 3 * (size_t)m->nv * sizeof(double), s);
  if (e == cudaSuccess) e = launch_gather<T>(m->nv, m->partial.as<T>(), m->off.as<int>(), m->g.as<double>(), s);
  if (e == cudaSuccess)
    e = launch_kick(m->nv, a, m->cnt.as<uint64_t>(), m->p.as<double>(), m->g.as<double>(), m->status.as<int>(), s);
  if (e == cudaSuccess)
    e = queue_mass_apply(m, nullptr, 1.0, nullptr, m->p.as<double>(), m->qdot.as<double>(), 0, s);
  if (e == cudaSuccess)
    e = launch_drift(m->nv, a, m->r.as<double>(), m->p.as<double>(), m->qdot.as<double>(), m->f32pos(),
                     m->status.as<int>(), s);
  return e;
}

static cudaError_t queue_step(umcp_mesh *m, const StepArgs &a, int use_mass, double threshold) {
  return (m->precision == UMCP_FP64) ? queue_step_t<double>(m, a, use_mass, threshold)
                                     : queue_step_t<float>(m, a, use_mass, threshold);
}

static bool same_args(const StepArgs &x, const StepArgs &y) { return memcmp(&x, &y, sizeof(StepArgs)) == 0; }

static umcp_status graph_for(umcp_mesh *m, const StepArgs &a, int use_mass, double threshold, int steps,
                             cudaGraphExec_t *out) {
  for (auto &g : m->graphs)
    if (g.steps == steps && g.use_mass == use_mass && g.threshold == threshold && same_args(g.args, a)) {
      *out = g.exec;
      return UMCP_OK;
    }
  cudaStream_t s = m->ctx->stream;
  cudaGraph_t g;
  UMCP_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < steps && e == cudaSuccess; ++i) e = queue_step(m, a, use_mass, threshold);
  cudaError_t e2 = cudaStreamEndCapture(s, &g);
  if (e != cudaSuccess) return fail(UMCP_ERR_CUDA, std::string("step capture: ") + cudaGetErrorString(e));
  if (e2 != cudaSuccess) return fail(UMCP_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(e2));
  umcp_mesh::CachedGraph cg;
  e = cudaGraphInstantiate(&cg.exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(UMCP_ERR_CUDA, std::string("graph: ") + cudaGetErrorString(e));
  cg.steps = steps;
  cg.args = a;
  cg.use_mass = use_mass;
  cg.threshold = threshold;
  m->graphs.push_back(cg);
  *out = cg.exec;
  return UMCP_OK;
}

static umcp_status run_steps(umcp_mesh *m, const umcp_integrator *it, uint64_t step0, int n_steps) {
  cudaStream_t s = m->ctx->stream;
  StepArgs a;
  umcp_status st = make_step_args(m, it, &a);
  if (st != UMCP_OK) return st;
  if ((size_t)n_steps > m->energies_cap) {
    m->drop_graphs();  // graphs hold the energies pointer
    UMCP_CUDA(m->energies.alloc((size_t)n_steps * sizeof(double)));
    m->energies_cap = (size_t)n_steps;
    if (m->batch) batch_mesh_changed(m->batch);  // so does its batch job entry
  }
  if (m->precision == UMCP_FP32_CENTRED && !m->split_valid)
    UMCP_CUDA(launch_split_positions(3 * m->nv, m->r.as<double>(), m->f32pos(), s));
  m->split_valid = true;  // every step rewrites the pairs of the new positions
  UMCP_CUDA(ensure_pinned(m));
  m->h_cnt[0] = step0;
  m->h_cnt[1] = 0;
  UMCP_CUDA(cudaMemcpyAsync(m->cnt.p, m->h_cnt, 2 * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
  UMCP_CUDA(cudaMemsetAsync(m->status.p, 0, sizeof(int), s));
  const int use_mass = (it->kind != 0 && it->use_mass) ? 1 : 0;
  // kGraphChunk steps at a time, then the rest as one captured run per set bit
  for (int left = n_steps; left > 0;) {
    int len = kGraphChunk;
    while (len > left) len >>= 1;
    cudaGraphExec_t g;
    st = graph_for(m, a, use_mass, it->divergence_threshold, len, &g);
    if (st != UMCP_OK) return st;
    UMCP_CUDA(cudaGraphLaunch(g, s));
    left -= len;
  }
  return UMCP_OK;
}

extern "C" umcp_status umcp_run(umcp_mesh *m, const umcp_integrator *it, uint64_t step0, int n_steps, double *energies) {
  if (!m || !it || n_steps < 0) return fail(UMCP_ERR_INVALID, "bad argument");
  if (n_steps == 0) return UMCP_OK;
  UMCP_CUDA(cudaSetDevice(m->ctx->device));
  umcp_status st = run_steps(m, it, step0, n_steps);
  if (st != UMCP_OK) return st;
  if (energies)
    UMCP_CUDA(cudaMemcpyAsync(energies, m->energies.p, (size_t)n_steps * sizeof(double), cudaMemcpyDeviceToHost,
                              m->ctx->stream));
  return check_status(m);
}

extern "C" umcp_status umcp_run_async(umcp_mesh *m, const umcp_integrator *it, uint64_t step0, int n_steps) {
  if (!m || !it || n_steps < 0) return fail(UMCP_ERR_INVALID, "bad argument");
  if (n_steps == 0) return UMCP_OK;
  UMCP_CUDA(cudaSetDevice(m->ctx->device));
  return run_steps(m, it, step0, n_steps);
}

extern "C" umcp_status umcp_step_host(umcp_mesh *m, const umcp_integrator *it, uint64_t step, double *r, double *p,
                                      double *E) {
  if (!m || !it || !r) return fail(UMCP_ERR_INVALID, "null argument");
  UMCP_CUDA(cudaSetDevice(m->ctx->device));
  UMCP_CUDA(ensure_pinned(m));
  cudaStream_t s = m->ctx->stream;
  const size_t nst = 3 * (size_t)m->nv + 3;
  memcpy(m->h_stage, r, nst * sizeof(double));
  UMCP_CUDA(cudaMemcpyAsync(m->r.p, m->h_stage, nst * sizeof(double), cudaMemcpyHostToDevice, s));
  m->split_valid = false;  // the precision form's hi/lo pairs still hold the previous state
  if (p) {
    memcpy(m->h_stage2, p, (nst - 3) * sizeof(double));
    UMCP_CUDA(cudaMemcpyAsync(m->p.p, m->h_stage2, (nst - 3) * sizeof(double), cudaMemcpyHostToDevice, s));
  }
  umcp_status st = run_steps(m, it, step, 1);
  if (st != UMCP_OK) return st;
  double e = 0;
  UMCP_CUDA(cudaMemcpyAsync(m->h_stage, m->r.p, nst * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (p) UMCP_CUDA(cudaMemcpyAsync(m->h_stage2, m->p.p, (nst - 3) * sizeof(double), cudaMemcpyDeviceToHost, s));
  UMCP_CUDA(cudaMemcpyAsync(&e, m->E.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  st = check_status(m);
  memcpy(r, m->h_stage, nst * sizeof(double));
  if (p) memcpy(p, m->h_stage2, (nst - 3) * sizeof(double));
  if (E) *E = e;
  return st;
}

// ------------------------------------------------------------------ energy+gradient without allocation
//
// For callers that must not allocate device memory at call time: code that
// runs inside someone else's stream capture (where cudaMalloc is not allowed),
// or that lives under a fixed device-memory budget owned by another runtime.
// The mesh's plan tables (made earlier, at set-up) are the inputs, the
// caller's d_r/d_E/d_g the state and outputs; all scratch of the face pass
// (gradient partials, block sums, the finished-block counter, the status
// word and the FP32 position pairs) lives in this file-scope array, which
// every GPU that loads the library holds until the process exits.

static constexpr size_t kStaticScratchBytes = (size_t)32 << 20;  // 32 MiB per device
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];
static void *g_static_scratch_addr[128];  // device address of the array, per device (host-side)

static size_t align256(size_t x) { return (x + 255) / 256 * 256; }

extern "C" umcp_status umcp_energy_grad_static(umcp_mesh *m, const double *d_r, double *d_E, double *d_g) {
  if (!m || !d_r) return fail(UMCP_ERR_INVALID, "null argument");
  if (!d_E) d_E = m->E.as<double>();  // allocated with the mesh
  if (m->rs.on) return fail(UMCP_ERR_UNSUPPORTED, "the static entry point has no area/volume restraint terms");
  const int dev = m->ctx->device;
  if (dev < 0 || dev >= 128) return fail(UMCP_ERR_INVALID, "device index out of range for the static scratch table");
  UMCP_CUDA(cudaSetDevice(dev));
  // Host code cannot use the array's name as a device address; look the
  // address up once per device, with that device current.
  if (!g_static_scratch_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p)
      return fail(UMCP_ERR_CUDA, std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e));
    g_static_scratch_addr[dev] = p;
  }
  unsigned char *base = (unsigned char *)g_static_scratch_addr[dev];
  const bool fp32 = (m->precision == UMCP_FP32_CENTRED);
  const size_t esize = fp32 ? sizeof(float) : sizeof(double);
  // layout: [status, done] | block partials | gradient partials | FP32 position pairs and displacements
  const size_t off_flags = 0, off_block = 256;
  const size_t off_partial = off_block + align256((size_t)m->nblocks * 6 * sizeof(double));
  const size_t f32_bytes = fp32 ? align256((size_t)3 * m->nv * sizeof(float)) : 0;
  const size_t off_hi = off_partial + align256((size_t)m->nslot_cap * 3 * esize);
  const size_t off_lo = off_hi + f32_bytes, off_dsp = off_lo + f32_bytes;
  const size_t need = off_dsp + f32_bytes;
  if (need > kStaticScratchBytes)
    return fail(UMCP_ERR_NOMEM, "mesh needs " + std::to_string(need) + " bytes of scratch; the static area holds " +
                                    std::to_string(kStaticScratchBytes) + " bytes");
  int *status = (int *)(base + off_flags);
  unsigned *done = (unsigned *)(base + off_flags + sizeof(int));
  double *blockpart = (double *)(base + off_block);
  F32Pos f32;
  if (fp32) {
    f32.hi = (float *)(base + off_hi);
    f32.lo = (float *)(base + off_lo);
    f32.r0 = m->r0.as<double>();
    f32.dsp = (float *)(base + off_dsp);
  }
  float *rhi = f32.hi, *rlo = f32.lo;
  cudaStream_t s = m->ctx->stream;
  // The array keeps the previous call's contents: the status word and the
  // finished-block counter must start at zero.
  UMCP_CUDA(cudaMemsetAsync(base + off_flags, 0, 256, s));
  if (fp32) UMCP_CUDA(launch_split_positions(3 * m->nv, d_r, f32, s));
  FinishArgs fin{m->nblocks, d_E, nullptr, d_g ? d_g + 3 * m->nv : nullptr, nullptr, nullptr, 0.0, status, done};
  for (size_t gi = 0; gi < m->groups.size(); ++gi) {
    auto &G = m->groups[gi];
    dev::FaceLaunch L;
    L.nfaces = G->nfaces;
    L.block_base = G->block_base;
    L.cp = G->cp.as<uint32_t>();
    L.g0 = G->g0.as<double>();
    L.rr0 = G->rr0.as<double>();
    L.comp = G->comp.as<double>();
    L.g0f = G->g0f.as<float>();
    L.rr0f = G->rr0f.as<float>();
    L.compf = G->compf.as<float>();
    L.basis = G->basis.as<double>();
    L.weight = G->weight.as<double>();
    L.dudv = G->dudv;
    L.irregular = G->irregular;
    const FinishArgs &f = fin;  // every block of every launch counts toward the finish
    cudaError_t e = (fp32 && G->tc) ? launch_faces_tc(L, G->dest.as<int>(), m->P, d_r, rhi, rlo, f32.dsp,
                                                       (float *)(base + off_partial), blockpart, status, G->nblocks, f, s)
                    : fp32 ? launch_faces<float>(L, G->dest.as<int>(), G->ncp, G->npt, m->P, d_r, f32,
                                               (float *)(base + off_partial), blockpart, status, G->nblocks, f, s)
                         : launch_faces<double>(L, G->dest.as<int>(), G->ncp, G->npt, m->P, d_r, f32,
                                                (double *)(base + off_partial), blockpart, status, G->nblocks, f, s);
    if (e != cudaSuccess) return fail(UMCP_ERR_CUDA, std::string("face pass: ") + cudaGetErrorString(e));
  }
  if (d_g) {
    cudaError_t e = fp32 ? launch_gather<float>(m->nv, (float *)(base + off_partial), m->off.as<int>(), d_g, s)
                         : launch_gather<double>(m->nv, (double *)(base + off_partial), m->off.as<int>(), d_g, s);
    if (e != cudaSuccess) return fail(UMCP_ERR_CUDA, std::string("gather: ") + cudaGetErrorString(e));
  }
  // The next call clears the array's status word: hand its bits (non-finite
  // energy, a tensor-core wait that gave up) to the mesh's own status word,
  // where umcp_mesh_check_status reads them.
  UMCP_CUDA(launch_status_merge(status, m->status.as<int>(), s));
  return UMCP_OK;
}

extern "C" umcp_status umcp_mesh_check_status(umcp_mesh *m) {
  if (!m) return fail(UMCP_ERR_INVALID, "null mesh");
  UMCP_CUDA(cudaSetDevice(m->ctx->device));
  const umcp_status st = check_status(m);  // synchronizes the mesh's stream
  UMCP_CUDA(cudaMemsetAsync(m->status.p, 0, sizeof(int), m->ctx->stream));
  UMCP_CUDA(cudaStreamSynchronize(m->ctx->stream));
  return st;
}
