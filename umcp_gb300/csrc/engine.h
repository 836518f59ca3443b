// Internal definitions shared by the engine's translation units (not part
// of the ABI): device buffers, the context and device mesh objects, and the
// error helper every entry point reports through.
#pragma once
#include <atomic>
#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "../../include/umcp_gpu.h"
#include "launch.h"

namespace umcp {

// Records the text umcp_last_error() returns on this host thread; returns s.
umcp_status set_error(umcp_status s, const std::string &msg);

constexpr int kGraphChunk = 32;  // steps captured per CUDA graph

// A device buffer: owned (cudaMalloc'd here and freed with it) or a view into
// memory another DevBuf owns (a mesh's creation-time arena). alloc() always
// leaves it owning a fresh allocation.
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  bool owned = true;
  ~DevBuf() { if (p && owned) cudaFree(p); }
  cudaError_t alloc(size_t b) {
    if (p && owned) cudaFree(p);
    p = nullptr;
    owned = true;
    bytes = b;
    return b ? cudaMalloc(&p, b) : cudaSuccess;
  }
  void view(void *at, size_t b) {
    if (p && owned) cudaFree(p);
    p = b ? at : nullptr;
    bytes = b;
    owned = false;
  }
  template <class T> T *as() const { return (T *)p; }
};

struct Group {
  int ncp = 0, npt = 0, nfaces = 0, slot_base = 0, irregular = 0;
  int valence = 6;                  // of the patch type's lowest corner
  std::vector<int> face_index;      // each face's index in the plan (regular faces, then irregular)
  bool tc = false;                  // regular faces of the precision form on the tensor cores
  int nblocks = 0, block_base = 0;  // persistent face-pass grid and its block-partial rows
  double dudv = 0.5;
  DevBuf cp, g0, rr0, comp, basis, weight, dest;
  DevBuf basis_w;           // value rows [npt][ncp] (area and volume terms)
  DevBuf g0f, rr0f, compf;  // FP32 copies for the precision form
  DevBuf geo_tab;           // FP32 restraint tables (GeoGroup::tab), built when restraints are first set
};
}  // namespace umcp

struct umcp_batch;

// Reference-counted: meshes and batches hold the context, so it outlives
// them whatever order they are destroyed in.
struct umcp_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  // A mesh's irregular face launches run on `side`, forked from `stream`
  // before the regular launch and joined after it (calls on a ctx are
  // serialised, so one pair serves every mesh of the ctx).
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  std::atomic<int> refs{1};  // the creator's reference plus one per live mesh or batch (meshes may be made on several threads)
};

namespace umcp {
inline umcp_ctx *ctx_retain(umcp_ctx *c) {
  ++c->refs;
  return c;
}
inline void ctx_release(umcp_ctx *c) {
  if (--c->refs > 0) return;
  cudaSetDevice(c->device);
  if (c->fork) cudaEventDestroy(c->fork);
  if (c->join) cudaEventDestroy(c->join);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}
}  // namespace umcp

struct umcp_mesh {
  umcp_ctx *ctx = nullptr;
  int nv = 0, nfaces = 0, nslots = 0;
  int nslot_cap = 0;  // partial slots allocated: nslots plus the padding of the interleaved numbering
  int precision = UMCP_FP64;
  umcp::dev::SurfaceParams P{};
  std::vector<std::unique_ptr<umcp::Group>> groups;
  umcp::DevBuf partial, off, blockpart;
  int nblocks = 0;
  umcp::DevBuf r, g, p, qdot, E, parts, status, cnt;  // cnt: {first step of the run, run index}
  umcp::DevBuf rhi, rlo;  // FP32 hi/lo pairs of r (precision form)
  umcp::DevBuf r0, dsp;   // precision form: reference state (FP64) and r - r0 (FP32)
  umcp::DevBuf r_eval;    // staging for host-pointer energy/gradient calls (keeps the resident state)
  umcp::DevBuf done;      // finished-block counter of the face pass
  bool split_valid = false;  // rhi/rlo hold the resident state r
  double kT = 0.592186663194;  // kcal/mol at the params' temperature (src/hd.C:142-143)
  umcp::DevBuf energies;
  size_t energies_cap = 0;
  umcp_batch *batch = nullptr;  // the batch this mesh is a job of, if any
  // global area/volume restraints (umcp_restraints_set)
  struct Restraints {
    bool on = false;
    double KA = 0, A0 = 0, KV = 0, V0 = 0;
  } rs;
  umcp::DevBuf geo_block, gterm, geo_done;
  umcp::DevBuf arena;         // one allocation holding the buffers made at creation (views into it)
  void *h_pinned = nullptr;   // one pinned block holding the three below
  double *h_stage = nullptr;  // pinned, 3*nv+3 doubles
  double *h_stage2 = nullptr; // pinned, 3*nv doubles
  uint64_t *h_cnt = nullptr;  // pinned, 2 counters
  // effective inverse mass: CSR (mrow, mcol, mval) or dense row-major (mdense);
  // FP64 values, or FP32 ones for meshes of the precision form (mass_f32),
  // whose apply reads an FP32 copy of its input (min32, nv float4 {x, y, z, 0})
  int mrows = 0;
  umcp::DevBuf mrow, mcol, mval, alphas, mdense, min32;
  bool mass_dense = false, mass_f32 = false;
  // the FP32 CSR's column indices as uint16 (meshes of at most 65,536 vertices:
  // 6 bytes per nonzero instead of 8 for an apply that HBM bounds)
  bool mcol16 = false;
  // captured step sequences, by length (powers of two up to kGraphChunk steps)
  struct CachedGraph {
    cudaGraphExec_t exec = nullptr;
    int steps = 0;
    umcp::StepArgs args{};
    int use_mass = -1;
    double threshold = 0;
  };
  std::vector<CachedGraph> graphs;
  void drop_graphs() {
    for (auto &g : graphs)
      if (g.exec) cudaGraphExecDestroy(g.exec);
    graphs.clear();
  }

  // Device bytes held by the mesh's buffers.
  size_t device_bytes() const {
    size_t b = 0;
    for (auto &G : groups)
      for (const umcp::DevBuf *x : {&G->cp, &G->g0, &G->rr0, &G->comp, &G->basis, &G->weight, &G->dest, &G->g0f,
                                    &G->rr0f, &G->compf, &G->basis_w, &G->geo_tab})
        b += x->bytes;
    for (const umcp::DevBuf *x : {&partial, &off, &blockpart, &r, &g, &p, &qdot, &E, &parts, &status, &cnt, &rhi,
                                  &rlo, &r0, &dsp, &r_eval, &done, &energies, &mrow, &mcol, &mval, &alphas, &mdense, &min32, &geo_block, &gterm,
                                  &geo_done})
      b += x->bytes;
    return b;
  }

  // The FP32 position copies the kernels read and write (all NULL in the plain path).
  umcp::F32Pos f32pos() const {
    umcp::F32Pos f;
    if (precision == UMCP_FP32_CENTRED) {
      f.hi = rhi.as<float>(); f.lo = rlo.as<float>(); f.r0 = r0.as<double>(); f.dsp = dsp.as<float>();
    }
    return f;
  }

  ~umcp_mesh() {
    drop_graphs();
    if (h_pinned) cudaFreeHost(h_pinned);
  }
};

namespace umcp {

struct Plan;
// Host-side plan of a umcp_plan.
const Plan &plan_of(const umcp_plan *p);

// out (+)= M^-1 in with the installed inverse mass, dense or CSR (see launch_spmv
// for the scaling arguments).
cudaError_t queue_mass_apply(umcp_mesh *m, const double *scalev, double scale, const double *alphas,
                             const double *in, double *out, int accumulate, cudaStream_t s);

// Integrator settings of a run on mesh m (validates it).
umcp_status make_step_args(const umcp_mesh *m, const umcp_integrator *it, StepArgs *a);
// A batch drops a job whose mesh is being destroyed (waits for its stream
// first); a batch rebuilds its tables after a job's mesh changed.
void batch_forget_mesh(umcp_batch *b, umcp_mesh *m);
void batch_mesh_changed(umcp_batch *b);

// Block-partial rows of a group's face launch, and the rows its footprint
// reserves (the larger of the two kernels' grids, so the footprint does not
// depend on the kernel choice).
int group_blocks(int precision, bool tc, int ncp, int npt, int nfaces);
size_t interleave_slots(const std::vector<int> &counts, std::vector<int> *loc);
int group_block_rows(int precision, int ncp, int npt, int nfaces);

inline uint32_t pack_cp(int v, const int8_t img[3]) {
  int code = (img[0] + 1) + 3 * (img[1] + 1) + 9 * (img[2] + 1);
  return (uint32_t)v | ((uint32_t)code << dev::kVertexBits);
}

template <class T>
inline cudaError_t upload(DevBuf &b, const std::vector<T> &h) {
  cudaError_t e = b.alloc(h.size() * sizeof(T));
  if (e != cudaSuccess || h.empty()) return e;
  return cudaMemcpy(b.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
}

}  // namespace umcp

#define UMCP_CUDA(call)                                                                          \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess)                                                                       \
      return umcp::set_error(UMCP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
