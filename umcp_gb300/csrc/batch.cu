// Batches: many device-resident meshes advanced together, one face launch per
// patch type per step over all of them. The reference runs one surface per
// process; each job here follows umcp_run's semantics for its own mesh, and
// its trajectory does not depend on the rest of the batch (the per-face and
// per-vertex arithmetic is the single-mesh path's).
//
// Tables (device): the job array, the face tiles of every patch type and the
// vertex tiles, each job's tile list, and a count array that every kernel
// reads at run time. Membership changes rewrite the tables between runs; the
// captured steps stay valid until a table outgrows its capacity.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <string>
#include <vector>

#include "engine.h"

using namespace umcp;

namespace {

constexpr int kTypes = 3;                      // regular, irregular valence 5, irregular valence 7
constexpr int kTypeNcp[kTypes] = {12, 11, 13};

int type_of(const Group &G) { return G.ncp == 12 ? 0 : (G.ncp == 11 ? 1 : (G.ncp == 13 ? 2 : -1)); }

struct Job {
  umcp_mesh *m = nullptr;
  StepArgs a{};
  double threshold = 0;
  uint64_t step0 = 0;
  int64_t n_steps = 0;
  bool start = true;  // counters, status and hi/lo pairs are reset at the next run
  int64_t done = 0;   // steps done and status bits, as of the latest harvest
  int status = 0;
};

}  // namespace

struct umcp_batch {
  umcp_ctx *ctx = nullptr;
  int precision = UMCP_FP64;
  int opt_tile_faces = 0, opt_blocks_per_sm = 0, opt_irr_tile = 0;
  std::string tune_cache;  // JSON file of tuned choices ("" = none)
  int tile_faces = 0;      // chosen at the first run when opt_tile_faces is 0
  int irr_tile = 0;        // faces per irregular tile (0: 4 per half-warp)
  int max_grid[3] = {0, 0, 0};  // the occupancy-limited persistent grids
  int tune_source = 0;     // 0 options, 1 timed, 2 tune cache
  double tuned_ms = 0;
  long long tuned_faces = 0;  // faces in the batch when the tile size was last timed
  std::vector<Job> jobs;
  bool dirty = true;
  // Each patch type's basis (the same for every mesh: it depends on the
  // valence only), copied from the first job that has the type.
  bool have_type[kTypes] = {false, false, false};
  int npt[kTypes] = {0, 0, 0};
  double dudv[kTypes] = {0, 0, 0};
  DevBuf basis[kTypes], weight[kTypes];
  int face_grid[kTypes] = {0, 0, 0};
  int vgrid = 0;
  // device tables
  DevBuf d_jobs, d_tiles, d_vtiles, d_tile_off, d_tile_idx, d_counts, d_live, d_prog, d_start, d_step0, d_tile_sums;
  DevBuf d_next_tile;  // {tiles handed out, blocks done} of the regular face launch (it resets them)
  // host-driven steps (umcp_batch_step_host): the jobs' states packed in job
  // order, each job's offset into the pack, and the jobs' latest energies
  DevBuf d_pack, d_pack_off, d_pack_E;
  size_t pack_doubles = 0;
  size_t cap_jobs = 0, cap_tiles = 0, cap_vtiles = 0;
  // host copies of the counts and the latest progress (pinned)
  int counts[kCountWords] = {};
  unsigned long long *h_prog = nullptr;
  size_t prog_jobs = 0;  // jobs whose progress the latest run is copying to h_prog
  // captured steps for the current capacities: g_pow[i] runs 2^i steps (up to kGraphChunk)
  static constexpr int kPows = 6;
  static_assert(1 << (kPows - 1) == kGraphChunk, "one captured length per power of two up to kGraphChunk");
  cudaGraphExec_t g_pow[kPows] = {};
  // The irregular face launches run on a second stream, forked from the
  // context's stream after the regular launch is queued and joined before the
  // per-job sums, so they fill the SMs the regular launch's tail leaves idle
  // (in a captured step, two branches of the graph).
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  void drop_graphs() {
    for (cudaGraphExec_t &g : g_pow) {
      if (g) cudaGraphExecDestroy(g);
      g = nullptr;
    }
  }
  ~umcp_batch() {
    drop_graphs();
    if (h_prog) cudaFreeHost(h_prog);
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    if (side) cudaStreamDestroy(side);
  }
};

static umcp_status harvest(umcp_batch *b);

namespace umcp {
void batch_forget_mesh(umcp_batch *b, umcp_mesh *m);
void batch_mesh_changed(umcp_batch *b);
}  // namespace umcp

void umcp::batch_mesh_changed(umcp_batch *b) { b->dirty = true; }

void umcp::batch_forget_mesh(umcp_batch *b, umcp_mesh *m) {
  harvest(b);
  auto it = std::find_if(b->jobs.begin(), b->jobs.end(), [&](const Job &j) { return j.m == m; });
  if (it != b->jobs.end()) b->jobs.erase(it);
  b->dirty = true;
  m->batch = nullptr;
}

static umcp_status fail(umcp_status s, const std::string &msg) { return umcp::set_error(s, msg); }

// Copies the progress of the latest run (in the job order of that run) into
// the jobs, once the run has finished.
static umcp_status harvest(umcp_batch *b) {
  if (!b->prog_jobs) return UMCP_OK;
  UMCP_CUDA(cudaStreamSynchronize(b->ctx->stream));
  for (size_t j = 0; j < b->prog_jobs && j < b->jobs.size(); ++j) {
    b->jobs[j].done = (int64_t)b->h_prog[2 * j];
    b->jobs[j].status = (int)b->h_prog[2 * j + 1];
  }
  b->prog_jobs = 0;
  return UMCP_OK;
}

static BatchJob job_entry(const Job &J) {
  umcp_mesh *m = J.m;
  BatchJob e;
  memset(&e, 0, sizeof(e));
  for (int t = 0; t < kTypes; ++t) e.f.src[t].nfaces = 0;
  for (auto &Gp : m->groups) {
    const Group &G = *Gp;
    const int t = type_of(G);
    dev::FaceSrc &s = e.f.src[t];
    s.cp = G.cp.as<uint32_t>();
    s.g0 = G.g0.as<double>(); s.rr0 = G.rr0.as<double>(); s.comp = G.comp.as<double>();
    s.g0f = G.g0f.as<float>(); s.rr0f = G.rr0f.as<float>(); s.compf = G.compf.as<float>();
    s.dest = G.dest.as<int>();
    s.r = m->r.as<double>();
    s.rhi = m->rhi.as<float>(); s.rlo = m->rlo.as<float>(); s.dsp = m->dsp.as<float>();
    s.nfaces = G.nfaces;
  }
  e.f.P = m->P;
  e.f.partial = m->partial.p;
  e.f.cnt = m->cnt.as<uint64_t>();
  e.f.limit = (uint64_t)J.n_steps;
  e.f.status = m->status.as<int>();
  e.off = m->off.as<int>();
  e.r = m->r.as<double>();
  e.p = m->p.as<double>();
  const bool f32 = m->precision == UMCP_FP32_CENTRED;
  e.rhi = f32 ? m->rhi.as<float>() : nullptr;
  e.rlo = f32 ? m->rlo.as<float>() : nullptr;
  e.r0 = f32 ? m->r0.as<double>() : nullptr;
  e.dsp = f32 ? m->dsp.as<float>() : nullptr;
  e.E = m->E.as<double>();
  e.parts = m->parts.as<double>();
  e.energies = m->energies.as<double>();
  e.threshold = J.threshold;
  e.a = J.a;
  return e;
}

// Rebuild and upload the tables for the current jobs and tile size.
static umcp_status rebuild(umcp_batch *b) {
  cudaStream_t s = b->ctx->stream;
  const int tf = b->tile_faces > 0 ? b->tile_faces : 64;
  std::vector<BatchJob> jt;
  std::vector<BatchTile> tiles, vtiles;
  std::vector<std::vector<int>> per_job(b->jobs.size());
  for (const Job &J : b->jobs) jt.push_back(job_entry(J));
  // Irregular faces (a few dozen per closed vesicle) go in tiles of at most
  // four faces per half-warp of their kernel, so that they spread over the
  // grid instead of queueing on one block per job.
  const int hw = b->precision == UMCP_FP64 ? dev::FaceCfg<double>::half_warps : dev::FaceCfg<float>::half_warps;
  for (int t = 0; t < kTypes; ++t) {
    b->counts[kCountTileBase + t] = (int)tiles.size();
    const int tft = t == 0 ? tf : (b->irr_tile > 0 ? b->irr_tile : std::min(tf, 4 * hw));
    for (size_t j = 0; j < b->jobs.size(); ++j) {
      const int nf = jt[j].f.src[t].nfaces;
      for (int first = 0; first < nf; first += tft) {
        per_job[j].push_back((int)tiles.size());
        tiles.push_back(BatchTile{(int)j, first, std::min(tft, nf - first)});
      }
    }
    b->counts[kCountTiles + t] = (int)tiles.size() - b->counts[kCountTileBase + t];
  }
  std::vector<int> tile_off(1, 0), tile_idx;
  for (auto &v : per_job) {
    tile_idx.insert(tile_idx.end(), v.begin(), v.end());
    tile_off.push_back((int)tile_idx.size());
  }
  for (size_t j = 0; j < b->jobs.size(); ++j)
    for (int first = 0; first < b->jobs[j].m->nv; first += kVertexTile)
      vtiles.push_back(BatchTile{(int)j, first, std::min(kVertexTile, b->jobs[j].m->nv - first)});
  b->counts[kCountJobs] = (int)b->jobs.size();
  b->counts[kCountVertexTiles] = (int)vtiles.size();
  std::vector<long long> pack_off(1, 0);
  for (const Job &J : b->jobs) pack_off.push_back(pack_off.back() + 3 * (long long)J.m->nv + 3);
  b->pack_doubles = (size_t)pack_off.back();

  const size_t nj = jt.size(), nt = tiles.size(), nvt = vtiles.size();
  if (nj > b->cap_jobs || nt > b->cap_tiles || nvt > b->cap_vtiles || !b->d_counts.p) {
    auto cap = [](size_t need, size_t c) { return need <= c ? c : std::max<size_t>({need, 2 * c, 16}); };
    b->cap_jobs = cap(nj, b->cap_jobs);
    b->cap_tiles = cap(nt, b->cap_tiles);
    b->cap_vtiles = cap(nvt, b->cap_vtiles);
    UMCP_CUDA(cudaStreamSynchronize(s));  // queued steps may still read the old tables
    b->drop_graphs();
    UMCP_CUDA(b->d_jobs.alloc(b->cap_jobs * sizeof(BatchJob)));
    UMCP_CUDA(b->d_tile_off.alloc((b->cap_jobs + 1) * sizeof(int)));
    UMCP_CUDA(b->d_live.alloc(b->cap_jobs * sizeof(int)));
    UMCP_CUDA(b->d_prog.alloc(2 * b->cap_jobs * sizeof(unsigned long long)));
    UMCP_CUDA(b->d_start.alloc(b->cap_jobs * sizeof(int)));
    UMCP_CUDA(b->d_step0.alloc(b->cap_jobs * sizeof(unsigned long long)));
    UMCP_CUDA(b->d_tiles.alloc(b->cap_tiles * sizeof(BatchTile)));
    UMCP_CUDA(b->d_tile_idx.alloc(b->cap_tiles * sizeof(int)));
    UMCP_CUDA(b->d_tile_sums.alloc(3 * b->cap_tiles * sizeof(double)));
    UMCP_CUDA(b->d_vtiles.alloc(b->cap_vtiles * sizeof(BatchTile)));
    UMCP_CUDA(b->d_counts.alloc(kCountWords * sizeof(int)));
    UMCP_CUDA(cudaMemsetAsync(b->d_live.p, 0, b->cap_jobs * sizeof(int), s));
    if (b->h_prog) cudaFreeHost(b->h_prog);
    b->h_prog = nullptr;
    UMCP_CUDA(cudaMallocHost((void **)&b->h_prog, 2 * b->cap_jobs * sizeof(unsigned long long)));
    UMCP_CUDA(b->d_pack_off.alloc((b->cap_jobs + 1) * sizeof(long long)));
    UMCP_CUDA(b->d_pack_E.alloc(b->cap_jobs * sizeof(double)));
  }
  if (b->pack_doubles * sizeof(double) > b->d_pack.bytes) {
    UMCP_CUDA(cudaStreamSynchronize(s));
    UMCP_CUDA(b->d_pack.alloc(std::max(b->pack_doubles * sizeof(double), 2 * b->d_pack.bytes)));
  }
  // Pageable sources: each copy has read its source when the call returns,
  // and the stream orders it after the steps already queued.
  if (!jt.empty()) {
    UMCP_CUDA(cudaMemcpyAsync(b->d_jobs.p, jt.data(), jt.size() * sizeof(BatchJob), cudaMemcpyHostToDevice, s));
    UMCP_CUDA(cudaMemcpyAsync(b->d_tile_off.p, tile_off.data(), tile_off.size() * sizeof(int),
                              cudaMemcpyHostToDevice, s));
  }
  if (!tiles.empty()) {
    UMCP_CUDA(cudaMemcpyAsync(b->d_tiles.p, tiles.data(), tiles.size() * sizeof(BatchTile), cudaMemcpyHostToDevice, s));
    UMCP_CUDA(cudaMemcpyAsync(b->d_tile_idx.p, tile_idx.data(), tile_idx.size() * sizeof(int),
                              cudaMemcpyHostToDevice, s));
  }
  if (!vtiles.empty())
    UMCP_CUDA(cudaMemcpyAsync(b->d_vtiles.p, vtiles.data(), vtiles.size() * sizeof(BatchTile),
                              cudaMemcpyHostToDevice, s));
  UMCP_CUDA(cudaMemcpyAsync(b->d_pack_off.p, pack_off.data(), pack_off.size() * sizeof(long long),
                            cudaMemcpyHostToDevice, s));
  UMCP_CUDA(cudaMemcpyAsync(b->d_counts.p, b->counts, sizeof(b->counts), cudaMemcpyHostToDevice, s));
  UMCP_CUDA(cudaStreamSynchronize(s));  // b->counts is rewritten by the next rebuild
  b->dirty = false;
  return UMCP_OK;
}

// Run start of the jobs added since the last run.
static umcp_status start_jobs(umcp_batch *b) {
  std::vector<int> start(b->jobs.size(), 0);
  std::vector<unsigned long long> step0(b->jobs.size(), 0);
  bool any = false;
  for (size_t j = 0; j < b->jobs.size(); ++j)
    if (b->jobs[j].start) {
      start[j] = 1;
      step0[j] = b->jobs[j].step0;
      any = true;
    }
  if (!any) return UMCP_OK;
  cudaStream_t s = b->ctx->stream;
  UMCP_CUDA(cudaMemcpyAsync(b->d_start.p, start.data(), start.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  UMCP_CUDA(cudaMemcpyAsync(b->d_step0.p, step0.data(), step0.size() * sizeof(unsigned long long),
                            cudaMemcpyHostToDevice, s));
  UMCP_CUDA(launch_batch_start(b->d_jobs.as<BatchJob>(), b->d_vtiles.as<BatchTile>(), b->d_counts.as<int>(),
                               b->d_start.as<int>(), b->d_step0.as<unsigned long long>(), b->vgrid, s));
  UMCP_CUDA(cudaStreamSynchronize(s));  // the pageable sources above go out of scope
  for (Job &J : b->jobs) {
    if (J.start) J.done = 0, J.status = 0;
    J.start = false;
    if (J.m->precision == UMCP_FP32_CENTRED) J.m->split_valid = true;
  }
  return UMCP_OK;
}

// The precision form's FP32 copies of every job's resident state: a mesh whose
// copies were last taken from another state (an energy call at other
// positions) gets them again before the batch reads them.
static umcp_status resplit(umcp_batch *b) {
  for (Job &J : b->jobs) {
    umcp_mesh *m = J.m;
    if (m->precision != UMCP_FP32_CENTRED || m->split_valid) continue;
    UMCP_CUDA(launch_split_positions(3 * m->nv, m->r.as<double>(), m->f32pos(), b->ctx->stream));
    m->split_valid = true;
  }
  return UMCP_OK;
}

template <typename T>
static cudaError_t queue_faces_t(umcp_batch *b) {
  cudaStream_t s = b->ctx->stream;
  auto launch = [&](int t, cudaStream_t on) {
    return launch_batch_faces<T>(b->d_jobs.as<BatchJob>(), t, b->d_tiles.as<BatchTile>(), b->d_counts.as<int>(),
                                 b->basis[t].as<double>(), b->weight[t].as<double>(), kTypeNcp[t], b->npt[t],
                                 b->dudv[t], t > 0, b->d_tile_sums.as<double>(), b->face_grid[t],
                                 b->d_next_tile.as<int>(), on);
  };
  cudaError_t e = cudaSuccess;
  const bool irregular = b->have_type[1] || b->have_type[2];
  if (irregular) {
    // the side stream starts after everything queued on s so far, then runs
    // beside the regular launch (they write disjoint slots and tile rows)
    if ((e = cudaEventRecord(b->fork, s)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(b->side, b->fork, 0)) != cudaSuccess) return e;
  }
  if (b->have_type[0] && (e = launch(0, s)) != cudaSuccess) return e;
  if (!irregular) return cudaSuccess;
  for (int t = 1; t < kTypes; ++t)
    if (b->have_type[t] && (e = launch(t, b->side)) != cudaSuccess) return e;
  if ((e = cudaEventRecord(b->join, b->side)) != cudaSuccess) return e;
  return cudaStreamWaitEvent(s, b->join, 0);
}

static cudaError_t queue_faces(umcp_batch *b) {
  return b->precision == UMCP_FP64 ? queue_faces_t<double>(b) : queue_faces_t<float>(b);
}

static cudaError_t queue_step(umcp_batch *b) {
  cudaStream_t s = b->ctx->stream;
  cudaError_t e = queue_faces(b);
  if (e == cudaSuccess)
    e = launch_batch_reduce(b->d_jobs.as<BatchJob>(), b->d_counts.as<int>(), (int)b->cap_jobs,
                            b->d_tile_off.as<int>(), b->d_tile_idx.as<int>(), b->d_tile_sums.as<double>(),
                            b->d_live.as<int>(), b->d_prog.as<unsigned long long>(), s);
  if (e == cudaSuccess)
    e = b->precision == UMCP_FP64
            ? launch_batch_gather_step<double>(b->d_jobs.as<BatchJob>(), b->d_vtiles.as<BatchTile>(),
                                               b->d_counts.as<int>(), b->d_live.as<int>(), b->vgrid, s)
            : launch_batch_gather_step<float>(b->d_jobs.as<BatchJob>(), b->d_vtiles.as<BatchTile>(),
                                              b->d_counts.as<int>(), b->d_live.as<int>(), b->vgrid, s);
  return e;
}

static umcp_status capture(umcp_batch *b, int steps, cudaGraphExec_t *out) {
  cudaStream_t s = b->ctx->stream;
  cudaGraph_t g;
  UMCP_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < steps && e == cudaSuccess; ++i) e = queue_step(b);
  cudaError_t e2 = cudaStreamEndCapture(s, &g);
  if (e != cudaSuccess) return fail(UMCP_ERR_CUDA, std::string("batch step capture: ") + cudaGetErrorString(e));
  if (e2 != cudaSuccess) return fail(UMCP_ERR_CUDA, std::string("batch end capture: ") + cudaGetErrorString(e2));
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(UMCP_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(e));
  return UMCP_OK;
}

// ---- the face launches' layout, tuned by timing and cached

namespace {

struct Layout {
  int tile_faces = 0, irr_tile = 0, blocks_per_sm = 0;
  double face_ms = 0;
};

// Key of a batch's kind: device, precision, patch types present, log2 of faces.
std::string layout_key(const umcp_batch *b, long long faces) {
  cudaDeviceProp prop;
  std::string dev = cudaGetDeviceProperties(&prop, b->ctx->device) == cudaSuccess ? prop.name : "device";
  std::string types;
  for (int t = 0; t < kTypes; ++t)
    if (b->have_type[t]) types += (types.empty() ? "" : "+") + std::to_string(t == 0 ? 6 : t == 1 ? 5 : 7);
  const int bucket = faces > 0 ? (int)std::floor(std::log2((double)faces)) : 0;
  return dev + "|" + (b->precision == UMCP_FP64 ? "fp64" : "fp32") + "|" + types + "|" + std::to_string(bucket);
}

// The cache file holds one JSON object, {"<key>": {"tile_faces": n,
// "irr_tile_faces": n, "blocks_per_sm": n, "face_ms": x}, ...}, written by
// this code only (the reader takes that layout, not general JSON).
std::map<std::string, Layout> read_layouts(const std::string &path) {
  std::map<std::string, Layout> out;
  FILE *f = fopen(path.c_str(), "r");
  if (!f) return out;
  std::string text;
  char buf[4096];
  size_t n;
  while ((n = fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, n);
  fclose(f);
  size_t p = 0;
  while ((p = text.find('"', p)) != std::string::npos) {
    const size_t e = text.find('"', p + 1);
    if (e == std::string::npos) break;
    const std::string key = text.substr(p + 1, e - p - 1);
    const size_t open = text.find('{', e), close = text.find('}', e);
    if (open == std::string::npos || close == std::string::npos || open > close) break;
    const std::string body = text.substr(open, close - open);
    Layout L;
    auto num = [&](const char *name) {
      const size_t q = body.find(std::string("\"") + name + "\"");
      return q == std::string::npos ? 0.0 : atof(body.c_str() + body.find(':', q) + 1);
    };
    L.tile_faces = (int)num("tile_faces");
    L.irr_tile = (int)num("irr_tile_faces");
    L.blocks_per_sm = (int)num("blocks_per_sm");
    L.face_ms = num("face_ms");
    if (L.tile_faces > 0) out[key] = L;
    p = close + 1;
  }
  return out;
}

void write_layouts(const std::string &path, const std::map<std::string, Layout> &all) {
  const std::string tmp = path + ".tmp";
  FILE *f = fopen(tmp.c_str(), "w");
  if (!f) return;
  fprintf(f, "{\n");
  size_t k = 0;
  for (const auto &e : all)
    fprintf(f, "  \"%s\": {\"tile_faces\": %d, \"irr_tile_faces\": %d, \"blocks_per_sm\": %d, \"face_ms\": %.6f}%s\n",
            e.first.c_str(), e.second.tile_faces, e.second.irr_tile, e.second.blocks_per_sm, e.second.face_ms,
            ++k < all.size() ? "," : "");
  fprintf(f, "}\n");
  fclose(f);
  rename(tmp.c_str(), path.c_str());  // replaces the file whole
}

}  // namespace

// Puts a layout in place: tiles and grids (the captured steps are re-made).
static umcp_status apply_layout(umcp_batch *b, const Layout &L) {
  int sms = 0;
  UMCP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->ctx->device));
  b->tile_faces = L.tile_faces;
  b->irr_tile = L.irr_tile;
  for (int t = 0; t < kTypes; ++t) {
    const int cap = t == 0 && L.blocks_per_sm > 0 ? L.blocks_per_sm * sms : b->max_grid[t];
    b->face_grid[t] = std::max(1, std::min(b->max_grid[t], cap));
  }
  b->drop_graphs();
  return rebuild(b);
}

static float time_face_launches(umcp_batch *b, cudaEvent_t e0, cudaEvent_t e1, umcp_status *st) {
  cudaStream_t s = b->ctx->stream;
  float ms = 0;
  if (queue_faces(b) != cudaSuccess || cudaEventRecord(e0, s) != cudaSuccess) { *st = UMCP_ERR_CUDA; return 0; }
  for (int k = 0; k < 3; ++k)
    if (queue_faces(b) != cudaSuccess) { *st = UMCP_ERR_CUDA; return 0; }
  if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
      cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) { *st = UMCP_ERR_CUDA; return 0; }
  return ms / 3;
}

// Chooses the face launches' layout for the batch's current jobs (after
// their run start): from the tune cache, else by timing the face launches,
// which change nothing but the gradient-partial slots and tile sums that
// every step rewrites. First the regular tile size (multiples of the face
// kernel's faces per block pass: 8 per FP64 block, 128 per thread-per-face
// block, up to 2048), then the irregular tile size (1 to 8 faces per
// half-warp), then the regular launch's blocks per SM (the occupancy limit or
// one fewer), each with the others held.
static umcp_status autotune(umcp_batch *b, long long faces) {
  const std::string key = layout_key(b, faces);
  std::map<std::string, Layout> cached;
  if (!b->tune_cache.empty()) {
    cached = read_layouts(b->tune_cache);
    auto it = cached.find(key);
    if (it != cached.end()) {
      b->tune_source = 2;
      b->tuned_ms = it->second.face_ms;
      return apply_layout(b, it->second);
    }
  }
  const bool f64 = b->precision == UMCP_FP64;
  const int hw = f64 ? dev::FaceCfg<double>::half_warps : dev::FaceCfg<float>::half_warps;
  int sms = 0;
  UMCP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->ctx->device));
  const int max_bps = std::max(1, b->max_grid[0] / std::max(sms, 1));
  cudaEvent_t e0, e1;
  UMCP_CUDA(cudaEventCreate(&e0));
  UMCP_CUDA(cudaEventCreate(&e1));
  umcp_status st = UMCP_OK;
  Layout best;
  auto trial = [&](Layout L) {
    if (st != UMCP_OK) return;
    if ((st = apply_layout(b, L)) != UMCP_OK) return;
    L.face_ms = time_face_launches(b, e0, e1, &st);
    if (st == UMCP_OK && (best.tile_faces == 0 || L.face_ms < best.face_ms)) best = L;
  };
  const int unit = f64 ? dev::FaceCfg<double>::half_warps : 32;
  for (int mult : {1, 2, 4, 8, 16, 32, 64}) {
    if ((f64 && mult > 32) || (!f64 && mult < 4)) continue;
    trial(Layout{unit * mult, 4 * hw, max_bps, 0});
  }
  if (b->have_type[1] || b->have_type[2])
    for (int per : {1, 2, 8}) trial(Layout{best.tile_faces, per * hw, best.blocks_per_sm, 0});
  if (max_bps > 1) trial(Layout{best.tile_faces, best.irr_tile, max_bps - 1, 0});
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != UMCP_OK) return st;
  b->tune_source = 1;
  b->tuned_ms = best.face_ms;
  if (!b->tune_cache.empty()) {
    cached = read_layouts(b->tune_cache);  // as of now: another batch may have written meanwhile
    cached[key] = best;
    write_layouts(b->tune_cache, cached);
  }
  return apply_layout(b, best);
}

extern "C" umcp_status umcp_batch_create(umcp_ctx *ctx, int precision, const umcp_batch_opts *opts,
                                         umcp_batch **out) {
  if (!ctx || !out) return fail(UMCP_ERR_INVALID, "null argument");
  if (precision != UMCP_FP64 && precision != UMCP_FP32_CENTRED) return fail(UMCP_ERR_INVALID, "unknown precision");
  UMCP_CUDA(cudaSetDevice(ctx->device));
  auto b = std::make_unique<umcp_batch>();
  UMCP_CUDA(cudaSetDevice(ctx->device));
  UMCP_CUDA(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking));
  UMCP_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
  UMCP_CUDA(cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming));
  UMCP_CUDA(b->d_next_tile.alloc(2 * sizeof(int)));
  UMCP_CUDA(cudaMemsetAsync(b->d_next_tile.p, 0, 2 * sizeof(int), ctx->stream));
  b->ctx = ctx;
  b->precision = precision;
  if (opts) {
    if (opts->tile_faces < 0 || opts->blocks_per_sm < 0 || opts->irr_tile_faces < 0)
      return fail(UMCP_ERR_INVALID, "negative batch option");
    b->opt_tile_faces = opts->tile_faces;
    b->opt_blocks_per_sm = opts->blocks_per_sm;
    b->opt_irr_tile = opts->irr_tile_faces;
    if (opts->tune_cache) b->tune_cache = opts->tune_cache;
  }
  b->tile_faces = b->opt_tile_faces;
  b->irr_tile = b->opt_irr_tile;
  int sms = 0;
  UMCP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  for (int t = 0; t < kTypes; ++t) {
    const int npt = t == 0 ? 15 : 16;
    int g = precision == UMCP_FP64 ? batch_face_blocks<double>(kTypeNcp[t], npt)
                                   : batch_face_blocks<float>(kTypeNcp[t], npt);
    b->max_grid[t] = std::max(g, 1);
    if (b->opt_blocks_per_sm > 0) g = std::min(g, b->opt_blocks_per_sm * sms);
    b->face_grid[t] = std::max(g, 1);
  }
  b->vgrid = sms * 8;
  *out = b.release();
  ctx_retain(ctx);
  return UMCP_OK;
}

extern "C" void umcp_batch_destroy(umcp_batch *b) {
  if (!b) return;
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(b->ctx->stream);
  for (Job &J : b->jobs) J.m->batch = nullptr;
  umcp_ctx *ctx = b->ctx;
  delete b;
  ctx_release(ctx);
}

extern "C" umcp_status umcp_batch_add(umcp_batch *b, umcp_mesh *m, const umcp_integrator *it, uint64_t step0,
                                      int64_t n_steps) {
  if (!b || !m || !it) return fail(UMCP_ERR_INVALID, "null argument");
  if (m->ctx != b->ctx) return fail(UMCP_ERR_INVALID, "mesh and batch belong to different contexts");
  if (m->precision != b->precision) return fail(UMCP_ERR_INVALID, "mesh precision differs from the batch's");
  if (m->batch) return fail(UMCP_ERR_INVALID, "mesh is already in a batch");
  if (n_steps < 0) return fail(UMCP_ERR_INVALID, "negative step count");
  if (it->use_mass) return fail(UMCP_ERR_INVALID, "batched jobs use the identity mass (use_mass must be 0)");
  if (m->rs.on) return fail(UMCP_ERR_UNSUPPORTED, "batched jobs have no area/volume restraints");
  for (auto &Gp : m->groups)
    if (type_of(*Gp) < 0) return fail(UMCP_ERR_INVALID, "patch type not supported in a batch");
  Job J;
  J.m = m;
  umcp_status st = make_step_args(m, it, &J.a);
  if (st != UMCP_OK) return st;
  J.threshold = it->divergence_threshold;
  J.step0 = step0;
  J.n_steps = n_steps;
  UMCP_CUDA(cudaSetDevice(b->ctx->device));
  if ((size_t)n_steps > m->energies_cap) {
    // A buffer that exists may be in use by queued steps; a new mesh has none.
    if (m->energies.p) UMCP_CUDA(cudaStreamSynchronize(b->ctx->stream));
    m->drop_graphs();  // the mesh's own graphs hold the energies pointer
    UMCP_CUDA(m->energies.alloc((size_t)n_steps * sizeof(double)));
    m->energies_cap = (size_t)n_steps;
  }
  for (auto &Gp : m->groups) {
    const Group &G = *Gp;
    const int t = type_of(G);
    if (b->have_type[t]) continue;
    UMCP_CUDA(b->basis[t].alloc(G.basis.bytes));
    UMCP_CUDA(b->weight[t].alloc(G.weight.bytes));
    UMCP_CUDA(cudaMemcpyAsync(b->basis[t].p, G.basis.p, G.basis.bytes, cudaMemcpyDeviceToDevice, b->ctx->stream));
    UMCP_CUDA(cudaMemcpyAsync(b->weight[t].p, G.weight.p, G.weight.bytes, cudaMemcpyDeviceToDevice, b->ctx->stream));
    b->npt[t] = G.npt;
    b->dudv[t] = G.dudv;
    b->have_type[t] = true;
    b->drop_graphs();  // the captured steps do not launch this type yet
  }
  b->jobs.push_back(J);
  m->batch = b;
  b->dirty = true;
  return UMCP_OK;
}

extern "C" umcp_status umcp_batch_remove(umcp_batch *b, umcp_mesh *m) {
  if (!b || !m) return fail(UMCP_ERR_INVALID, "null argument");
  if (m->batch != b) return fail(UMCP_ERR_INVALID, "mesh is not in this batch");
  UMCP_CUDA(cudaSetDevice(b->ctx->device));
  UMCP_CUDA(cudaStreamSynchronize(b->ctx->stream));
  batch_forget_mesh(b, m);
  return UMCP_OK;
}

extern "C" umcp_status umcp_batch_run(umcp_batch *b, int n_steps) {
  if (!b || n_steps < 0) return fail(UMCP_ERR_INVALID, "bad argument");
  if (n_steps == 0 || b->jobs.empty()) return UMCP_OK;
  UMCP_CUDA(cudaSetDevice(b->ctx->device));
  cudaStream_t s = b->ctx->stream;
  umcp_status st;
  if ((st = harvest(b)) != UMCP_OK) return st;
  if (b->dirty && (st = rebuild(b)) != UMCP_OK) return st;
  if ((st = start_jobs(b)) != UMCP_OK) return st;
  if ((st = resplit(b)) != UMCP_OK) return st;
  // The face launches' layout (tune cache or timing), at the first run and
  // again whenever the batch has grown fourfold in faces since (a few times
  // at most over a batch's life).
  long long faces = 0;
  for (const Job &J : b->jobs) faces += J.m->nfaces;
  if (b->opt_tile_faces == 0 && (b->tile_faces == 0 || faces >= 4 * b->tuned_faces)) {
    if ((st = autotune(b, faces)) != UMCP_OK) return st;
    b->tuned_faces = faces;
  }
  // kGraphChunk steps at a time, then the rest as one captured run per set bit
  // (20 steps: 16 + 4), so short runs are a few graph launches, not one per
  // step. All six lengths are captured together (at the first run and after a
  // table outgrows its capacity), so no later run pays for a capture.
  for (int i = 0; i < umcp_batch::kPows; ++i)
    if (!b->g_pow[i] && (st = capture(b, 1 << i, &b->g_pow[i])) != UMCP_OK) return st;
  for (int left = n_steps; left > 0;) {
    int i = umcp_batch::kPows - 1;
    while ((1 << i) > left) --i;
    UMCP_CUDA(cudaGraphLaunch(b->g_pow[i], s));
    left -= 1 << i;
  }
  UMCP_CUDA(cudaMemcpyAsync(b->h_prog, b->d_prog.p, 2 * b->jobs.size() * sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, s));
  b->prog_jobs = b->jobs.size();
  return UMCP_OK;
}

static umcp_status status_code(unsigned long long st) {
  if (st & kStatusNonFinite) return UMCP_ERR_NONFINITE;
  if (st & kStatusDiverged) return UMCP_ERR_DIVERGED;
  return UMCP_OK;
}

extern "C" umcp_status umcp_batch_poll(umcp_batch *b, int64_t *steps_done, int *job_status) {
  if (!b) return fail(UMCP_ERR_INVALID, "null argument");
  UMCP_CUDA(cudaSetDevice(b->ctx->device));
  umcp_status st = harvest(b);
  if (st != UMCP_OK) return st;
  for (size_t j = 0; j < b->jobs.size(); ++j) {
    if (steps_done) steps_done[j] = b->jobs[j].done;
    if (job_status) job_status[j] = status_code((unsigned long long)b->jobs[j].status);
  }
  return UMCP_OK;
}

extern "C" umcp_status umcp_batch_job(umcp_batch *b, const umcp_mesh *m, int64_t *steps_done, int *job_status) {
  if (!b || !m) return fail(UMCP_ERR_INVALID, "null argument");
  size_t j = 0;
  while (j < b->jobs.size() && b->jobs[j].m != m) ++j;
  if (j == b->jobs.size()) return fail(UMCP_ERR_INVALID, "mesh is not in this batch");
  std::vector<int64_t> d(b->jobs.size());
  std::vector<int> s(b->jobs.size());
  umcp_status st = umcp_batch_poll(b, d.data(), s.data());
  if (st != UMCP_OK) return st;
  if (steps_done) *steps_done = d[j];
  if (job_status) *job_status = s[j];
  return UMCP_OK;
}

extern "C" umcp_status umcp_batch_info_get(const umcp_batch *b, umcp_batch_info *info) {
  if (!b || !info) return fail(UMCP_ERR_INVALID, "null argument");
  memset(info, 0, sizeof(*info));
  info->n_jobs = (int)b->jobs.size();
  for (const Job &J : b->jobs) {
    info->n_vertices += J.m->nv;
    info->n_faces += J.m->nfaces;
  }
  for (int t = 0; t < kTypes; ++t) {
    info->n_tiles[t] = b->dirty ? 0 : b->counts[kCountTiles + t];
    info->face_grid[t] = b->face_grid[t];
    info->kernels_per_step += b->have_type[t] ? 1 : 0;
  }
  info->kernels_per_step += 2;  // reduce, gather + update
  info->n_vertex_tiles = b->dirty ? 0 : b->counts[kCountVertexTiles];
  info->tile_faces = b->tile_faces;
  info->tuned_face_ms = b->tuned_ms;
  info->irr_tile_faces = b->irr_tile;
  info->tune_source = b->tune_source;
  return UMCP_OK;
}

extern "C" umcp_status umcp_batch_step_host(umcp_batch *b, const double *r_in, double *r_out, double *E,
                                            int n_steps) {
  if (!b || n_steps < 0) return fail(UMCP_ERR_INVALID, "bad argument");
  if (b->jobs.empty()) return UMCP_OK;
  UMCP_CUDA(cudaSetDevice(b->ctx->device));
  cudaStream_t s = b->ctx->stream;
  umcp_status st;
  if ((st = harvest(b)) != UMCP_OK) return st;
  if (b->dirty && (st = rebuild(b)) != UMCP_OK) return st;
  if ((st = start_jobs(b)) != UMCP_OK) return st;
  if ((st = resplit(b)) != UMCP_OK) return st;  // the unpacking keeps the copies of unchanged coordinates
  const size_t bytes = b->pack_doubles * sizeof(double);
  // One copy each way through a device staging pack. (Reading and writing
  // page-locked host memory in place from the (un)pack kernels, over the
  // CPU-GPU link, was slower on GB300: 1.32 ms against 1.11 ms per 256-vesicle
  // host step.)
  if (r_in) {
    UMCP_CUDA(cudaMemcpyAsync(b->d_pack.p, r_in, bytes, cudaMemcpyHostToDevice, s));
    UMCP_CUDA(launch_batch_unpack(b->d_jobs.as<BatchJob>(), b->d_vtiles.as<BatchTile>(), b->d_counts.as<int>(),
                                  b->d_pack_off.as<long long>(), b->d_pack.as<double>(), b->vgrid, s));
  }
  if ((st = umcp_batch_run(b, n_steps)) != UMCP_OK) return st;
  if (r_out || E) {
    UMCP_CUDA(launch_batch_pack(b->d_jobs.as<BatchJob>(), b->d_vtiles.as<BatchTile>(), b->d_counts.as<int>(),
                                b->d_pack_off.as<long long>(), b->d_pack.as<double>(), b->d_pack_E.as<double>(),
                                b->vgrid, s));
    if (r_out) UMCP_CUDA(cudaMemcpyAsync(r_out, b->d_pack.p, bytes, cudaMemcpyDeviceToHost, s));
    if (E) UMCP_CUDA(cudaMemcpyAsync(E, b->d_pack_E.p, b->jobs.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  UMCP_CUDA(cudaStreamSynchronize(s));
  return harvest(b);
}

extern "C" umcp_status umcp_batch_face_pass(umcp_batch *b) {
  if (!b) return fail(UMCP_ERR_INVALID, "null batch");
  if (b->dirty || b->jobs.empty()) return fail(UMCP_ERR_INVALID, "the batch has not run with its current jobs");
  UMCP_CUDA(cudaSetDevice(b->ctx->device));
  UMCP_CUDA(queue_faces(b));
  return UMCP_OK;
}
