// The limit-surface effective mass and its inverse on the device
// (getSparseEffectiveMass, src/modes.C:1719-1990), and the M^-1 apply.
//
// M is assembled on the device, directly as a dense FP64 matrix: every mass
// point of a face is a combination of the face's control points with weights
// that depend on the patch type only, so the 66 points of a face give one
// block per patch type (plan.cpp face_mass_block), which each face adds at
// its control points. Each row's thread adds the blocks of its vertex's
// (face, control point) incidences in their fixed order, so M is
// deterministic and no float atomics are used. It is then factorised and
// inverted there (Cholesky: potrf + potri, as the reference
// does with LAPACK), symmetrised and truncated at the reference's relative
// tolerance (|M^-1_ij| / sqrt(|M^-1_ii M^-1_jj|) > rel_tol, src/modes.C:1893).
// At or above 30% fill M^-1 stays dense and the apply is a dense matrix times
// the three Cartesian components; below it it is stored as CSR (the
// reference's tolerance of 1e-20 leaves a 40,962-vertex vesicle's M^-1 24.7%
// full). The precision form stores FP32 values, with 16-bit columns up to
// 65,536 rows.
//
// The factorisation uses cuSOLVER's dense Cholesky routines, loaded at run
// time so the engine does not depend on the library where no mass matrix is
// built.
#include <dlfcn.h>
#include <stdint.h>
#include <string.h>

#include <chrono>
#include <cmath>
#include <vector>

#include "engine.h"
#include "plan.h"

using namespace umcp;

namespace {

// The dense Cholesky entry points of cuSOLVER, by their C ABI: the handle is
// an opaque pointer, status and fill-mode enums are ints (0 = success,
// 0 = lower triangle).
constexpr int kFillLower = 0;
struct Solver {
  using create_t = int (*)(void **);
  using destroy_t = int (*)(void *);
  using stream_t = int (*)(void *, cudaStream_t);
  using size_t_ = int (*)(void *, int, int, double *, int, int *);
  using run_t = int (*)(void *, int, int, double *, int, double *, int, int *);
  void *lib = nullptr;
  create_t create = nullptr;
  destroy_t destroy = nullptr;
  stream_t set_stream = nullptr;
  size_t_ potrf_size = nullptr, potri_size = nullptr;
  run_t potrf = nullptr, potri = nullptr;
  bool ok() const { return potri != nullptr; }
};

const Solver &solver() {
  static Solver s = [] {
    Solver x;
    for (const char *name : {"libcusolver.so.12", "libcusolver.so.13", "libcusolver.so.11", "libcusolver.so"}) {
      x.lib = dlopen(name, RTLD_NOW | RTLD_LOCAL);
      if (x.lib) break;
    }
    if (!x.lib) return x;
    x.create = (Solver::create_t)dlsym(x.lib, "cusolverDnCreate");
    x.destroy = (Solver::destroy_t)dlsym(x.lib, "cusolverDnDestroy");
    x.set_stream = (Solver::stream_t)dlsym(x.lib, "cusolverDnSetStream");
    x.potrf_size = (Solver::size_t_)dlsym(x.lib, "cusolverDnDpotrf_bufferSize");
    x.potrf = (Solver::run_t)dlsym(x.lib, "cusolverDnDpotrf");
    x.potri_size = (Solver::size_t_)dlsym(x.lib, "cusolverDnDpotri_bufferSize");
    x.potri = (Solver::run_t)dlsym(x.lib, "cusolverDnDpotri");
    if (!x.create || !x.destroy || !x.set_stream || !x.potrf_size || !x.potrf || !x.potri_size) x.potri = nullptr;
    return x;
  }();
  return s;
}

// The face groups of a mesh for the assembly: control points and the group's
// face block (ncp x ncp, row-major).
struct MassGroups {
  const uint32_t *cp[3];
  const double *block[3];
  int ncp[3];
};

// owner[slot] = group << 30 | face << 4 | control point, for every
// gradient-partial slot of the group (slots are one per (face, control point)).
__global__ void slot_owner_kernel(int nfaces, int ncp, int group, const int *__restrict__ dest,
                                  unsigned *__restrict__ owner) {
  const int total = nfaces * ncp;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x)
    owner[dest[t]] = ((unsigned)group << 30) | ((unsigned)(t / ncp) << 4) | (unsigned)(t % ncp);
}

// Row r of M: the rows of the face blocks of r's incidences, in slot order
// (ascending (face, control point)), added into A[r][.]: each row is one
// thread's, so the sums have a fixed order and nothing races.
__global__ void mass_assemble_kernel(int n, const int *__restrict__ off, const unsigned *__restrict__ owner,
                                     MassGroups G, double *__restrict__ A) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const int base = off[2 * r], cnt = off[2 * r + 1];
    double *row = A + (size_t)r * n;
    for (int k = 0; k < cnt; ++k) {
      const unsigned o = owner[base + 32 * k];
      const int g = (int)(o >> 30), f = (int)((o >> 4) & ((1u << 26) - 1)), a = (int)(o & 15u);
      const int N = G.ncp[g];
      const uint32_t *cp = G.cp[g] + (size_t)f * N;
      const double *B = G.block[g] + (size_t)a * N;
      for (int b = 0; b < N; ++b) row[cp[b] & dev::kVertexMask] += B[b];
    }
  }
}

// Nonzero entries of the dense n x n matrix.
__global__ void count_nonzero_kernel(size_t total, const double *__restrict__ A, unsigned long long *__restrict__ cnt) {
  unsigned long long c = 0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
    c += A[e] != 0.0;
  for (int o = 16; o >= 1; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(cnt, c);
}

// potri with the lower triangle (column-major) leaves the inverse in the
// row-major upper triangle; mirror it below the diagonal.
__global__ void symmetrize_kernel(int n, double *__restrict__ A) {
  const size_t total = (size_t)n * n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    if (i > j) A[e] = A[(size_t)j * n + i];
  }
}

// Drops entries at or below rel_tol of the geometric mean of their diagonal
// entries; counts those kept (integer atomics: the count is exact).
__global__ void truncate_kernel(int n, double rel_tol, double *__restrict__ A, unsigned long long *__restrict__ kept) {
  const size_t total = (size_t)n * n;
  unsigned long long k = 0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    const double a = A[e];
    const double d = sqrt(fabs(A[(size_t)i * n + i] * A[(size_t)j * n + j]));
    if (fabs(a) / d > rel_tol) ++k;
    else A[e] = 0.0;
  }
  for (int off = 16; off >= 1; off >>= 1) k += __shfl_xor_sync(0xffffffffu, k, off);
  if ((threadIdx.x & 31) == 0) atomicAdd(kept, k);
}

// out[3i+c] (+)= scale/alpha_c^2 * (scalev ? scalev[c*n+i] : 1) * sum_j A[i][j] in[3j+c].
// One block per row (grid-stride), fixed-order block reduction.
__global__ void dense_apply_kernel(int n, const double *__restrict__ A, const double *__restrict__ scalev, double scale,
                                   const double *__restrict__ alphas, const double *__restrict__ in,
                                   double *__restrict__ out, int accumulate) {
  __shared__ double red[3][8];
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const double *row = A + (size_t)i * n;
    double a0 = 0, a1 = 0, a2 = 0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      const double m = row[j];
      a0 += m * in[3 * (size_t)j];
      a1 += m * in[3 * (size_t)j + 1];
      a2 += m * in[3 * (size_t)j + 2];
    }
    for (int off = 16; off >= 1; off >>= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, off);
      a1 += __shfl_xor_sync(0xffffffffu, a1, off);
      a2 += __shfl_xor_sync(0xffffffffu, a2, off);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { red[0][w] = a0; red[1][w] = a1; red[2][w] = a2; }
    __syncthreads();
    if (threadIdx.x < 3) {
      const int c = threadIdx.x;
      double s = 0;
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[c][k];
      const double al = alphas ? alphas[c] : 1.0;
      double f = scale / (al * al);
      if (scalev) f *= scalev[(size_t)c * n + i];
      const double v = f * s;
      out[3 * (size_t)i + c] = accumulate ? out[3 * (size_t)i + c] + v : v;
    }
    __syncthreads();
  }
}

// dense_apply_kernel on FP32 values and an FP32 input packed as one float4
// per row. One warp takes kDenseRows rows at once, so each coalesced load of
// the input serves all of them; every lane keeps kDenseAhead columns' loads of
// each row in flight (the matrix streams from HBM once, with an evict-first
// hint, while the input stays cached). Kahan-compensated FP32 sums per lane
// and row, then the lanes' sums in FP64 in a fixed butterfly order, and the
// scaling in FP64. (L2 prefetches 8 iterations ahead of each row's loads, as
// the CSR apply makes, took 10,242 rows from 153.5 to 163.9 us; two warps per
// nine rows, one per half of the columns, with twice the loads in flight per
// SM, took 164-166 us.)
constexpr int kDenseRows = 4;
constexpr int kDenseAhead = 4;
constexpr int kDenseThreads = 256;
__global__ void __launch_bounds__(kDenseThreads, 3) dense_apply32_kernel(int n, const float *__restrict__ A,
                                                                      const double *__restrict__ scalev, double scale,
                                                                      const double *__restrict__ alphas,
                                                                      const float4 *__restrict__ in4,
                                                                      double *__restrict__ out, int accumulate) {
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (kDenseThreads / 32);
  for (int i0 = (blockIdx.x * (kDenseThreads / 32) + (threadIdx.x >> 5)) * kDenseRows; i0 < n;
       i0 += warps * kDenseRows) {
    const int nr = n - i0 < kDenseRows ? n - i0 : kDenseRows;
    float s[kDenseRows][3], c[kDenseRows][3];
#pragma unroll
    for (int r = 0; r < kDenseRows; ++r)
#pragma unroll
      for (int q = 0; q < 3; ++q) s[r][q] = c[r][q] = 0.f;
    for (int j0 = lane; j0 < n; j0 += 32 * kDenseAhead) {
      float4 x[kDenseAhead];
      float m[kDenseRows][kDenseAhead];
#pragma unroll
      for (int u = 0; u < kDenseAhead; ++u) {
        const int j = j0 + 32 * u;
        x[u] = j < n ? __ldg(&in4[j]) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int r = 0; r < kDenseRows; ++r)
          m[r][u] = (j < n && r < nr) ? __ldcs(&A[(size_t)(i0 + r) * n + j]) : 0.f;
      }
#pragma unroll
      for (int u = 0; u < kDenseAhead; ++u) {
        if (j0 + 32 * u >= n) break;
        const float xv[3] = {x[u].x, x[u].y, x[u].z};
#pragma unroll
        for (int r = 0; r < kDenseRows; ++r)
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            const float y = fmaf(m[r][u], xv[q], -c[r][q]), t = s[r][q] + y;
            c[r][q] = (t - s[r][q]) - y;
            s[r][q] = t;
          }
      }
    }
    double a[kDenseRows][3];
#pragma unroll
    for (int r = 0; r < kDenseRows; ++r)
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        a[r][q] = (double)s[r][q] - (double)c[r][q];
        for (int off = 16; off >= 1; off >>= 1) a[r][q] += __shfl_xor_sync(0xffffffffu, a[r][q], off);
      }
    // lane 3 r + q writes component q of row i0 + r
#pragma unroll
    for (int r = 0; r < kDenseRows; ++r)
#pragma unroll
      for (int q = 0; q < 3; ++q)
        if (lane == 3 * r + q && r < nr) {
          const int i = i0 + r;
          const double al = alphas ? alphas[q] : 1.0;
          double f = scale / (al * al);
          if (scalev) f *= scalev[(size_t)q * n + i];
          const double v = f * a[r][q];
          out[3 * (size_t)i + q] = accumulate ? out[3 * (size_t)i + q] + v : v;
        }
  }
}

// Kept entries of each row of the truncated inverse (one warp per row).
__global__ void row_count_kernel(int n, const double *__restrict__ A, int *__restrict__ cnt) {
  const int lane = threadIdx.x & 31;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += (gridDim.x * blockDim.x) >> 5) {
    const double *row = A + (size_t)i * n;
    int c = 0;
    for (int j = lane; j < n; j += 32) c += row[j] != 0.0;
    for (int off = 16; off >= 1; off >>= 1) c += __shfl_xor_sync(0xffffffffu, c, off);
    if (lane == 0) cnt[i] = c;
  }
}

// CSR of the truncated inverse, columns ascending within each row (one warp
// per row: a ballot over 32 columns at a time gives each kept entry its
// place). V is double (plain path) or float (precision form, rounded once).
template <typename V, typename C>  // C: int, or uint16_t for up to 65,536 columns
__global__ void row_fill_kernel(int n, const double *__restrict__ A, const int *__restrict__ row_ptr,
                                C *__restrict__ col, V *__restrict__ val) {
  const int lane = threadIdx.x & 31;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += (gridDim.x * blockDim.x) >> 5) {
    const double *row = A + (size_t)i * n;
    int w = row_ptr[i];
    for (int j0 = 0; j0 < n; j0 += 32) {
      const int j = j0 + lane;
      const double a = j < n ? row[j] : 0.0;
      const unsigned keep = __ballot_sync(0xffffffffu, a != 0.0);
      if (a != 0.0) {
        const int at = w + __popc(keep & ((1u << lane) - 1u));
        col[at] = (C)j;
        val[at] = (V)a;
      }
      w += __popc(keep);
    }
  }
}

__global__ void dense_to_f32_kernel(size_t total, const double *__restrict__ A, float *__restrict__ B) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
    B[e] = (float)A[e];
}

}  // namespace

cudaError_t umcp::queue_mass_apply(umcp_mesh *m, const double *scalev, double scale, const double *alphas,
                                   const double *in, double *out, int accumulate, cudaStream_t s) {
  if (m->mass_f32) {
    cudaError_t e = launch_to_f32x4(m->mrows, in, m->min32.as<float4>(), s);
    if (e != cudaSuccess) return e;
    if (!m->mass_dense)
      return launch_spmv32(m->mrows, m->mrow.as<int>(), m->mcol.p, m->mcol16, m->mval.as<float>(), scalev, scale, alphas,
                           m->min32.as<float4>(), out, accumulate, s);
  }
  if (m->mass_dense) {
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->ctx->device);
    const int grid = m->mrows < sms * 8 ? m->mrows : sms * 8;
    if (m->mass_f32) {
      const int groups = (m->mrows + kDenseRows - 1) / kDenseRows, per_block = kDenseThreads / 32;
      const int blocks = (groups + per_block - 1) / per_block;
      dense_apply32_kernel<<<blocks < sms * 8 ? blocks : sms * 8, kDenseThreads, 0, s>>>(
          m->mrows, m->mdense.as<float>(), scalev, scale, alphas, m->min32.as<float4>(), out, accumulate);
    } else
      dense_apply_kernel<<<grid, 256, 0, s>>>(m->mrows, m->mdense.as<double>(), scalev, scale, alphas, in, out,
                                              accumulate);
    return cudaGetLastError();
  }
  return launch_spmv(m->mrows, m->mrow.as<int>(), m->mcol.as<int>(), m->mval.as<double>(), scalev, scale, alphas, in,
                     out, accumulate, s);
}

static umcp_status fail(umcp_status s, const std::string &msg) { return umcp::set_error(s, msg); }

extern "C" umcp_status umcp_mass_build(umcp_mesh *m, const umcp_plan *plan, const umcp_mass_opts *opts,
                                       umcp_mass_info *info) {
  if (!m || !plan) return fail(UMCP_ERR_INVALID, "null argument");
  umcp_mass_opts o{5.0, 10, 1e-20};
  if (opts) o = *opts;
  if (!(o.mass_scale > 0) || o.points_per_edge < 1 || !(o.rel_tol >= 0))
    return fail(UMCP_ERR_INVALID, "mass options: mass_scale > 0, points_per_edge >= 1, rel_tol >= 0");
  const Plan &P = plan_of(plan);
  const int n = m->nv;
  if ((int)(P.reg_faces.size() + P.irr_faces.size()) != m->nfaces) return fail(UMCP_ERR_INVALID, "plan does not match the mesh");
  const Solver &S = solver();
  if (!S.ok()) return fail(UMCP_ERR_UNSUPPORTED, "cuSOLVER (dense Cholesky) is not available on this host");

  if (m->groups.size() > 3 || m->nfaces >= (1 << 26)) return fail(UMCP_ERR_UNSUPPORTED, "mesh too large for the mass assembly");
  const auto t_start = std::chrono::steady_clock::now();
  const MassPoints MP = mass_points(P, o.mass_scale, o.points_per_edge);

  UMCP_CUDA(cudaSetDevice(m->ctx->device));
  cudaStream_t s = m->ctx->stream;
  UMCP_CUDA(cudaStreamSynchronize(s));  // queued steps may still read the previous M^-1
  m->drop_graphs();
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->ctx->device);
  DevBuf A, owner, blocks[3], work, dinfo, dkept, dnnz;
  UMCP_CUDA(A.alloc((size_t)n * n * sizeof(double)));
  UMCP_CUDA(cudaMemsetAsync(A.p, 0, A.bytes, s));
  UMCP_CUDA(owner.alloc((size_t)std::max(m->nslot_cap, 1) * sizeof(unsigned)));
  MassGroups MG{};
  for (size_t g = 0; g < m->groups.size(); ++g) {
    const Group &G = *m->groups[g];
    std::vector<double> B((size_t)G.ncp * G.ncp);
    face_mass_block(G.valence, G.ncp, o.points_per_edge, MP.mass_per_point, B.data());
    UMCP_CUDA(upload(blocks[g], B));
    MG.cp[g] = G.cp.as<uint32_t>();
    MG.block[g] = blocks[g].as<double>();
    MG.ncp[g] = G.ncp;
    if (G.nfaces)
      slot_owner_kernel<<<sms * 4, 256, 0, s>>>(G.nfaces, G.ncp, (int)g, G.dest.as<int>(), owner.as<unsigned>());
  }
  mass_assemble_kernel<<<(n + 127) / 128, 128, 0, s>>>(n, m->off.as<int>(), owner.as<unsigned>(), MG, A.as<double>());
  UMCP_CUDA(cudaGetLastError());
  UMCP_CUDA(dnnz.alloc(sizeof(unsigned long long)));
  UMCP_CUDA(cudaMemsetAsync(dnnz.p, 0, sizeof(unsigned long long), s));
  count_nonzero_kernel<<<sms * 8, 256, 0, s>>>((size_t)n * n, A.as<double>(), dnnz.as<unsigned long long>());
  UMCP_CUDA(cudaGetLastError());
  unsigned long long nnz_mass = 0;
  UMCP_CUDA(cudaMemcpyAsync(&nnz_mass, dnnz.p, sizeof nnz_mass, cudaMemcpyDeviceToHost, s));
  UMCP_CUDA(cudaStreamSynchronize(s));
  const auto t_assembled = std::chrono::steady_clock::now();

  void *h = nullptr;
  if (S.create(&h) != 0) return fail(UMCP_ERR_CUDA, "cusolverDnCreate failed");
  struct Guard { const Solver &S; void *h; ~Guard() { S.destroy(h); } } guard{S, h};
  S.set_stream(h, s);
  int lw1 = 0, lw2 = 0;
  if (S.potrf_size(h, kFillLower, n, A.as<double>(), n, &lw1) != 0 ||
      S.potri_size(h, kFillLower, n, A.as<double>(), n, &lw2) != 0)
    return fail(UMCP_ERR_CUDA, "cuSOLVER workspace query failed");
  UMCP_CUDA(work.alloc((size_t)std::max(std::max(lw1, lw2), 1) * sizeof(double)));
  UMCP_CUDA(dinfo.alloc(sizeof(int)));
  int hinfo = 0;
  if (S.potrf(h, kFillLower, n, A.as<double>(), n, work.as<double>(), lw1, dinfo.as<int>()) !=
      0)
    return fail(UMCP_ERR_CUDA, "cusolverDnDpotrf failed");
  UMCP_CUDA(cudaMemcpyAsync(&hinfo, dinfo.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  UMCP_CUDA(cudaStreamSynchronize(s));
  if (hinfo != 0)
    return fail(UMCP_ERR_INVALID, "effective mass matrix is not positive definite (the reference stops here, "
                                  "src/modes.C:1833-1837)");
  if (S.potri(h, kFillLower, n, A.as<double>(), n, work.as<double>(), lw2, dinfo.as<int>()) !=
      0)
    return fail(UMCP_ERR_CUDA, "cusolverDnDpotri failed");
  UMCP_CUDA(cudaMemcpyAsync(&hinfo, dinfo.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  UMCP_CUDA(cudaStreamSynchronize(s));
  if (hinfo != 0) return fail(UMCP_ERR_INVALID, "effective mass matrix could not be inverted");
  const auto t_inverted = std::chrono::steady_clock::now();
  symmetrize_kernel<<<sms * 8, 256, 0, s>>>(n, A.as<double>());
  UMCP_CUDA(cudaGetLastError());
  UMCP_CUDA(dkept.alloc(sizeof(unsigned long long)));
  UMCP_CUDA(cudaMemsetAsync(dkept.p, 0, sizeof(unsigned long long), s));
  truncate_kernel<<<sms * 8, 256, 0, s>>>(n, o.rel_tol, A.as<double>(), dkept.as<unsigned long long>());
  UMCP_CUDA(cudaGetLastError());
  unsigned long long kept = 0;
  UMCP_CUDA(cudaMemcpyAsync(&kept, dkept.p, sizeof kept, cudaMemcpyDeviceToHost, s));
  UMCP_CUDA(cudaStreamSynchronize(s));

  const double fill = (double)kept / ((double)n * n);
  // the precision form keeps M^-1 in FP32 (rounded once from the FP64 inverse)
  const bool f32 = m->precision == UMCP_FP32_CENTRED;
  if (fill >= 0.3) {
    if (f32) {
      UMCP_CUDA(m->mdense.alloc((size_t)n * n * sizeof(float)));
      dense_to_f32_kernel<<<sms * 8, 256, 0, s>>>((size_t)n * n, A.as<double>(), m->mdense.as<float>());
      UMCP_CUDA(cudaGetLastError());
      UMCP_CUDA(cudaStreamSynchronize(s));
    } else {
      std::swap(m->mdense.p, A.p);
      std::swap(m->mdense.bytes, A.bytes);
    }
    m->mass_dense = true;
    m->mcol16 = false;
    UMCP_CUDA(m->mrow.alloc(0));
    UMCP_CUDA(m->mcol.alloc(0));
    UMCP_CUDA(m->mval.alloc(0));
  } else {
    // CSR on the device: kept entries per row, their prefix sums (on the
    // host: n + 1 integers), then each row's entries in column order.
    if (kept > (unsigned long long)INT32_MAX) return fail(UMCP_ERR_UNSUPPORTED, "M^-1 has more than 2^31 nonzeros");
    DevBuf dcnt;
    UMCP_CUDA(dcnt.alloc((size_t)n * sizeof(int)));
    row_count_kernel<<<sms * 8, 256, 0, s>>>(n, A.as<double>(), dcnt.as<int>());
    UMCP_CUDA(cudaGetLastError());
    std::vector<int> cnt((size_t)n), rp((size_t)n + 1, 0);
    UMCP_CUDA(cudaMemcpyAsync(cnt.data(), dcnt.p, cnt.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
    UMCP_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < n; ++i) rp[(size_t)i + 1] = rp[i] + cnt[i];
    if ((unsigned long long)rp[n] != kept) return fail(UMCP_ERR_CUDA, "M^-1 nonzero count mismatch between the truncation and the CSR pass");
    UMCP_CUDA(upload(m->mrow, rp));
    m->mcol16 = f32 && n <= 65536;
    UMCP_CUDA(m->mcol.alloc(kept * (m->mcol16 ? sizeof(uint16_t) : sizeof(int))));
    UMCP_CUDA(m->mval.alloc(kept * (f32 ? sizeof(float) : sizeof(double))));
    if (m->mcol16)
      row_fill_kernel<float, uint16_t><<<sms * 8, 256, 0, s>>>(n, A.as<double>(), m->mrow.as<int>(),
                                                              m->mcol.as<uint16_t>(), m->mval.as<float>());
    else if (f32)
      row_fill_kernel<float, int><<<sms * 8, 256, 0, s>>>(n, A.as<double>(), m->mrow.as<int>(), m->mcol.as<int>(),
                                                         m->mval.as<float>());
    else
      row_fill_kernel<double, int><<<sms * 8, 256, 0, s>>>(n, A.as<double>(), m->mrow.as<int>(), m->mcol.as<int>(),
                                                          m->mval.as<double>());
    UMCP_CUDA(cudaGetLastError());
    UMCP_CUDA(cudaStreamSynchronize(s));
    UMCP_CUDA(m->mdense.alloc(0));
    m->mass_dense = false;
  }
  m->mass_f32 = f32;
  UMCP_CUDA(m->min32.alloc(f32 ? (size_t)n * sizeof(float4) : 0));
  m->mrows = n;
  if (info) {
    const auto t_end = std::chrono::steady_clock::now();
    auto sec = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
      return std::chrono::duration<double>(b - a).count();
    };
    memset(info, 0, sizeof(*info));
    info->area0 = MP.area0;
    info->mass_per_point = MP.mass_per_point;
    info->points = MP.points;
    info->nnz_mass = (long long)nnz_mass;
    info->nnz_inverse = (long long)kept;
    info->dense = m->mass_dense ? 1 : 0;
    info->column_bytes = (long long)(m->mass_dense ? 0 : m->mcol.bytes);
    info->assembly_s = sec(t_start, t_assembled);
    info->inverse_s = sec(t_assembled, t_inverted);
    info->truncation_s = sec(t_inverted, t_end);
  }
  return UMCP_OK;
}

extern "C" umcp_status umcp_mass_get(umcp_mesh *m, double *dense) {
  if (!m || !dense) return fail(UMCP_ERR_INVALID, "null argument");
  if (!m->mrows) return fail(UMCP_ERR_INVALID, "no mass matrix installed");
  UMCP_CUDA(cudaSetDevice(m->ctx->device));
  UMCP_CUDA(cudaStreamSynchronize(m->ctx->stream));
  const int n = m->mrows;
  if (m->mass_dense) {
    if (m->mass_f32) {
      std::vector<float> a((size_t)n * n);
      UMCP_CUDA(cudaMemcpy(a.data(), m->mdense.p, a.size() * sizeof(float), cudaMemcpyDeviceToHost));
      for (size_t e = 0; e < a.size(); ++e) dense[e] = a[e];
    } else {
      UMCP_CUDA(cudaMemcpy(dense, m->mdense.p, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToHost));
    }
    return UMCP_OK;
  }
  std::vector<int> rp((size_t)n + 1);
  UMCP_CUDA(cudaMemcpy(rp.data(), m->mrow.p, rp.size() * sizeof(int), cudaMemcpyDeviceToHost));
  std::vector<int> cl((size_t)rp[n]);
  std::vector<double> vl((size_t)rp[n]);
  if (rp[n] > 0) {
    if (m->mcol16) {
      std::vector<uint16_t> c16(cl.size());
      UMCP_CUDA(cudaMemcpy(c16.data(), m->mcol.p, c16.size() * sizeof(uint16_t), cudaMemcpyDeviceToHost));
      for (size_t k = 0; k < cl.size(); ++k) cl[k] = c16[k];
    } else {
      UMCP_CUDA(cudaMemcpy(cl.data(), m->mcol.p, cl.size() * sizeof(int), cudaMemcpyDeviceToHost));
    }
    if (m->mass_f32) {
      std::vector<float> v32(vl.size());
      UMCP_CUDA(cudaMemcpy(v32.data(), m->mval.p, v32.size() * sizeof(float), cudaMemcpyDeviceToHost));
      for (size_t k = 0; k < vl.size(); ++k) vl[k] = v32[k];
    } else {
      UMCP_CUDA(cudaMemcpy(vl.data(), m->mval.p, vl.size() * sizeof(double), cudaMemcpyDeviceToHost));
    }
  }
  memset(dense, 0, (size_t)n * n * sizeof(double));
  for (int i = 0; i < n; ++i)
    for (int k = rp[i]; k < rp[(size_t)i + 1]; ++k) dense[(size_t)i * n + cl[k]] += vl[k];
  return UMCP_OK;
}
