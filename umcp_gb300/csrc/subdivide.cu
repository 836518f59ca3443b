// Batched Loop subdivision of regular 12-point patches (the fast_sub6_*
// stencils of src/fast_mm.C used by the reference's mesh-collision code): each
// patch's 12 control points (36 doubles, xyz per point) give the 4 x 12
// control points of its child patches. The 4 x 12 x 12 stencil (plan.cpp
// subdivision_stencils) sits in constant memory; one thread per output
// coordinate, so reads of a patch are shared through L1 and writes coalesce.
#include <mutex>

#include "engine.h"
#include "plan.h"

using namespace umcp;

namespace {

__constant__ double c_stencil[4][12][12];

__global__ void subdivide_kernel(long long n, const double *__restrict__ in, double *__restrict__ out) {
  const long long total = n * 144;  // 4 children x 36 coordinates per patch
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long p = e / 144;
    const int r = (int)(e % 144), k = r / 36, i = (r % 36) / 3, c = r % 3;
    const double *src = in + p * 36 + c;
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 12; ++j) s += c_stencil[k][i][j] * src[3 * j];
    out[e] = s;
  }
}

std::once_flag g_once[128];
cudaError_t g_upload[128];

}  // namespace

static umcp_status fail(umcp_status s, const std::string &msg) { return umcp::set_error(s, msg); }

extern "C" umcp_status umcp_subdivision_stencils(double *S) {
  if (!S) return fail(UMCP_ERR_INVALID, "null argument");
  subdivision_stencils(reinterpret_cast<double(*)[12][12]>(S));
  return UMCP_OK;
}

extern "C" umcp_status umcp_subdivide_patches(umcp_ctx *ctx, const double *d_in, double *d_out, long long n) {
  if (!ctx || n < 0 || (n > 0 && (!d_in || !d_out))) return fail(UMCP_ERR_INVALID, "bad argument");
  if (n == 0) return UMCP_OK;
  UMCP_CUDA(cudaSetDevice(ctx->device));
  if (ctx->device < 0 || ctx->device >= 128) return fail(UMCP_ERR_INVALID, "device index out of range");
  std::call_once(g_once[ctx->device], [&] {
    double S[4][12][12];
    subdivision_stencils(S);
    g_upload[ctx->device] = cudaMemcpyToSymbol(c_stencil, S, sizeof S);
  });
  UMCP_CUDA(g_upload[ctx->device]);
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  const long long blocks = (n * 144 + 255) / 256;
  const int grid = (int)(blocks < sms * 8 ? blocks : sms * 8);
  subdivide_kernel<<<grid, 256, 0, ctx->stream>>>(n, d_in, d_out);
  UMCP_CUDA(cudaGetLastError());
  return UMCP_OK;
}
