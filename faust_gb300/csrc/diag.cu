// diag.cu — FP64 FMA throughput probe (roofline denominator of the FP64
// kernels: the measured copy bandwidth and GEMM rates do not cover the
// scalar FP64 pipe).
#include "fgb_internal.cuh"
#include "../../include/fgb_diag.h"

namespace fgb {

__global__ void __launch_bounds__(256) k_fp64_fma(double* out, int iters, double a) {
  double x[8];
#pragma unroll
  for (int u = 0; u < 8; ++u) x[u] = (double)(threadIdx.x + u) * 1e-3;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 8; ++u) x[u] = __fma_rn(x[u], a, 1e-9);
  }
  double s = 0;
#pragma unroll
  for (int u = 0; u < 8; ++u) s += x[u];
  if (s == 12345.678) out[blockIdx.x] = s;  // keeps the loop; never true for these inputs
}

}  // namespace fgb

using namespace fgb;

extern "C" fgb_status fgb_probe_fp64_fma(fgb_ctx* ctx, double* flops) {
  if (!ctx || !flops) return FGB_ERR_INVALID_ARG;
  FGB_CUDA(ctx, cudaSetDevice(ctx->device));
  double* out = nullptr;
  const int blocks = ctx->sm_count * 8, iters = 4096;
  FGB_TRY(dmalloc(ctx, (void**)&out, sizeof(double) * blocks));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  fgb_status s = cuda_check(ctx, cudaEventCreate(&e0), "event");
  if (s == FGB_OK) s = cuda_check(ctx, cudaEventCreate(&e1), "event");
  float ms = 0;
  if (s == FGB_OK) {
    k_fp64_fma<<<blocks, 256, 0, ctx->stream>>>(out, iters / 8, 0.999999);  // warm-up
    cudaEventRecord(e0, ctx->stream);
    k_fp64_fma<<<blocks, 256, 0, ctx->stream>>>(out, iters, 0.999999);
    cudaEventRecord(e1, ctx->stream);
    s = cuda_check(ctx, cudaEventSynchronize(e1), "fp64 probe");
    ctx->launches.fetch_add(2);
  }
  if (s == FGB_OK) s = cuda_check(ctx, cudaEventElapsedTime(&ms, e0, e1), "elapsed");
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  dfree(out);
  if (s != FGB_OK) return s;
  *flops = 2.0 * (double)blocks * 256 * iters * 8 / (ms * 1e-3);
  return FGB_OK;
}
