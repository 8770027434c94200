// ctx.cu — context, errors and allocation helpers of libfaust_gb300.
#include <cstdarg>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>

#include "fgb_internal.cuh"

namespace fgb {

fgb_status fail(fgb_ctx* ctx, fgb_status st, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    ctx->err = buf;
  }
  return st;
}

fgb_status cuda_check(fgb_ctx* ctx, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return FGB_OK;
  if (e == cudaErrorMemoryAllocation) return fail(ctx, FGB_ERR_OOM, "%s: out of device memory", what);
  return fail(ctx, FGB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

size_t dtype_size(fgb_dtype t) {
  switch (t) {
    case FGB_F32: return 4;
    case FGB_F64: return 8;
    case FGB_BF16: return 2;
  }
  return 0;
}

fgb_status dmalloc(fgb_ctx* ctx, void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return cuda_check(ctx, e, "cudaMalloc");
  }
  return FGB_OK;
}

fgb_status kernel_err_word(fgb_ctx* ctx, int** out) {
  if (!ctx->kerr) {
    void* d = nullptr;
    FGB_TRY(dmalloc(ctx, &d, sizeof(int)));
    cudaError_t e = cudaMemsetAsync(d, 0, sizeof(int), ctx->stream);
    if (e != cudaSuccess) {
      cudaFree(d);
      return cuda_check(ctx, e, "kernel error word");
    }
    ctx->kerr = (int*)d;
  }
  *out = ctx->kerr;
  return FGB_OK;
}

fgb_status check_kernel_err(fgb_ctx* ctx) {
  if (!ctx->kerr) return FGB_OK;
  int h = 0;
  FGB_CUDA(ctx, cudaMemcpy(&h, ctx->kerr, sizeof(int), cudaMemcpyDeviceToHost));
  if (!h) return FGB_OK;
  FGB_CUDA(ctx, cudaMemset(ctx->kerr, 0, sizeof(int)));
  return fail(ctx, FGB_ERR_TIMEOUT, "a bounded device-side wait ran out in a tensor-core or butterfly kernel");
}

fgb_status smem_opt_in(fgb_ctx* ctx, const void* func, size_t bytes) {
  if (bytes <= 48 * 1024) return FGB_OK;
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> done;
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = done[{func, ctx->device}];
  if (cur >= bytes) return FGB_OK;
  FGB_CUDA(ctx, cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  cur = bytes;
  return FGB_OK;
}

void dfree(void* p) {
  if (p) cudaFree(p);
}

}  // namespace fgb

using namespace fgb;

extern "C" {

fgb_status fgb_ctx_create(int device, void* cuda_stream, fgb_ctx** out) {
  if (!out) return FGB_ERR_INVALID_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return FGB_ERR_CUDA;
  }
  if (device < 0 || device >= ndev) return FGB_ERR_INVALID_ARG;
  fgb_ctx* ctx = new fgb_ctx();
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess) {
    delete ctx;
    return FGB_ERR_CUDA;
  }
  cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  ctx->smem_optin = (size_t)optin;
  // The caller's stream is used as given; NULL is the legacy default stream.
  ctx->stream = (cudaStream_t)cuda_stream;
  ctx->own_stream = false;
  void* hp = nullptr;
  if (cudaHostAlloc(&hp, sizeof(int), cudaHostAllocMapped) == cudaSuccess) {
    ctx->cancel_host = (volatile int*)hp;
    *ctx->cancel_host = 0;
    void* dp = nullptr;
    if (cudaHostGetDevicePointer(&dp, hp, 0) == cudaSuccess) ctx->cancel_dev = (int*)dp;
  }
  if (cudaStreamCreateWithFlags(&ctx->s_long, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_long_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_long_join, cudaEventDisableTiming) != cudaSuccess) {
    if (ctx->s_long) cudaStreamDestroy(ctx->s_long);
    if (ctx->ev_long_fork) cudaEventDestroy(ctx->ev_long_fork);
    ctx->s_long = nullptr;
    ctx->ev_long_fork = nullptr;
    ctx->ev_long_join = nullptr;
  }
  cudaGetLastError();
  *out = ctx;
  return FGB_OK;
}

fgb_status fgb_ctx_destroy(fgb_ctx* ctx) {
  if (!ctx) return FGB_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->cancel_host) cudaFreeHost((void*)ctx->cancel_host);
  if (ctx->rand_dev) cudaFree(ctx->rand_dev);
  if (ctx->x0_d) cudaFree(ctx->x0_d);
  if (ctx->x0_f) cudaFree(ctx->x0_f);
  if (ctx->kerr) cudaFree(ctx->kerr);
  if (ctx->s_long) {
    cudaStreamSynchronize(ctx->s_long);
    cudaStreamDestroy(ctx->s_long);
  }
  if (ctx->ev_long_fork) cudaEventDestroy(ctx->ev_long_fork);
  if (ctx->ev_long_join) cudaEventDestroy(ctx->ev_long_join);
  delete ctx;
  return FGB_OK;
}

const char* fgb_last_error(const fgb_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

fgb_status fgb_ctx_synchronize(fgb_ctx* ctx) {
  if (!ctx) return FGB_ERR_INVALID_ARG;
  FGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return check_kernel_err(ctx);
}

fgb_status fgb_cancel(fgb_ctx* ctx) {
  if (!ctx || !ctx->cancel_host) return FGB_ERR_INVALID_ARG;
  *ctx->cancel_host = 1;
  return FGB_OK;
}

long long fgb_ctx_kernel_launches(const fgb_ctx* ctx) { return ctx ? ctx->launches.load() : -1; }

}  // extern "C"
