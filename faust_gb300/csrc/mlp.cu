// mlp.cu — elementwise kernels and entry points of the warm-start MLP
// (declared in include/fgb_mlp.h); the GEMMs run in gemm_tc.cu.
#include <algorithm>

#include "../../include/fgb_mlp.h"
#include "fgb_internal.cuh"

namespace fgb {
fgb_status launch_gemm_bf16(fgb_ctx* ctx, int M, int N, int K, const void* A, long lda, const void* B, long ldb,
                            void* C, long ldc, int c_f32, const float* bias, int act, int split_k, float* work);

static int grid_n(fgb_ctx* ctx, long n) {
  return (int)std::max(1L, std::min((n + 255) / 256, 8L * ctx->sm_count));
}

// 32 x 32 tiles through shared memory
__global__ void k_transpose_bf16(const __nv_bfloat16* __restrict__ in, long ldi, int rows, int cols,
                                 __nv_bfloat16* __restrict__ out, long ldo) {
  __shared__ __nv_bfloat16 t[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = r0 + j, c = c0 + threadIdx.x;
    if (r < rows && c < cols) t[j][threadIdx.x] = in[(long)r * ldi + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int c = c0 + j, r = r0 + threadIdx.x;
    if (r < rows && c < cols) out[(long)c * ldo + r] = t[threadIdx.x][j];
  }
}

__global__ void k_relu_grad(long n, const __nv_bfloat16* __restrict__ dy, const __nv_bfloat16* __restrict__ y,
                            __nv_bfloat16* __restrict__ dx) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    dx[i] = __bfloat162float(y[i]) > 0.f ? dy[i] : __float2bfloat16(0.f);
}

__global__ void k_colsum(int rows, int cols, const __nv_bfloat16* __restrict__ x, long ld, float* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int r = 0; r < rows; ++r) s += __bfloat162float(x[(long)r * ld + c]);
  out[c] = s;
}

__global__ void k_mse_grad(long n, const float* __restrict__ pred, const float* __restrict__ target, float scale,
                           __nv_bfloat16* __restrict__ grad, float* loss) {
  float acc = 0.f;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float d = pred[i] - target[i];
    grad[i] = __float2bfloat16(scale * d);
    acc += d * d;
  }
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, 0.5f * scale * acc);
}

__global__ void k_adam(long n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, __nv_bfloat16* __restrict__ wb, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
  }
}

__global__ void k_f2b(long n, const float* __restrict__ in, __nv_bfloat16* __restrict__ out) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = __float2bfloat16(in[i]);
}
__global__ void k_b2f(long n, const __nv_bfloat16* __restrict__ in, float* __restrict__ out) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = __bfloat162float(in[i]);
}

}  // namespace fgb

using namespace fgb;

extern "C" {

fgb_status fgb_gemm_bf16(fgb_ctx* ctx, int M, int N, int K, const void* A, long lda, const void* B, long ldb,
                         void* C, long ldc, int c_dtype, const float* bias, int relu, int split_k, float* workspace) {
  if (!ctx || !A || !B || !C) return FGB_ERR_INVALID_ARG;
  if (c_dtype != FGB_F32 && c_dtype != FGB_BF16) return fail(ctx, FGB_ERR_INVALID_ARG, "gemm: C is F32 or BF16");
  return launch_gemm_bf16(ctx, M, N, K, A, lda, B, ldb, C, ldc, c_dtype == FGB_F32, bias, relu ? 1 : 0, split_k,
                          workspace);
}

fgb_status fgb_mlp_transpose_bf16(fgb_ctx* ctx, int rows, int cols, const void* in, long ldi, void* out, long ldo) {
  if (!ctx || !in || !out || rows < 0 || cols < 0) return FGB_ERR_INVALID_ARG;
  dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
  k_transpose_bf16<<<grid, block, 0, ctx->stream>>>((const __nv_bfloat16*)in, ldi, rows, cols, (__nv_bfloat16*)out,
                                                    ldo);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

fgb_status fgb_mlp_relu_grad(fgb_ctx* ctx, long n, const void* dy, const void* y, void* dx) {
  if (!ctx || !dy || !y || !dx) return FGB_ERR_INVALID_ARG;
  k_relu_grad<<<grid_n(ctx, n), 256, 0, ctx->stream>>>(n, (const __nv_bfloat16*)dy, (const __nv_bfloat16*)y,
                                                       (__nv_bfloat16*)dx);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

fgb_status fgb_mlp_colsum(fgb_ctx* ctx, int rows, int cols, const void* x, long ld, float* out) {
  if (!ctx || !x || !out) return FGB_ERR_INVALID_ARG;
  k_colsum<<<(cols + 255) / 256, 256, 0, ctx->stream>>>(rows, cols, (const __nv_bfloat16*)x, ld, out);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

fgb_status fgb_mlp_mse_grad(fgb_ctx* ctx, long n, const float* pred, const float* target, float scale, void* grad,
                            float* loss) {
  if (!ctx || !pred || !target || !grad) return FGB_ERR_INVALID_ARG;
  k_mse_grad<<<grid_n(ctx, n), 256, 0, ctx->stream>>>(n, pred, target, scale, (__nv_bfloat16*)grad, loss);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

fgb_status fgb_mlp_adam(fgb_ctx* ctx, long n, float* w, const float* g, float* m, float* v, void* w_bf16, float lr,
                        float beta1, float beta2, float eps, int step) {
  if (!ctx || !w || !g || !m || !v || step < 1) return FGB_ERR_INVALID_ARG;
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  k_adam<<<grid_n(ctx, n), 256, 0, ctx->stream>>>(n, w, g, m, v, (__nv_bfloat16*)w_bf16, lr, beta1, beta2, eps, c1,
                                                  c2);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

fgb_status fgb_mlp_f32_to_bf16(fgb_ctx* ctx, long n, const float* in, void* out) {
  if (!ctx || !in || !out) return FGB_ERR_INVALID_ARG;
  k_f2b<<<grid_n(ctx, n), 256, 0, ctx->stream>>>(n, in, (__nv_bfloat16*)out);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

fgb_status fgb_mlp_bf16_to_f32(fgb_ctx* ctx, long n, const void* in, float* out) {
  if (!ctx || !in || !out) return FGB_ERR_INVALID_ARG;
  k_b2f<<<grid_n(ctx, n), 256, 0, ctx->stream>>>(n, (const __nv_bfloat16*)in, out);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

}  // extern "C"
