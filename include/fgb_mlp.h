/* fgb_mlp.h — kernels of the learned warm start for palm4msa2: a BF16 MLP
 * that predicts butterfly-factor values from the target matrix.  These entry
 * points have no counterpart in the reference (FAuST has no learned
 * initialisation); they are the network's own forward / backward / update
 * kernels.  Same conventions as fgb.h: fgb_status returns, work queued on the
 * context's stream, DEVICE pointers, row-major matrices with leading
 * dimensions in elements. */
#ifndef FGB_MLP_H
#define FGB_MLP_H

#include "fgb.h"

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* C[M x N] = A[M x K] * B[N x K]^T (+ bias[N]) (ReLU if relu) on the tcgen05
 * tensor cores: A, B BF16 row-major, FP32 accumulation, C BF16 (c_dtype =
 * FGB_BF16) or FP32 (FGB_F32).  M, N multiples of 128, K of 64.  split_k > 1
 * splits K over CTAs with FP32 atomics into `workspace` (M*N floats; may be
 * NULL when C is FP32 without bias/ReLU). */
fgb_status fgb_gemm_bf16(fgb_ctx* ctx, int M, int N, int K, const void* A, long lda, const void* B, long ldb,
                         void* C, long ldc, int c_dtype, const float* bias, int relu, int split_k, float* workspace);

/* out[c, r] = in[r, c] for a rows x cols BF16 matrix. */
fgb_status fgb_mlp_transpose_bf16(fgb_ctx* ctx, int rows, int cols, const void* in, long ldi, void* out, long ldo);

/* dx = dy * (y > 0), BF16, n entries (ReLU backward from its output). */
fgb_status fgb_mlp_relu_grad(fgb_ctx* ctx, long n, const void* dy, const void* y, void* dx);

/* out[c] = sum_r x[r, c] (FP32) of a rows x cols BF16 matrix (bias gradient). */
fgb_status fgb_mlp_colsum(fgb_ctx* ctx, int rows, int cols, const void* x, long ld, float* out);

/* grad = scale * (pred - target) as BF16 and loss = 0.5*scale*sum (pred - target)^2
 * (FP32 device scalar, accumulated atomically: zero it first). */
fgb_status fgb_mlp_mse_grad(fgb_ctx* ctx, long n, const float* pred, const float* target, float scale, void* grad,
                            float* loss);

/* Adam step on FP32 master weights w with FP32 gradient g, moments m, v;
 * refreshes the BF16 copy w_bf16 (may be NULL). */
fgb_status fgb_mlp_adam(fgb_ctx* ctx, long n, float* w, const float* g, float* m, float* v, void* w_bf16, float lr,
                        float beta1, float beta2, float eps, int step);

/* BF16 <-> FP32 conversions. */
fgb_status fgb_mlp_f32_to_bf16(fgb_ctx* ctx, long n, const float* in, void* out);
fgb_status fgb_mlp_bf16_to_f32(fgb_ctx* ctx, long n, const void* in, float* out);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif

#endif /* FGB_MLP_H */
