// bsr_simt.cu — BSR x dense with BF16 operands and FP32 accumulation on the
// CUDA cores.  Correctness baseline and fallback for shapes the tensor-core
// kernel does not take; BSRMat::mul (faust_MatBSR.hpp:827-836) semantics:
// Y(block row r) = sum over the stored blocks (r, c) of B_rc X(block row c).
#include <algorithm>

#include "fgb_internal.cuh"

namespace fgb {

constexpr int BS = 64;   // block size (bm = bn = 64)
constexpr int TN = 64;   // columns of X per CTA

// Grid: x = block rows, y = column tiles of 64.  256 threads, each computing
// a 4 x 4 patch of the 64 x 64 output tile.
__global__ void __launch_bounds__(256)
    k_bsr_simt(const int* __restrict__ browptr, const int* __restrict__ bcolind,
               const __nv_bfloat16* __restrict__ blocks, const __nv_bfloat16* __restrict__ X, int ldx, int ncols,
               __nv_bfloat16* __restrict__ Y, int ldy) {
  __shared__ float sB[BS][BS + 1];  // [row][k]
  __shared__ float sX[BS][TN + 1];  // [k][col]
  const int br = blockIdx.x;
  const int j0 = blockIdx.y * TN;
  const int tr = threadIdx.x / 16, tc = threadIdx.x % 16;  // 16 x 16 threads
  float acc[4][4] = {};
  for (int p = browptr[br]; p < browptr[br + 1]; ++p) {
    const __nv_bfloat16* B = blocks + (size_t)p * BS * BS;  // column-major 64 x 64
    const int bc = bcolind[p];
    for (int e = threadIdx.x; e < BS * BS; e += blockDim.x) {
      const int r = e % BS, k = e / BS;
      sB[r][k] = __bfloat162float(B[e]);
    }
    for (int e = threadIdx.x; e < BS * TN; e += blockDim.x) {
      const int k = e % BS, c = e / BS;
      sX[k][c] = (j0 + c < ncols) ? __bfloat162float(X[(size_t)(bc * BS + k) + (size_t)(j0 + c) * ldx]) : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < BS; ++k) {
      float a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) a[u] = sB[tr + 16 * u][k];
#pragma unroll
      for (int v = 0; v < 4; ++v) b[v] = sX[k][tc + 16 * v];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const int c = j0 + tc + 16 * v;
    if (c >= ncols) continue;
#pragma unroll
    for (int u = 0; u < 4; ++u) Y[(size_t)(br * BS + tr + 16 * u) + (size_t)c * ldy] = __float2bfloat16(acc[u][v]);
  }
}

fgb_status launch_bsr_simt(fgb_ctx* ctx, const DevFactor& f, const __nv_bfloat16* X, int ldx, int ncols,
                           __nv_bfloat16* Y, int ldy) {
  dim3 grid(f.rows / BS, (ncols + TN - 1) / TN);
  k_bsr_simt<<<grid, 256, 0, ctx->stream>>>(f.rowptr, f.colind, (const __nv_bfloat16*)f.val, X, ldx, ncols, Y, ldy);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

}  // namespace fgb

namespace fgb {
fgb_status launch_bsr_tc(fgb_ctx* ctx, const DevFactor& f, const __nv_bfloat16* X, int ldx, int ncols,
                         __nv_bfloat16* Y, int ldy, bool* taken);

// BSR product dispatch: the tcgen05 kernel when it takes the shape, else the
// CUDA-core kernel.
fgb_status launch_bsr_spmm(fgb_ctx* ctx, const DevFactor& f, const __nv_bfloat16* X, int ldx, int ncols,
                           __nv_bfloat16* Y, int ldy) {
  bool taken = false;
  FGB_TRY(launch_bsr_tc(ctx, f, X, ldx, ncols, Y, ldy, &taken));
  if (taken) return FGB_OK;
  return launch_bsr_simt(ctx, f, X, ldx, ncols, Y, ldy);
}
}  // namespace fgb
