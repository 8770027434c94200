// csr.cu — CSR factor kernels: single-factor SpMM (shared-memory staged
// column tiles of X or direct gathers), the fused chain kernel that keeps the
// whole right-to-left product of a column tile on chip, X S^T, device-side
// transposition and dense images.
#include <algorithm>
#include <climits>

#include "csr.cuh"
#include "rowdot.cuh"

namespace fgb {

constexpr int SPMM_THREADS = 512;

// ------------------------------------------------------------------ helpers
template <typename T, int TC>
struct Vec;
template <>
struct Vec<float, 4> {
  using type = float4;
};
template <>
struct Vec<float, 2> {
  using type = float2;
};
template <>
struct Vec<double, 2> {
  using type = double2;
};

// Reads TC consecutive values of a shared-memory row (row-major tile) with
// 16-byte loads where the width allows.
template <typename T, int TC>
__device__ __forceinline__ void load_row(const T* __restrict__ p, T (&x)[TC]) {
  if constexpr (sizeof(T) * TC % 16 == 0) {
    constexpr int W = 16 / sizeof(T);
    using V = typename Vec<T, W>::type;
#pragma unroll
    for (int u = 0; u < TC / W; ++u) {
      V v = reinterpret_cast<const V*>(p)[u];
      if constexpr (W == 4) {
        x[4 * u + 0] = v.x;
        x[4 * u + 1] = v.y;
        x[4 * u + 2] = v.z;
        x[4 * u + 3] = v.w;
      } else {
        x[2 * u + 0] = v.x;
        x[2 * u + 1] = v.y;
      }
    }
  } else {
#pragma unroll
    for (int t = 0; t < TC; ++t) x[t] = p[t];
  }
}

// Copies the column tile X[0:inner, j0:j0+TC) into shared memory as a
// row-major inner x TC tile (zero beyond ncols).  Global reads walk each
// column contiguously.
template <typename T, int TC>
__device__ __forceinline__ void stage_tile(T* __restrict__ tile, const T* __restrict__ X, long ldx, int inner,
                                           int j0, int ncols) {
  for (int t = 0; t < TC; ++t) {
    const bool ok = j0 + t < ncols;
    const T* col = X + (long)(j0 + t) * ldx;
    for (int r = threadIdx.x; r < inner; r += blockDim.x) tile[(long)r * TC + t] = ok ? col[r] : T(0);
  }
}

// ------------------------------------------------------------------ Y = S X
// Grid: x = column tiles of width TC, y = row blocks.  STAGED copies the X
// tile to shared memory first (random column indices then gather from SMEM);
// otherwise entries are gathered from global memory / L2.
template <typename T, int TC, bool STAGED>
__global__ void __launch_bounds__(SPMM_THREADS)
    k_csr_spmm(const int* __restrict__ rowptr, const int* __restrict__ colind, const T* __restrict__ val, int rows,
               int inner, const T* __restrict__ X, int ldx, int ncols, T* __restrict__ Y, int ldy, Epi<T> epi,
               int long_row) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* tile = reinterpret_cast<T*>(smem_raw);
  const int j0 = blockIdx.x * TC;
  const T s = epi.scal ? *epi.scal : T(0);
  int first = blockIdx.y * blockDim.x + threadIdx.x;  // first row of the generic loop below
  if (STAGED) {
    // (one row block) The thread's first two rows and their first SP_PF
    // entries are read before the tile is staged, so those L2 round trips
    // overlap the staging.  The tile is only needed by rows this kernel
    // computes (1 .. long_row-1 entries); factors whose entries all sit in
    // long rows skip it.
    const int i0 = threadIdx.x, i1 = threadIdx.x + blockDim.x;
    int b0 = 0, e0 = 0, b1 = 0, e1 = 0;
    if (i0 < rows) b0 = rowptr[i0], e0 = rowptr[i0 + 1];
    if (i1 < rows) b1 = rowptr[i1], e1 = rowptr[i1 + 1];
    if (e0 - b0 >= long_row) e0 = b0 = 0;  // a long row: written by the long-row kernel
    if (e1 - b1 >= long_row) e1 = b1 = 0;
    int need = e0 > b0 || e1 > b1;
    for (int r = i1 + blockDim.x; r < rows; r += blockDim.x) {
      const int L = rowptr[r + 1] - rowptr[r];
      need |= (L > 0 && L < long_row);
    }
    constexpr int SP_PF = 4;
    int c0[SP_PF], c1[SP_PF];
    T v0[SP_PF], v1[SP_PF];
#pragma unroll
    for (int u = 0; u < SP_PF; ++u) {
      c0[u] = b0 + u < e0 ? colind[b0 + u] : 0;
      v0[u] = b0 + u < e0 ? val[b0 + u] : T(0);
      c1[u] = b1 + u < e1 ? colind[b1 + u] : 0;
      v1[u] = b1 + u < e1 ? val[b1 + u] : T(0);
    }
    if (__syncthreads_or(need)) {
      stage_tile<T, TC>(tile, X, ldx, inner, j0, ncols);
      __syncthreads();
    }
    auto row = [&](int i, int b, int e, const int (&c)[SP_PF], const T (&v)[SP_PF]) {
      T acc[TC];
#pragma unroll
      for (int t = 0; t < TC; ++t) acc[t] = T(0);
#pragma unroll
      for (int u = 0; u < SP_PF; ++u)
        if (b + u < e) {
          T x[TC];
          load_row<T, TC>(tile + (long)c[u] * TC, x);
#pragma unroll
          for (int t = 0; t < TC; ++t) acc[t] = fmad(v[u], x[t], acc[t]);
        }
      for (int p = b + SP_PF; p < e; ++p) {
        const T vp = val[p];
        T x[TC];
        load_row<T, TC>(tile + (long)colind[p] * TC, x);
#pragma unroll
        for (int t = 0; t < TC; ++t) acc[t] = fmad(vp, x[t], acc[t]);
      }
#pragma unroll
      for (int t = 0; t < TC; ++t)
        if (j0 + t < ncols) Y[i + (long)(j0 + t) * ldy] = epi_apply(epi, acc[t], i, j0 + t, s);
    };
    // rows without entries still write their zeros (and epilogue)
    if (i0 < rows && rowptr[i0 + 1] - rowptr[i0] < long_row) row(i0, b0, e0, c0, v0);
    if (i1 < rows && rowptr[i1 + 1] - rowptr[i1] < long_row) row(i1, b1, e1, c1, v1);
    first = i1 + blockDim.x;
  }
  for (int i = first; i < rows; i += gridDim.y * blockDim.x) {
    T acc[TC];
#pragma unroll
    for (int t = 0; t < TC; ++t) acc[t] = T(0);
    const int p0 = rowptr[i], p1 = rowptr[i + 1];
    if (p1 - p0 >= long_row) continue;  // k_csr_spmm_long writes this row (chunked order)
    for (int p = p0; p < p1; ++p) {
      const T v = val[p];
      const int c = colind[p];
      T x[TC];
      if (STAGED) {
        load_row<T, TC>(tile + (long)c * TC, x);
      } else {
#pragma unroll
        for (int t = 0; t < TC; ++t) x[t] = (j0 + t < ncols) ? X[c + (long)(j0 + t) * ldx] : T(0);
      }
#pragma unroll
      for (int t = 0; t < TC; ++t) acc[t] = fmad(v, x[t], acc[t]);
    }
#pragma unroll
    for (int t = 0; t < TC; ++t)
      if (j0 + t < ncols) Y[i + (long)(j0 + t) * ldy] = epi_apply(epi, acc[t], i, j0 + t, s);
  }
}

// Rows of more than ROW_CHUNK entries: one block of 8 warps per (row, 32
// columns), lanes along the columns, the row's chunk groups split over the
// warps (rowdot.cuh), so every FP64 FMA instruction has 32 active lanes and
// a row of L entries takes about L / 8 dependent steps instead of L.
// The long rows among rows y, y + ny, y + 2 ny, ... (up to 256 per pass,
// found by all threads at once) into a shared list; returns their number.
__device__ __forceinline__ int long_rows_scan(const int* __restrict__ rowptr, int rows, int i0, int stride, int* list,
                                              int* cnt) {
  if (threadIdx.x == 0) *cnt = 0;
  __syncthreads();
  const int i = i0 + (int)threadIdx.x * stride;
  if (i < rows && rowptr[i + 1] - rowptr[i] > ROW_CHUNK) list[atomicAdd(cnt, 1)] = i;
  __syncthreads();
  return *cnt;
}

// d_max: the longest row on the device (null or negative: unknown); a factor
// without long rows ends the kernel at once.
__device__ __forceinline__ bool no_long_rows(const int* d_max) {
  if (!d_max) return false;
  const int m = __ldg(d_max);
  return m >= 0 && m <= ROW_CHUNK;
}

template <typename T>
__global__ void __launch_bounds__(256)
    k_csr_spmm_long(const int* __restrict__ rowptr, const int* __restrict__ colind, const T* __restrict__ val,
                    int rows, const T* __restrict__ X, int ldx, int ncols, T* __restrict__ Y, int ldy, Epi<T> epi,
                    const int* __restrict__ d_max) {
  if (no_long_rows(d_max)) return;
  __shared__ T roots[ROW_GROUPS * 32];
  __shared__ int list[256], cnt;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long j = (long)blockIdx.x * 32 + lane;
  const bool okj = j < ncols;
  const T* __restrict__ xcol = X + (okj ? j : 0) * (long)ldx;
  // rows y + gridDim.y * t, 256 of them per pass
  for (int i0 = blockIdx.y; i0 < rows; i0 += gridDim.y * 256) {
    const int nl = long_rows_scan(rowptr, rows, i0, gridDim.y, list, &cnt);
    for (int q = 0; q < nl; ++q) {
      const int i = list[q];
      const T v = row_block_long<T, 8>(val, colind, rowptr[i], rowptr[i + 1], [&](int c) { return __ldg(xcol + c); },
                                       roots, lane, warp);
      if (warp == 0 && okj) Y[i + j * (long)ldy] = epi_apply(epi, v, i, j, epi.scal ? *epi.scal : T(0));
    }
    __syncthreads();
  }
}

// X S^T for rows c of S with more than ROW_CHUNK entries: lanes along the rows
// of X, the row's chunk groups split over 8 warps.
template <typename T>
__global__ void __launch_bounds__(256)
    k_dense_csrT_long(const T* __restrict__ X, int ldx, int xrows, const int* __restrict__ rowptr,
                      const int* __restrict__ colind, const T* __restrict__ val, int srows, T* __restrict__ Y, int ldy,
                      Epi<T> epi, const int* __restrict__ d_max) {
  if (no_long_rows(d_max)) return;
  __shared__ T roots[ROW_GROUPS * 32];
  __shared__ int list[256], cnt;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int r = blockIdx.x * 32 + lane;
  const bool okr = r < xrows;
  const T* __restrict__ xr = X + (okr ? r : 0);
  for (int c0 = blockIdx.y; c0 < srows; c0 += gridDim.y * 256) {
    const int nl = long_rows_scan(rowptr, srows, c0, gridDim.y, list, &cnt);
    for (int q = 0; q < nl; ++q) {
      const int c = list[q];
      const T v = row_block_long<T, 8>(val, colind, rowptr[c], rowptr[c + 1],
                                       [&](int k) { return __ldg(xr + (long)k * ldx); }, roots, lane, warp);
      if (warp == 0 && okr) Y[r + (long)c * ldy] = epi_apply(epi, v, r, c, epi.scal ? *epi.scal : T(0));
    }
    __syncthreads();
  }
}

template <typename T, int TC, bool STAGED>
static fgb_status launch_spmm_tc(fgb_ctx* ctx, const int* rowptr, const int* colind, const T* val, int rows,
                                 int inner, const T* X, int ldx, int ncols, T* Y, int ldy, const Epi<T>& epi,
                                 int long_row) {
  const int tiles = (ncols + TC - 1) / TC;
  size_t smem = STAGED ? (size_t)inner * TC * sizeof(T) : 0;
  int rblocks = 1;
  if (!STAGED) {
    // Enough blocks to cover the SMs several times.
    long want = 4L * ctx->sm_count;
    rblocks = (int)std::max(1L, std::min((long)((rows + SPMM_THREADS - 1) / SPMM_THREADS), want / std::max(1, tiles)));
  }
  auto kern = k_csr_spmm<T, TC, STAGED>;
  FGB_TRY(smem_opt_in(ctx, (const void*)kern, smem));
  dim3 grid(tiles, rblocks);
  kern<<<grid, SPMM_THREADS, smem, ctx->stream>>>(rowptr, colind, val, rows, inner, X, ldx, ncols, Y, ldy, epi,
                                                   long_row);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

// The long-row kernel of a product runs on the context's side stream beside
// the short-row kernel (they write disjoint rows of Y): fork before it, join
// after the short-row launch.  In a captured graph the two become parallel
// nodes.
static fgb_status long_fork(fgb_ctx* ctx, cudaStream_t* s) {
  *s = ctx->stream;
  if (!ctx->s_long) return FGB_OK;
  FGB_CUDA(ctx, cudaEventRecord(ctx->ev_long_fork, ctx->stream));
  FGB_CUDA(ctx, cudaStreamWaitEvent(ctx->s_long, ctx->ev_long_fork, 0));
  *s = ctx->s_long;
  return FGB_OK;
}
static fgb_status long_join(fgb_ctx* ctx) {
  if (!ctx->s_long) return FGB_OK;
  FGB_CUDA(ctx, cudaEventRecord(ctx->ev_long_join, ctx->s_long));
  FGB_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_long_join, 0));
  return FGB_OK;
}

template <typename T>
fgb_status launch_csr_spmm(fgb_ctx* ctx, const int* rowptr, const int* colind, const T* val, int rows, int inner,
                           const T* X, int ldx, int ncols, T* Y, int ldy, const Epi<T>& epi, int max_row,
                           const int* d_max_row) {
  if (rows == 0 || ncols == 0) return FGB_OK;
  constexpr int TC = 16 / sizeof(T) * 2;  // 8 floats or 4 doubles per thread
  const size_t staged = (size_t)inner * TC * sizeof(T);
  const long tiles = (ncols + TC - 1) / TC;
  // rows of more than ROW_CHUNK entries (known absent when max_row is) go to
  // their own kernel
  const bool has_long = max_row < 0 || max_row > ROW_CHUNK;
  const int long_row = has_long ? ROW_CHUNK + 1 : INT_MAX;
  if (has_long) {
    cudaStream_t s;
    FGB_TRY(long_fork(ctx, &s));
    dim3 g((unsigned)((ncols + 31) / 32), (unsigned)std::min((rows + 255) / 256 * 4, 16));
    k_csr_spmm_long<T><<<g, 256, 0, s>>>(rowptr, colind, val, rows, X, ldx, ncols, Y, ldy, epi, d_max_row);
    FGB_LAUNCHED(ctx);
  }
  // Stage when the tile fits comfortably and there are enough tiles to fill
  // the GPU; small problems (PALM blocks) gather straight from L2.
  if (staged <= 96 * 1024 && tiles >= ctx->sm_count)
    FGB_TRY((launch_spmm_tc<T, TC, true>(ctx, rowptr, colind, val, rows, inner, X, ldx, ncols, Y, ldy, epi,
                                         long_row)));
  // Half-width tiles when a full one does not fit (e.g. 4096 FP32 rows): the
  // gathers still come from shared memory instead of dependent L2 round trips.
  else if (staged / 2 <= 96 * 1024 && 2 * tiles >= 4L * ctx->sm_count)
    FGB_TRY((launch_spmm_tc<T, TC / 2, true>(ctx, rowptr, colind, val, rows, inner, X, ldx, ncols, Y, ldy, epi,
                                             long_row)));
  else
    FGB_TRY((launch_spmm_tc<T, TC / 2, false>(ctx, rowptr, colind, val, rows, inner, X, ldx, ncols, Y, ldy, epi,
                                              long_row)));
  return has_long ? long_join(ctx) : FGB_OK;
}

// ------------------------------------------------------------------ Y = X S^T
// Grid: x = output columns (rows of S), y = row blocks of X.  Each output
// column c combines the columns of X named by row c of S.
template <typename T>
__global__ void __launch_bounds__(SPMM_THREADS)
    k_dense_csrT(const T* __restrict__ X, int ldx, int xrows, const int* __restrict__ rowptr,
                 const int* __restrict__ colind, const T* __restrict__ val, int srows, T* __restrict__ Y, int ldy,
                 Epi<T> epi) {
  const int c = blockIdx.x;
  const int p0 = rowptr[c], p1 = rowptr[c + 1];
  const T s = epi.scal ? *epi.scal : T(0);
  if (p1 - p0 > ROW_CHUNK) return;  // k_dense_csrT_long writes this column (chunked order)
  for (int r = blockIdx.y * blockDim.x + threadIdx.x; r < xrows; r += gridDim.y * blockDim.x) {
    T acc = T(0);
    for (int p = p0; p < p1; ++p) acc = fmad(__ldg(val + p), __ldg(X + r + (long)__ldg(colind + p) * ldx), acc);
    Y[r + (long)c * ldy] = epi_apply(epi, acc, r, c, s);
  }
}

template <typename T>
fgb_status launch_dense_csrT(fgb_ctx* ctx, const T* X, int ldx, int xrows, const int* rowptr, const int* colind,
                             const T* val, int srows, int scols, T* Y, int ldy, const Epi<T>& epi, int max_row,
                             const int* d_max_row) {
  (void)scols;
  if (srows == 0 || xrows == 0) return FGB_OK;
  const bool has_long = max_row < 0 || max_row > ROW_CHUNK;
  if (has_long) {
    cudaStream_t s;
    FGB_TRY(long_fork(ctx, &s));
    dim3 g((unsigned)((xrows + 31) / 32), (unsigned)std::min((srows + 255) / 256 * 4, 16));
    k_dense_csrT_long<T><<<g, 256, 0, s>>>(X, ldx, xrows, rowptr, colind, val, srows, Y, ldy, epi, d_max_row);
    FGB_LAUNCHED(ctx);
  }
  // rows of at most ROW_CHUNK entries: one block per output column
  int rblocks = std::max(1, std::min((xrows + SPMM_THREADS - 1) / SPMM_THREADS, 8));
  dim3 grid(srows, rblocks);
  k_dense_csrT<T><<<grid, SPMM_THREADS, 0, ctx->stream>>>(X, ldx, xrows, rowptr, colind, val, srows, Y, ldy, epi);
  FGB_LAUNCHED(ctx);
  return has_long ? long_join(ctx) : FGB_OK;
}

// ------------------------------------------------------------------ fused chain
// One block owns the column tile X[:, j0:j0+TC) and applies every factor in
// turn, right to left, with the intermediate tile kept in shared memory
// (two buffers of maxdim x TC).  Only X is read from HBM and only Y written;
// the factors are read from L2 by every block.
constexpr int CHAIN_THREADS = 1024;
constexpr int CHAIN_ILP = 4;

template <typename T, int TC>
__device__ __forceinline__ void chain_row(const ChainDesc& d, const T* __restrict__ val, const T* __restrict__ in,
                                          int i, T (&acc)[TC]) {
#pragma unroll
  for (int t = 0; t < TC; ++t) acc[t] = T(0);
  const int p1 = __ldg(d.rowptr + i + 1);
  for (int p = __ldg(d.rowptr + i); p < p1; ++p) {
    const T v = __ldg(val + p);
    T x[TC];
    load_row<T, TC>(in + (long)__ldg(d.colind + p) * TC, x);
#pragma unroll
    for (int t = 0; t < TC; ++t) acc[t] = fmad(v, x[t], acc[t]);
  }
}

template <typename T, int TC>
__global__ void __launch_bounds__(CHAIN_THREADS)
    k_csr_chain_fused(const ChainDesc* __restrict__ desc, int nfac, const T* __restrict__ X, int ldx, int ncols,
                      T* __restrict__ Y, int ldy, int maxdim) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* bufA = reinterpret_cast<T*>(smem_raw);
  T* bufB = bufA + (long)maxdim * TC;
  const int j0 = blockIdx.x * TC;
  stage_tile<T, TC>(bufA, X, ldx, desc[nfac - 1].cols, j0, ncols);
  __syncthreads();
  T* in = bufA;
  T* out = bufB;
  for (int f = nfac - 1; f >= 0; --f) {
    const ChainDesc d = desc[f];
    const T* __restrict__ val = reinterpret_cast<const T*>(d.val);
    const bool last = (f == 0);
    // CHAIN_ILP rows per pass: their rowptr / entry loads are issued
    // together, so each thread keeps several L2 requests in flight
    for (int i0 = threadIdx.x; i0 < d.rows; i0 += CHAIN_ILP * blockDim.x) {
      int rb[CHAIN_ILP], re[CHAIN_ILP];
#pragma unroll
      for (int u = 0; u < CHAIN_ILP; ++u) {
        const int i = i0 + u * blockDim.x;
        rb[u] = i < d.rows ? __ldg(d.rowptr + i) : 0;
        re[u] = i < d.rows ? __ldg(d.rowptr + i + 1) : 0;
      }
      T acc[CHAIN_ILP][TC];
#pragma unroll
      for (int u = 0; u < CHAIN_ILP; ++u)
#pragma unroll
        for (int t = 0; t < TC; ++t) acc[u][t] = T(0);
      int maxlen = 0;
#pragma unroll
      for (int u = 0; u < CHAIN_ILP; ++u) maxlen = max(maxlen, re[u] - rb[u]);
      for (int q = 0; q < maxlen; ++q) {
        T v[CHAIN_ILP];
        int c[CHAIN_ILP];
#pragma unroll
        for (int u = 0; u < CHAIN_ILP; ++u) {
          const bool ok = rb[u] + q < re[u];
          v[u] = ok ? __ldg(val + rb[u] + q) : T(0);
          c[u] = ok ? __ldg(d.colind + rb[u] + q) : -1;
        }
#pragma unroll
        for (int u = 0; u < CHAIN_ILP; ++u) {
          if (c[u] >= 0) {
            T x[TC];
            load_row<T, TC>(in + (long)c[u] * TC, x);
#pragma unroll
            for (int t = 0; t < TC; ++t) acc[u][t] = fmad(v[u], x[t], acc[u][t]);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < CHAIN_ILP; ++u) {
        const int i = i0 + u * blockDim.x;
        if (i >= d.rows) continue;
        if (last) {
#pragma unroll
          for (int t = 0; t < TC; ++t)
            if (j0 + t < ncols) Y[i + (long)(j0 + t) * ldy] = acc[u][t];
        } else {
#pragma unroll
          for (int t = 0; t < TC; ++t) out[(long)i * TC + t] = acc[u][t];
        }
      }
    }
    __syncthreads();
    T* tmp = in;
    in = out;
    out = tmp;
  }
}

template <typename T, int TC>
static fgb_status launch_chain_tc(fgb_ctx* ctx, const ChainDesc* d_desc, int nfac, const T* X, int ldx, int ncols,
                                  T* Y, int ldy, int maxdim) {
  const size_t smem = 2 * (size_t)maxdim * TC * sizeof(T);
  auto kern = k_csr_chain_fused<T, TC>;
  FGB_TRY(smem_opt_in(ctx, (const void*)kern, smem));
  const int tiles = (ncols + TC - 1) / TC;
  kern<<<tiles, CHAIN_THREADS, smem, ctx->stream>>>(d_desc, nfac, X, ldx, ncols, Y, ldy, maxdim);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

// Picks the tile width: the widest that fits shared memory while still giving
// at least one block per SM; returns 0 when no width fits.
template <typename T>
static int chain_tile_width(fgb_ctx* ctx, int maxdim, int ncols) {
  const size_t cap = std::min<size_t>(ctx->smem_optin ? ctx->smem_optin : 227 * 1024, 200 * 1024);
  const int widths[] = {8, 4, 2};
  int best = 0;
  for (int w : widths) {
    if (sizeof(T) * w < 8) continue;  // keep 8-byte rows at least
    if (2 * (size_t)maxdim * w * sizeof(T) > cap) continue;
    if (!best) best = w;
    if ((ncols + w - 1) / w >= ctx->sm_count) return w;
    best = w;
  }
  return best;
}

fgb_status chain_fused(fgb_ctx* ctx, fgb_dtype dt, const ChainDesc* d_desc, int nfac, const void* X, int ldx,
                       int ncols, void* Y, int ldy, int maxdim, bool probe_only, bool* fits) {
  int w = (dt == FGB_F64) ? chain_tile_width<double>(ctx, maxdim, ncols)
                          : (dt == FGB_F32 ? chain_tile_width<float>(ctx, maxdim, ncols) : 0);
  if (fits) *fits = (w != 0);
  if (probe_only || w == 0) return w ? FGB_OK : FGB_ERR_NOT_SUPPORTED;
  if (dt == FGB_F64) {
    const double* x = (const double*)X;
    double* y = (double*)Y;
    if (w == 8) return launch_chain_tc<double, 8>(ctx, d_desc, nfac, x, ldx, ncols, y, ldy, maxdim);
    if (w == 4) return launch_chain_tc<double, 4>(ctx, d_desc, nfac, x, ldx, ncols, y, ldy, maxdim);
    return launch_chain_tc<double, 2>(ctx, d_desc, nfac, x, ldx, ncols, y, ldy, maxdim);
  }
  const float* x = (const float*)X;
  float* y = (float*)Y;
  if (w == 8) return launch_chain_tc<float, 8>(ctx, d_desc, nfac, x, ldx, ncols, y, ldy, maxdim);
  if (w == 4) return launch_chain_tc<float, 4>(ctx, d_desc, nfac, x, ldx, ncols, y, ldy, maxdim);
  return launch_chain_tc<float, 2>(ctx, d_desc, nfac, x, ldx, ncols, y, ldy, maxdim);
}

// ------------------------------------------------------------------ transpose
// Single-block CSR transpose whose transposed rows list entries in increasing
// original row: a column histogram, a block scan, then an ordered scatter by
// one warp (ranks inside each 32-entry batch come from __match_any_sync).
template <typename T>
__global__ void __launch_bounds__(1024)
    k_csr_transpose(const int* __restrict__ rowptr, const int* __restrict__ colind, const T* __restrict__ val,
                    int rows, int cols, int* __restrict__ t_rowptr, int* __restrict__ t_colind,
                    T* __restrict__ t_val, int* __restrict__ cursor) {
  const int nnz = rowptr[rows];
  for (int c = threadIdx.x; c <= cols; c += blockDim.x) cursor[c] = 0;
  __syncthreads();
  for (int p = threadIdx.x; p < nnz; p += blockDim.x) atomicAdd(&cursor[colind[p] + 1], 1);
  __syncthreads();
  // Inclusive scan of cursor[1..cols] by thread 0 in chunks (cols is small
  // for PALM factors); t_rowptr = exclusive offsets.
  if (threadIdx.x == 0) {
    int run = 0;
    t_rowptr[0] = 0;
    for (int c = 0; c < cols; ++c) {
      run += cursor[c + 1];
      t_rowptr[c + 1] = run;
    }
  }
  __syncthreads();
  for (int c = threadIdx.x; c < cols; c += blockDim.x) cursor[c] = t_rowptr[c];
  __syncthreads();
  if (threadIdx.x < 32) {
    const unsigned lane = threadIdx.x;
    for (int base = 0; base < nnz; base += 32) {
      const int p = base + (int)lane;
      const bool ok = p < nnz;
      int r = 0;
      if (ok) {
        // row of entry p: last row whose rowptr is <= p
        int lo = 0, hi = rows - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (rowptr[mid] <= p) lo = mid; else hi = mid - 1;
        }
        r = lo;
      }
      const int c = ok ? colind[p] : -1 - (int)lane;
      const unsigned same = __match_any_sync(0xffffffffu, c);
      const int rank = __popc(same & ((1u << lane) - 1u));
      int slot = 0;
      if (ok) slot = cursor[c] + rank;
      __syncwarp();
      if (ok) {
        t_colind[slot] = r;
        t_val[slot] = val[p];
        // the highest lane of each column group advances the cursor
        if ((same >> lane) == 1u) cursor[c] = slot + 1;
      }
      __syncwarp();
    }
  }
}

fgb_status csr_build_transpose(fgb_ctx* ctx, fgb_dtype dt, DevFactor& f) {
  if (f.format != FGB_CSR) return fail(ctx, FGB_ERR_INVALID_ARG, "transpose: CSR factors only");
  const size_t es = dtype_size(dt);
  if (!f.t_rowptr) FGB_TRY(dmalloc(ctx, (void**)&f.t_rowptr, sizeof(int) * (f.cols + 1)));
  if (!f.t_colind) FGB_TRY(dmalloc(ctx, (void**)&f.t_colind, sizeof(int) * std::max(1, f.cap)));
  if (!f.t_val) FGB_TRY(dmalloc(ctx, &f.t_val, es * std::max(1, f.cap)));
  int* cursor = nullptr;
  FGB_TRY(dmalloc(ctx, (void**)&cursor, sizeof(int) * (f.cols + 2)));
  if (dt == FGB_F64)
    k_csr_transpose<double><<<1, 1024, 0, ctx->stream>>>(f.rowptr, f.colind, (const double*)f.val, f.rows, f.cols,
                                                         f.t_rowptr, f.t_colind, (double*)f.t_val, cursor);
  else
    k_csr_transpose<float><<<1, 1024, 0, ctx->stream>>>(f.rowptr, f.colind, (const float*)f.val, f.rows, f.cols,
                                                        f.t_rowptr, f.t_colind, (float*)f.t_val, cursor);
  ctx->launches.fetch_add(1);
  cudaError_t e = cudaGetLastError();
  cudaStreamSynchronize(ctx->stream);
  dfree(cursor);
  if (e != cudaSuccess) return cuda_check(ctx, e, "csr transpose");
  f.has_t = true;
  return FGB_OK;
}

// ------------------------------------------------------------------ dense image
template <typename T>
__global__ void k_csr_to_dense(const int* __restrict__ rowptr, const int* __restrict__ colind,
                               const T* __restrict__ val, int rows, int cols, T* __restrict__ out) {
  const long n = (long)rows * cols;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) out[i] = T(0);
}
template <typename T>
__global__ void k_csr_scatter(const int* __restrict__ rowptr, const int* __restrict__ colind,
                              const T* __restrict__ val, int rows, T* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += gridDim.x * blockDim.x)
    for (int p = rowptr[i]; p < rowptr[i + 1]; ++p) out[i + (long)colind[p] * rows] = val[p];
}

template <typename T>
fgb_status launch_csr_to_dense(fgb_ctx* ctx, const DevFactor& f, T* out) {
  const int g = 2 * ctx->sm_count;
  k_csr_to_dense<T><<<g, 256, 0, ctx->stream>>>(f.rowptr, f.colind, (const T*)f.val, f.rows, f.cols, out);
  FGB_LAUNCHED(ctx);
  k_csr_scatter<T><<<std::max(1, std::min(g, (f.rows + 255) / 256)), 256, 0, ctx->stream>>>(
      f.rowptr, f.colind, (const T*)f.val, f.rows, out);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

template fgb_status launch_csr_spmm<float>(fgb_ctx*, const int*, const int*, const float*, int, int, const float*, int,
                                           int, float*, int, const Epi<float>&, int, const int*);
template fgb_status launch_csr_spmm<double>(fgb_ctx*, const int*, const int*, const double*, int, int, const double*,
                                            int, int, double*, int, const Epi<double>&, int, const int*);
template fgb_status launch_dense_csrT<float>(fgb_ctx*, const float*, int, int, const int*, const int*, const float*,
                                             int, int, float*, int, const Epi<float>&, int, const int*);
template fgb_status launch_dense_csrT<double>(fgb_ctx*, const double*, int, int, const int*, const int*,
                                              const double*, int, int, double*, int, const Epi<double>&, int,
                                              const int*);
template fgb_status launch_csr_to_dense<float>(fgb_ctx*, const DevFactor&, float*);
template fgb_status launch_csr_to_dense<double>(fgb_ctx*, const DevFactor&, double*);

}  // namespace fgb
