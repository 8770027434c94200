// product.cu — the dense product of a Faust (TransformHelper::get_product,
// src/faust_linear_operator/CPU/faust_TransformHelper.hpp:1132-1178) and the
// DYNPROG product order (dynprog_multiply, src/faust_linear_operator/
// faust_prod_opt_gen.hpp:1-202, cost model CPU/faust_prod_opt.cpp:1-80).
//
// Orders:
//   DEFAULT_L2R  Transform::get_product (CPU/faust_Transform.hpp:598-656):
//                dense(S[J-1]) first, then S[i] * M for i = J-2 .. 0
//                (op T/H: dense(S[0]^T), then S[i]^T * M for i = 1 .. J-1).
//   DYNPROG      the split points of the reference's dynamic program over
//                its integer cost model, evaluated bottom-up.
//
// Every pairwise product keeps the canonical entry order of the rest of the
// library (a sequential fused multiply-add from +0 over the sparse operand's
// stored entries, or over k ascending for dense x dense), so the oracle's
// restatement gives identical bits.  The split search is host code (a few
// hundred integer operations); the products are device kernels on ctx->stream:
//   sparse x sparse  csr_spmm(op(A), dense image of op(B))
//   sparse x dense   csr_spmm(op(A), D)
//   dense x sparse   dense_csrT(D, CSR of op(B)^T)
//   dense x dense    k_gemm_seq below
#include <climits>
#include <cstdint>
#include <vector>

#include "csr.cuh"
#include "fgb_internal.cuh"

namespace fgb {

// ------------------------------------------------------------------ cost model
// The reference evaluates its costs in C int; products that leave the 32-bit
// range wrap (two's complement), which this restatement makes explicit.
static inline int w32(int64_t v) { return (int)(int32_t)(uint32_t)(uint64_t)v; }
static inline int mul32(int a, int b) { return w32((int64_t)a * (int64_t)b); }
static inline int div32(int a, int b) { return b == 0 ? 0 : (int)((int64_t)a / (int64_t)b); }

static int cost_sparse_dense(int a_nnz, int b_nrows, int b_ncols, bool b_transp) {
  return mul32(a_nnz, b_transp ? b_nrows : b_ncols);
}
static int cost_sparse_sparse(int a_nrows, int a_ncols, int a_nnz, bool a_transp, int b_nnz) {
  return div32(mul32(a_nnz, b_nnz), a_transp ? a_ncols : a_nrows);
}
static int cost_dense_dense(int a_nrows, int a_ncols, int b_nrows, int b_ncols, bool b_transp) {
  return mul32(mul32(a_nrows, a_ncols), b_transp ? b_nrows : b_ncols);
}
static int cost_dense_sparse(int a_nrows, int a_ncols, bool a_transp, int b_nnz) {
  return mul32(a_transp ? a_ncols : a_nrows, b_nnz);
}

// Split table of dynprog_multiply (faust_prod_opt_gen.hpp:113-190): split[i*n+j]
// = k for i < j (the product of leaves i..j is (i..k)(k+1..j)), -1 elsewhere.
// Leaf dimensions are the stored ones (before op), as in the reference.
static void dynprog_splits(int n, const int* rows, const int* cols, const int* nnz, const int* dense, char op,
                           std::vector<int>& split) {
  std::vector<int> c((size_t)n * n, 0);
  split.assign((size_t)n * n, -1);
  const bool tr = op != 'N';
  for (int p = 1; p < n; ++p)
    for (int i = 0; i < n - p; ++i) {
      const int j = p + i;
      int best = INT_MAX;
      for (int k = i; k < j; ++k) {
        const bool rf_init = k + 1 == j;
        int cost = w32((int64_t)c[(size_t)i * n + k] + c[(size_t)(k + 1) * n + j]);
        const int mf_ncols = cols[k];
        int add = 0;
        if (dense[i] && dense[j])
          add = cost_dense_dense(rows[i], mf_ncols, rows[j], cols[j], tr && rf_init);
        else if (dense[i])
          add = cost_dense_sparse(rows[i], mf_ncols, tr && k == i, nnz[j]);
        else if (dense[j])
          add = cost_sparse_dense(nnz[i], rows[j], cols[j], tr && rf_init);
        else
          add = cost_sparse_sparse(rows[i], cols[i], nnz[i], tr, nnz[j]);
        cost = w32((int64_t)cost + add);
        if (cost < best) {
          best = cost;
          split[(size_t)i * n + j] = k;
        }
      }
      // every candidate at INT_MAX leaves the reference's split unset
      // (uninitialised); the first candidate is taken here
      if (split[(size_t)i * n + j] < 0) split[(size_t)i * n + j] = i;
      c[(size_t)i * n + j] = best;
    }
}

// ------------------------------------------------------------------ dense x dense
// C = A B (column-major), c(r,q) = sequential fma over k = 0..K-1 from +0.
// 64 x 64 output tile per block, 256 threads with 4 x 4 entries each
// (rows tx + 16 i, columns ty + 16 j), K staged 16 at a time in shared memory.
// Tiles past K are not multiplied (an fma with a zero would turn -0 into +0).
constexpr int GS_T = 64, GS_K = 16;

template <typename T>
__global__ void __launch_bounds__(256) k_gemm_seq(const T* __restrict__ A, int lda, const T* __restrict__ B, int ldb,
                                                  T* __restrict__ C, int ldc, int M, int N, int K) {
  __shared__ T As[GS_K][GS_T + 1];
  __shared__ T Bs[GS_K][GS_T + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const long m0 = (long)blockIdx.x * GS_T, n0 = (long)blockIdx.y * GS_T;
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
  for (int k0 = 0; k0 < K; k0 += GS_K) {
    const int kn = min(GS_K, K - k0);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int idx = tid + 256 * e;  // 0..1023
      const int m = idx & 63, kk = idx >> 6;  // A tile: m fastest (column-major A)
      const long gm = m0 + m;
      As[kk][m] = (kk < kn && gm < M) ? A[gm + (long)(k0 + kk) * lda] : T(0);
      const int kb = idx & 15, q = idx >> 4;  // B tile: k fastest (column-major B)
      const long gq = n0 + q;
      Bs[kb][q] = (kb < kn && gq < N) ? B[(long)(k0 + kb) + gq * ldb] : T(0);
    }
    __syncthreads();
    for (int kk = 0; kk < kn; ++kk) {
      T a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmad(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const long q = n0 + ty + 16 * j;
    if (q >= N) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const long r = m0 + tx + 16 * i;
      if (r < M) C[r + q * (long)ldc] = acc[i][j];
    }
  }
}

template <typename T>
static fgb_status launch_gemm_seq(fgb_ctx* ctx, const T* A, int lda, const T* B, int ldb, T* C, int ldc, int M, int N,
                                  int K) {
  if (M == 0 || N == 0) return FGB_OK;
  dim3 grid((M + GS_T - 1) / GS_T, (N + GS_T - 1) / GS_T);
  k_gemm_seq<T><<<grid, 256, 0, ctx->stream>>>(A, lda, B, ldb, C, ldc, M, N, K);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

// Column-major zero fill of a rows x cols region with leading dimension ld.
template <typename T>
__global__ void k_zero2d(T* Y, int ld, int rows, int cols) {
  const long n = (long)rows * cols;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
    Y[(e % rows) + (e / rows) * (long)ld] = T(0);
}

// ------------------------------------------------------------------ plan
// A node of the product tree: a leaf (CSR factor or the dense operand) or a
// dense intermediate (column-major, ld = rows) in the workspace or in Y.
struct PNode {
  int leaf = -1;          // leaf index, or -1 for a computed product
  const DevFactor* f = nullptr;
  const void* D = nullptr;  // dense data (dense leaf or intermediate)
  int ld = 0;
  int rows = 0, cols = 0;   // stored dimensions (before op)
};

struct CsrView {
  const int* rp;
  const int* ci;
  const void* v;
  int rows, cols;
};

static CsrView csr_op(const DevFactor& f, char op) {
  if (op == 'N') return {f.rowptr, f.colind, f.val, f.rows, f.cols};
  return {f.t_rowptr, f.t_colind, f.t_val, f.cols, f.rows};
}

template <typename T>
struct ProductRun {
  fgb_ctx* ctx;
  std::vector<PNode> leaves;
  std::vector<int> split;
  int n = 0;
  char op = 'N', last_op = 'N';
  T* ws = nullptr;     // workspace cursor
  T* Y = nullptr;      // destination of the root product
  int ldy = 0;

  T* take(size_t elems) {
    T* p = ws;
    ws += (elems + 31) & ~size_t(31);  // 256-byte multiples for FP64
    return p;
  }

  // out = op_l(L) * op_r(R) written to dst (ld ldd).
  fgb_status gemm(const PNode& L, char opl, const PNode& R, char opr, T* dst, int ldd) {
    const Epi<T> epi;
    const int lrows = opl == 'N' ? L.rows : L.cols, inner = opl == 'N' ? L.cols : L.rows;
    const int rcols = opr == 'N' ? R.cols : R.rows;
    if (L.f) {
      const CsrView a = csr_op(*L.f, opl);
      const T* Dr = nullptr;
      int ldr = 0;
      if (R.f) {
        // dense image of op_r(R)
        DevFactor img = *R.f;
        if (opr != 'N') {
          img.rowptr = R.f->t_rowptr;
          img.colind = R.f->t_colind;
          img.val = R.f->t_val;
          img.rows = R.f->cols;
          img.cols = R.f->rows;
        }
        T* tmp = take((size_t)img.rows * img.cols);
        FGB_TRY(launch_csr_to_dense<T>(ctx, img, tmp));
        Dr = tmp;
        ldr = img.rows;
      } else {
        Dr = (const T*)R.D;
        ldr = R.ld;
      }
      if (lrows > 0 && rcols > 0 && inner == 0) return zero(dst, ldd, lrows, rcols);
      return launch_csr_spmm<T>(ctx, a.rp, a.ci, (const T*)a.v, a.rows, a.cols, Dr, ldr, rcols, dst, ldd, epi);
    }
    if (R.f) {
      // X op(R) = X (op(R)^T)^T: the CSR of op(R)^T is R's CSR for op T, its transpose's for N
      const CsrView b = csr_op(*R.f, opr == 'N' ? 'T' : 'N');
      if (lrows > 0 && rcols > 0 && inner == 0) return zero(dst, ldd, lrows, rcols);
      return launch_dense_csrT<T>(ctx, (const T*)L.D, L.ld, lrows, b.rp, b.ci, (const T*)b.v, b.rows, b.cols, dst,
                                  ldd, epi);
    }
    if (lrows > 0 && rcols > 0 && inner == 0) return zero(dst, ldd, lrows, rcols);
    return launch_gemm_seq<T>(ctx, (const T*)L.D, L.ld, (const T*)R.D, R.ld, dst, ldd, lrows, rcols, inner);
  }

  fgb_status zero(T* dst, int ldd, int rows, int cols) {
    const int g = std::max(1, std::min(4 * ctx->sm_count, (int)(((long)rows * cols + 255) / 256)));
    k_zero2d<T><<<g, 256, 0, ctx->stream>>>(dst, ldd, rows, cols);
    FGB_LAUNCHED(ctx);
    return FGB_OK;
  }

  // dynprog_multiply_rec (faust_prod_opt_gen.hpp:8-79).
  fgb_status rec(int i, int j, bool root, PNode& out) {
    if (i == j) {
      out = leaves[i];
      return FGB_OK;
    }
    PNode p1, p2;
    char opl, opr;
    if (j - i == 1) {
      p1 = leaves[i];
      p2 = leaves[j];
      opl = op;
      opr = j < n - 1 ? op : last_op;
    } else {
      const int k = split[(size_t)i * n + j];
      FGB_TRY(rec(i, k, false, p1));
      FGB_TRY(rec(k + 1, j, false, p2));
      opl = i == k ? op : 'N';
      opr = k + 1 == j ? (j == n - 1 ? last_op : op) : 'N';
    }
    const int rows = opl == 'N' ? p1.rows : p1.cols, cols = opr == 'N' ? p2.cols : p2.rows;
    T* dst = root ? Y : take((size_t)rows * cols);
    const int ldd = root ? ldy : std::max(1, rows);
    FGB_TRY(gemm(p1, opl, p2, opr, dst, ldd));
    out = PNode();
    out.D = dst;
    out.ld = ldd;
    out.rows = rows;
    out.cols = cols;
    return FGB_OK;
  }
};

// Elements of workspace the DYNPROG evaluation takes (upper bound: every
// computed product plus a dense image per sparse x sparse leaf pair).
static size_t dynprog_ws_elems(int n, const std::vector<PNode>& lv, const std::vector<int>& split, char op,
                               char last_op) {
  size_t total = 0;
  // walk the tree the way ProductRun::rec does, summing take() sizes
  struct W {
    int n;
    const std::vector<PNode>& lv;
    const std::vector<int>& split;
    char op, last_op;
    size_t total = 0;
    void dims(int i, int j, int& r, int& c) {
      if (i == j) {
        r = lv[i].rows;
        c = lv[i].cols;
        return;
      }
      int k, r1, c1, r2, c2;
      char opl, opr;
      if (j - i == 1) {
        r1 = lv[i].rows, c1 = lv[i].cols, r2 = lv[j].rows, c2 = lv[j].cols;
        opl = op;
        opr = j < n - 1 ? op : last_op;
        if (lv[i].f && lv[j].f) total += (((size_t)r2 * c2) + 31) & ~size_t(31);
      } else {
        k = split[(size_t)i * n + j];
        dims(i, k, r1, c1);
        dims(k + 1, j, r2, c2);
        opl = i == k ? op : 'N';
        opr = k + 1 == j ? (j == n - 1 ? last_op : op) : 'N';
      }
      r = opl == 'N' ? r1 : c1;
      c = opr == 'N' ? c2 : r2;
      total += (((size_t)r * c) + 31) & ~size_t(31);
    }
  } w{n, lv, split, op, last_op};
  int r, c;
  w.dims(0, n - 1, r, c);
  total += w.total;
  return total;
}

static fgb_status ensure_ws(fgb_faust* F, size_t bytes) {
  if (F->pws_bytes >= bytes) return FGB_OK;
  dfree(F->pws);
  F->pws = nullptr;
  F->pws_bytes = 0;
  FGB_TRY(dmalloc(F->ctx, &F->pws, bytes));
  F->pws_bytes = bytes;
  return FGB_OK;
}

// Transform::get_product (CPU/faust_Transform.hpp:598-656): the dense image
// of the last factor of op(F)'s product order, then the other J-1 factors
// applied to it right to left (one fused launch when the intermediates would
// leave L2, as for Faust x dense).
template <typename T>
static fgb_status run_default(fgb_faust* F, char op, void* Y, int ldy) {
  fgb_ctx* ctx = F->ctx;
  const int J = (int)F->f.size();
  const DevFactor& last = op == 'N' ? F->f[J - 1] : F->f[0];
  DevFactor img = last;
  if (op != 'N') {
    img.rowptr = last.t_rowptr;
    img.colind = last.t_colind;
    img.val = last.t_val;
    img.rows = last.cols;
    img.cols = last.rows;
  }
  if (J == 1 && ldy == std::max(1, img.rows)) return launch_csr_to_dense<T>(ctx, img, (T*)Y);
  FGB_TRY(ensure_ws(F, sizeof(T) * std::max<size_t>(32, (size_t)img.rows * img.cols)));
  T* im = (T*)F->pws;
  FGB_TRY(launch_csr_to_dense<T>(ctx, img, im));
  if (J == 1) {
    FGB_CUDA(ctx, cudaMemcpy2DAsync(Y, sizeof(T) * ldy, im, sizeof(T) * img.rows, sizeof(T) * img.rows, img.cols,
                                    cudaMemcpyDeviceToDevice, ctx->stream));
    return FGB_OK;
  }
  return faust_apply_prefix(F, op, J - 1, im, std::max(1, img.rows), img.cols, Y, ldy);
}

template <typename T>
static fgb_status run_dynprog(fgb_faust* F, char op, const void* X, int ldx, int ncols, void* Y, int ldy) {
  fgb_ctx* ctx = F->ctx;
  ProductRun<T> pr;
  pr.ctx = ctx;
  const int J = (int)F->f.size();
  // factors in product order: reversed for op T/H (TransformHelper.hpp:1146-1151)
  for (int q = 0; q < J; ++q) {
    const DevFactor& f = F->f[op == 'N' ? q : J - 1 - q];
    PNode nd;
    nd.leaf = q;
    nd.f = &f;
    nd.rows = f.rows;
    nd.cols = f.cols;
    pr.leaves.push_back(nd);
  }
  pr.op = op;
  pr.last_op = op;
  if (X) {
    PNode nd;
    nd.leaf = J;
    nd.D = X;
    nd.ld = ldx;
    nd.rows = op == 'N' ? F->f.back().cols : F->f.front().rows;
    nd.cols = ncols;
    pr.leaves.push_back(nd);
    pr.last_op = 'N';
  }
  pr.n = (int)pr.leaves.size();
  pr.Y = (T*)Y;
  pr.ldy = ldy;
  if (pr.n == 1) {
    // one factor, no operand: Transform::get_product's copy (handled by the caller)
    return fail(ctx, FGB_ERR_INVALID_ARG, "dynprog: a single leaf is a copy, not a product");
  }
  std::vector<int> rows, cols, nnz, dense;
  for (auto& l : pr.leaves) {
    rows.push_back(l.rows);
    cols.push_back(l.cols);
    nnz.push_back(l.f ? l.f->nnz : mul32(l.rows, l.cols));
    dense.push_back(l.f ? 0 : 1);
  }
  dynprog_splits(pr.n, rows.data(), cols.data(), nnz.data(), dense.data(), op, pr.split);
  // A plan that splits off the leftmost leaf at every level is the
  // right-to-left chain: the same products in the same order as the default
  // path, which runs them as one fused launch where that pays.
  bool r2l = true;
  for (int i = 0; i + 2 < pr.n; ++i) r2l = r2l && pr.split[(size_t)i * pr.n + pr.n - 1] == i;
  if (r2l) {
    if (!X) return run_default<T>(F, op, Y, ldy);
    return faust_apply_prefix(F, op, J, X, ldx, ncols, Y, ldy);
  }
  FGB_TRY(ensure_ws(F, sizeof(T) * std::max<size_t>(32, dynprog_ws_elems(pr.n, pr.leaves, pr.split, op,
                                                                              pr.last_op))));
  pr.ws = (T*)F->pws;
  PNode root;
  return pr.rec(0, pr.n - 1, true, root);
}

static bool product_ok(fgb_faust* F, char& op) {
  if (op == 'n') op = 'N';
  if (op == 't' || op == 'h' || op == 'H') op = 'T';  // real scalars: adjoint = transpose
  return op == 'N' || op == 'T';
}

static bool all_csr_f(const fgb_faust* F) {
  for (auto& f : F->f)
    if (f.format != FGB_CSR) return false;
  return !F->f.empty();
}

}  // namespace fgb

using namespace fgb;

extern "C" {

fgb_status fgb_dynprog_plan(int n, const int* rows, const int* cols, const int* nnz, const int* is_dense, char op,
                            int* split) {
  if (n <= 0 || !rows || !cols || !nnz || !is_dense || !split) return FGB_ERR_INVALID_ARG;
  if (op == 'n') op = 'N';
  std::vector<int> s;
  dynprog_splits(n, rows, cols, nnz, is_dense, op, s);
  for (size_t e = 0; e < s.size(); ++e) split[e] = s[e];
  return FGB_OK;
}

fgb_status fgb_faust_product(fgb_faust* F, char op, int order, void* Y, int ldy) {
  if (!F) return FGB_ERR_INVALID_ARG;
  fgb_ctx* ctx = F->ctx;
  if (!Y) return fail(ctx, FGB_ERR_INVALID_ARG, "fgb_faust_product: null output");
  if (!product_ok(F, op)) return fail(ctx, FGB_ERR_INVALID_ARG, "fgb_faust_product: op must be N, T or H");
  if (order != FGB_ORDER_DEFAULT_L2R && order != FGB_ORDER_DYNPROG)
    return fail(ctx, FGB_ERR_NOT_SUPPORTED, "fgb_faust_product: order must be DEFAULT_L2R or DYNPROG");
  if (!all_csr_f(F)) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "fgb_faust_product: CSR Fausts only");
  const int rows = op == 'N' ? F->f.front().rows : F->f.back().cols;
  if (ldy < std::max(1, rows)) return fail(ctx, FGB_ERR_INVALID_ARG, "fgb_faust_product: ldy smaller than the rows");
  FGB_CUDA(ctx, cudaSetDevice(ctx->device));
  if (op != 'N')
    for (auto& f : F->f)
      if (!f.has_t) FGB_TRY(csr_build_transpose(ctx, F->dtype, f));
  // one factor, or the default order: Transform::get_product (TransformHelper.hpp:1144-1161)
  if (order == FGB_ORDER_DEFAULT_L2R || F->f.size() == 1) {
    if (F->dtype == FGB_F64) return run_default<double>(F, op, Y, ldy);
    return run_default<float>(F, op, Y, ldy);
  }
  // dense x sparse products walk the transposes of the right-hand factors
  for (auto& f : F->f)
    if (!f.has_t) FGB_TRY(csr_build_transpose(ctx, F->dtype, f));
  if (F->dtype == FGB_F64) return run_dynprog<double>(F, op, nullptr, 0, 0, Y, ldy);
  return run_dynprog<float>(F, op, nullptr, 0, 0, Y, ldy);
}

fgb_status fgb_faust_mul_dynprog(fgb_faust* F, char op, const void* X, int ldx, int ncols, void* Y, int ldy) {
  if (!F) return FGB_ERR_INVALID_ARG;
  fgb_ctx* ctx = F->ctx;
  if (!X || !Y || ncols < 0) return fail(ctx, FGB_ERR_INVALID_ARG, "fgb_faust_mul_dynprog: null operand");
  if (!product_ok(F, op)) return fail(ctx, FGB_ERR_INVALID_ARG, "fgb_faust_mul_dynprog: op must be N, T or H");
  if (!all_csr_f(F)) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "fgb_faust_mul_dynprog: CSR Fausts only");
  const int in_rows = op == 'N' ? F->f.back().cols : F->f.front().rows;
  const int out_rows = op == 'N' ? F->f.front().rows : F->f.back().cols;
  if (ldx < std::max(1, in_rows) || ldy < std::max(1, out_rows))
    return fail(ctx, FGB_ERR_INVALID_ARG, "fgb_faust_mul_dynprog: leading dimension smaller than the row count");
  if (ncols == 0) return FGB_OK;
  FGB_CUDA(ctx, cudaSetDevice(ctx->device));
  for (auto& f : F->f)
    if (!f.has_t) FGB_TRY(csr_build_transpose(ctx, F->dtype, f));
  if (F->dtype == FGB_F64) return run_dynprog<double>(F, op, X, ldx, ncols, Y, ldy);
  return run_dynprog<float>(F, op, X, ldx, ncols, Y, ldy);
}

}  // extern "C"
