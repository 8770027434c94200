// faust.cu — the Faust handle: device-resident factor chains and the
// Faust x dense product entry points (fgb_faust_*).
#include <algorithm>
#include <cstring>

#include "csr.cuh"
#include "power.cuh"

namespace fgb {
fgb_status chain_fused(fgb_ctx* ctx, fgb_dtype dt, const ChainDesc* d_desc, int nfac, const void* X, int ldx,
                       int ncols, void* Y, int ldy, int maxdim, bool probe_only, bool* fits);
fgb_status launch_bsr_spmm(fgb_ctx* ctx, const DevFactor& f, const __nv_bfloat16* X, int ldx, int ncols,
                           __nv_bfloat16* Y, int ldy);

fgb_status bsr_tc_prepare(fgb_ctx* ctx, DevFactor& f);

void free_factor(DevFactor& f) {
  dfree(f.aux);
  dfree(f.rowptr);
  dfree(f.colind);
  dfree(f.val);
  dfree(f.t_rowptr);
  dfree(f.t_colind);
  dfree(f.t_val);
  dfree(f.d_maxrc);
  f = DevFactor();
}

// Copies one host factor description into device memory.
static fgb_status upload_factor(fgb_ctx* ctx, fgb_dtype dt, const fgb_factor_desc& d, DevFactor& f) {
  const size_t es = dtype_size(dt);
  f.format = d.format;
  f.rows = d.rows;
  f.cols = d.cols;
  f.nnz = d.nnz;
  f.cap = std::max(1, d.nnz);
  f.bm = d.bm;
  f.bn = d.bn;
  int nrp = 0;
  size_t nval = 0;
  if (d.format == FGB_CSR) {
    nrp = d.rows + 1;
    nval = (size_t)d.nnz;
  } else {
    nrp = d.rows / d.bm + 1;
    nval = (size_t)d.nnz * d.bm * d.bn;
  }
  FGB_TRY(dmalloc(ctx, (void**)&f.rowptr, sizeof(int) * nrp));
  FGB_TRY(dmalloc(ctx, (void**)&f.colind, sizeof(int) * std::max(1, d.nnz)));
  FGB_TRY(dmalloc(ctx, &f.val, es * std::max<size_t>(1, nval)));
  FGB_CUDA(ctx, cudaMemcpyAsync(f.rowptr, d.rowptr, sizeof(int) * nrp, cudaMemcpyHostToDevice, ctx->stream));
  if (d.nnz > 0) {
    FGB_CUDA(ctx, cudaMemcpyAsync(f.colind, d.colind, sizeof(int) * d.nnz, cudaMemcpyHostToDevice, ctx->stream));
    FGB_CUDA(ctx, cudaMemcpyAsync(f.val, d.values, es * nval, cudaMemcpyHostToDevice, ctx->stream));
  }
  if (d.format == FGB_BSR) FGB_TRY(bsr_tc_prepare(ctx, f));
  if (d.format == FGB_CSR) {
    // longest row and column: products skip the long-row kernel without them
    std::vector<int> cc(std::max(1, d.cols), 0);
    int mr = 0, mc = 0;
    for (int r = 0; r < d.rows; ++r) mr = std::max(mr, d.rowptr[r + 1] - d.rowptr[r]);
    for (int p = 0; p < d.nnz; ++p) mc = std::max(mc, ++cc[d.colind[p]]);
    f.max_row = mr;
    f.max_col = mc;
  }
  return FGB_OK;
}

static fgb_status validate_desc(fgb_ctx* ctx, fgb_dtype dt, const fgb_factor_desc& d) {
  if (d.rows <= 0 || d.cols <= 0 || d.nnz < 0) return fail(ctx, FGB_ERR_INVALID_ARG, "factor: bad shape or nnz");
  if (!d.rowptr || (d.nnz > 0 && (!d.colind || !d.values)))
    return fail(ctx, FGB_ERR_INVALID_ARG, "factor: null array");
  if (d.format == FGB_CSR) {
    if (dt == FGB_BF16) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "CSR factors are F32 or F64");
    if (d.rowptr[0] != 0 || d.rowptr[d.rows] != d.nnz)
      return fail(ctx, FGB_ERR_INVALID_ARG, "CSR rowptr must start at 0 and end at nnz");
    for (int i = 0; i < d.rows; ++i) {
      if (d.rowptr[i + 1] < d.rowptr[i]) return fail(ctx, FGB_ERR_INVALID_ARG, "CSR rowptr not monotone");
      for (int p = d.rowptr[i]; p < d.rowptr[i + 1]; ++p) {
        if (d.colind[p] < 0 || d.colind[p] >= d.cols) return fail(ctx, FGB_ERR_INVALID_ARG, "CSR column out of range");
        if (p > d.rowptr[i] && d.colind[p] <= d.colind[p - 1])
          return fail(ctx, FGB_ERR_INVALID_ARG, "CSR columns must be sorted and unique within a row");
      }
    }
  } else if (d.format == FGB_BSR) {
    if (dt != FGB_BF16) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "BSR factors are BF16 (FP32 accumulation)");
    if (d.bm != 64 || d.bn != 64) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "BSR blocks must be 64 x 64");
    if (d.rows % d.bm || d.cols % d.bn) return fail(ctx, FGB_ERR_INVALID_ARG, "BSR shape not a multiple of the block");
    const int nbr = d.rows / d.bm, nbc = d.cols / d.bn;
    if (d.rowptr[0] != 0 || d.rowptr[nbr] != d.nnz)
      return fail(ctx, FGB_ERR_INVALID_ARG, "BSR browptr must start at 0 and end at the block count");
    for (int i = 0; i < nbr; ++i) {
      if (d.rowptr[i + 1] < d.rowptr[i]) return fail(ctx, FGB_ERR_INVALID_ARG, "BSR browptr not monotone");
      for (int p = d.rowptr[i]; p < d.rowptr[i + 1]; ++p)
        if (d.colind[p] < 0 || d.colind[p] >= nbc) return fail(ctx, FGB_ERR_INVALID_ARG, "BSR block column out of range");
    }
  } else {
    return fail(ctx, FGB_ERR_INVALID_ARG, "unknown factor format");
  }
  return FGB_OK;
}

static fgb_status ensure(fgb_ctx* ctx, void** p, size_t* have, size_t need) {
  if (*have >= need && *p) return FGB_OK;
  dfree(*p);
  *p = nullptr;
  *have = 0;
  FGB_TRY(dmalloc(ctx, p, need));
  *have = need;
  return FGB_OK;
}

// One launch per factor, right to left, ping-ponging between two buffers.
static fgb_status mul_per_factor(fgb_faust* F, const void* X, int ldx, int ncols, void* Y, int ldy) {
  fgb_ctx* ctx = F->ctx;
  const int J = (int)F->f.size();
  const size_t es = dtype_size(F->dtype);
  int maxrows = 0;
  for (auto& f : F->f) maxrows = std::max(maxrows, f.rows);
  if (J > 1) {
    size_t need = (size_t)maxrows * ncols * es;
    if (F->buf_bytes < need) {
      dfree(F->buf[0]);
      dfree(F->buf[1]);
      F->buf[0] = F->buf[1] = nullptr;
      F->buf_bytes = 0;
      FGB_TRY(dmalloc(ctx, &F->buf[0], need));
      FGB_TRY(dmalloc(ctx, &F->buf[1], need));
      F->buf_bytes = need;
    }
  }
  const void* in = X;
  int ldin = ldx;
  for (int k = J - 1; k >= 0; --k) {
    const DevFactor& f = F->f[k];
    void* out = (k == 0) ? Y : F->buf[(J - 1 - k) & 1];
    int ldout = (k == 0) ? ldy : f.rows;
    if (f.format == FGB_BSR) {
      FGB_TRY(launch_bsr_spmm(ctx, f, (const __nv_bfloat16*)in, ldin, ncols, (__nv_bfloat16*)out, ldout));
    } else if (F->dtype == FGB_F64) {
      FGB_TRY(launch_csr_spmm<double>(ctx, f.rowptr, f.colind, (const double*)f.val, f.rows, f.cols,
                                      (const double*)in, ldin, ncols, (double*)out, ldout, Epi<double>(), f.max_row,
                                      f.d_maxrc));
    } else {
      FGB_TRY(launch_csr_spmm<float>(ctx, f.rowptr, f.colind, (const float*)f.val, f.rows, f.cols,
                                     (const float*)in, ldin, ncols, (float*)out, ldout, Epi<float>(), f.max_row,
                                     f.d_maxrc));
    }
    in = out;
    ldin = ldout;
  }
  return FGB_OK;
}

static fgb_status fused_desc(fgb_faust* F) {
  if (F->chain_desc) return FGB_OK;
  std::vector<ChainDesc> h(F->f.size());
  for (size_t i = 0; i < F->f.size(); ++i) h[i] = ChainDesc{F->f[i].rowptr, F->f[i].colind, F->f[i].val,
                                                            F->f[i].rows, F->f[i].cols};
  FGB_TRY(dmalloc(F->ctx, &F->chain_desc, sizeof(ChainDesc) * h.size()));
  FGB_CUDA(F->ctx, cudaMemcpyAsync(F->chain_desc, h.data(), sizeof(ChainDesc) * h.size(), cudaMemcpyHostToDevice,
                                   F->ctx->stream));
  return FGB_OK;
}

// F^T X = S_J^T (... (S_1^T X)): the transposed factors applied first to last.
static fgb_status mul_per_factor_t(fgb_faust* F, const void* X, int ldx, int ncols, void* Y, int ldy) {
  fgb_ctx* ctx = F->ctx;
  const int J = (int)F->f.size();
  const size_t es = dtype_size(F->dtype);
  int maxcols = 0;
  for (auto& f : F->f) maxcols = std::max(maxcols, f.cols);
  if (J > 1) {
    size_t need = (size_t)maxcols * ncols * es;
    if (F->buf_bytes < need) {
      dfree(F->buf[0]);
      dfree(F->buf[1]);
      F->buf[0] = F->buf[1] = nullptr;
      F->buf_bytes = 0;
      FGB_TRY(dmalloc(ctx, &F->buf[0], need));
      FGB_TRY(dmalloc(ctx, &F->buf[1], need));
      F->buf_bytes = need;
    }
  }
  const void* in = X;
  int ldin = ldx;
  for (int k = 0; k < J; ++k) {
    const DevFactor& f = F->f[k];
    void* out = (k == J - 1) ? Y : F->buf[k & 1];
    int ldout = (k == J - 1) ? ldy : f.cols;
    if (F->dtype == FGB_F64) {
      FGB_TRY(launch_csr_spmm<double>(ctx, f.t_rowptr, f.t_colind, (const double*)f.t_val, f.cols, f.rows,
                                      (const double*)in, ldin, ncols, (double*)out, ldout, Epi<double>(), f.max_col,
                                      f.d_maxrc ? f.d_maxrc + 1 : nullptr));
    } else {
      FGB_TRY(launch_csr_spmm<float>(ctx, f.t_rowptr, f.t_colind, (const float*)f.t_val, f.cols, f.rows,
                                     (const float*)in, ldin, ncols, (float*)out, ldout, Epi<float>(), f.max_col,
                                     f.d_maxrc ? f.d_maxrc + 1 : nullptr));
    }
    in = out;
    ldin = ldout;
  }
  return FGB_OK;
}

static fgb_status fused_desc_t(fgb_faust* F) {
  if (F->chain_desc_t) return FGB_OK;
  const size_t J = F->f.size();
  std::vector<ChainDesc> h(J);
  for (size_t i = 0; i < J; ++i) {
    const DevFactor& f = F->f[J - 1 - i];
    h[i] = ChainDesc{f.t_rowptr, f.t_colind, f.t_val, f.cols, f.rows};
  }
  FGB_TRY(dmalloc(F->ctx, &F->chain_desc_t, sizeof(ChainDesc) * J));
  FGB_CUDA(F->ctx, cudaMemcpyAsync(F->chain_desc_t, h.data(), sizeof(ChainDesc) * J, cudaMemcpyHostToDevice,
                                   F->ctx->stream));
  return FGB_OK;
}

// Automatic mode: the fused chain saves the intermediate products' trips
// through memory, which only matters when they would leave L2; when every
// intermediate fits in L2 the per-factor launches (whole grid per factor,
// more rows in flight) are faster.  Threshold: a quarter of the L2.
static bool fused_pays(const fgb_faust* F, int ncols) {
  int dev = F->ctx->device, l2 = 0;
  cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
  size_t maxrows = 0;
  for (auto& f : F->f) maxrows = std::max(maxrows, (size_t)std::max(f.rows, f.cols));
  return maxrows * (size_t)ncols * dtype_size(F->dtype) > (size_t)std::max(l2, 1) / 4;
}

// The fused chain kernel sums each row in one sequential chain, the canonical
// order only for rows of at most ROW_CHUNK (16) entries: it runs only when
// every factor is known to have no longer row (columns for the transposed
// chain).
static bool rows_short(const fgb_faust* F, bool transposed) {
  for (auto& f : F->f) {
    const int m = transposed ? f.max_col : f.max_row;
    if (m < 0 || m > 16) return false;
  }
  return true;
}

static bool all_csr(const fgb_faust* F) {
  for (auto& f : F->f)
    if (f.format != FGB_CSR) return false;
  return true;
}

static int max_dim(const fgb_faust* F) {
  int m = 0;
  for (auto& f : F->f) m = std::max(m, std::max(f.rows, f.cols));
  return m;
}

// The first nfac factors of op(F)'s product order applied to X, right to
// left: G_0 ... G_{nfac-1} X with G_q = S_q (op N) or S_{J-1-q}^T (op T).
// Automatic mode as in fgb_faust_mul: the fused chain when it fits on chip
// and the intermediates would leave L2, else one launch per factor.
fgb_status faust_apply_prefix(fgb_faust* F, char op, int nfac, const void* X, int ldx, int ncols, void* Y, int ldy) {
  fgb_ctx* ctx = F->ctx;
  const int J = (int)F->f.size();
  const bool tr = op != 'N';
  if (nfac <= 0 || nfac > J) return fail(ctx, FGB_ERR_INVALID_ARG, "faust_apply_prefix: bad factor count");
  const int maxd = max_dim(F);
  bool fits = false, ran = false;
  if (nfac > 1) {
    FGB_TRY(bfly_chain(F, op, nfac, X, ldx, ncols, Y, ldy, false, &ran));
    if (ran) return FGB_OK;
  }
  if (rows_short(F, tr)) {
    FGB_TRY(tr ? fused_desc_t(F) : fused_desc(F));
    const ChainDesc* d = (const ChainDesc*)(tr ? F->chain_desc_t : F->chain_desc);
    chain_fused(ctx, F->dtype, d, nfac, X, ldx, ncols, Y, ldy, maxd, true, &fits);
    if (fits && nfac > 1 && fused_pays(F, ncols))
      return chain_fused(ctx, F->dtype, d, nfac, X, ldx, ncols, Y, ldy, maxd, false, nullptr);
  }
  const size_t es = dtype_size(F->dtype);
  if (nfac > 1) {
    size_t need = (size_t)maxd * ncols * es;
    if (F->buf_bytes < need) {
      dfree(F->buf[0]);
      dfree(F->buf[1]);
      F->buf[0] = F->buf[1] = nullptr;
      F->buf_bytes = 0;
      FGB_TRY(dmalloc(ctx, &F->buf[0], need));
      FGB_TRY(dmalloc(ctx, &F->buf[1], need));
      F->buf_bytes = need;
    }
  }
  const void* in = X;
  int ldin = ldx;
  for (int q = nfac - 1; q >= 0; --q) {
    const DevFactor& f = F->f[tr ? J - 1 - q : q];
    const int* rp = tr ? f.t_rowptr : f.rowptr;
    const int* ci = tr ? f.t_colind : f.colind;
    const void* v = tr ? f.t_val : f.val;
    const int rows = tr ? f.cols : f.rows, inner = tr ? f.rows : f.cols;
    void* out = (q == 0) ? Y : F->buf[(nfac - 1 - q) & 1];
    const int ldout = (q == 0) ? ldy : std::max(1, rows);
    const int ml = tr ? f.max_col : f.max_row;
    const int* dml = f.d_maxrc ? f.d_maxrc + (tr ? 1 : 0) : nullptr;
    if (F->dtype == FGB_F64)
      FGB_TRY(launch_csr_spmm<double>(ctx, rp, ci, (const double*)v, rows, inner, (const double*)in, ldin, ncols,
                                      (double*)out, ldout, Epi<double>(), ml, dml));
    else
      FGB_TRY(launch_csr_spmm<float>(ctx, rp, ci, (const float*)v, rows, inner, (const float*)in, ldin, ncols,
                                     (float*)out, ldout, Epi<float>(), ml, dml));
    in = out;
    ldin = ldout;
  }
  return FGB_OK;
}

}  // namespace fgb

fgb_faust::~fgb_faust() {
  if (pool) {
    for (auto& x : f) {
      fgb::dfree(x.aux);
      x = fgb::DevFactor();
    }
  }
  for (auto& x : f) fgb::free_factor(x);
  fgb::dfree(buf[0]);
  fgb::dfree(buf[1]);
  fgb::dfree(dx);
  fgb::dfree(dy);
  fgb::dfree(chain_desc);
  fgb::dfree(chain_desc_t);
  fgb::dfree(pws);
  fgb::dfree(brv[0]);
  fgb::dfree(brv[1]);
  if (s_in) {
    cudaStreamSynchronize(s_in);
    cudaStreamSynchronize(s_out);
    cudaStreamDestroy(s_in);
    cudaStreamDestroy(s_out);
    for (int c = 0; c < 4; ++c) {
      cudaEventDestroy(ev_in[c]);
      cudaEventDestroy(ev_done[c]);
    }
    cudaEventDestroy(ev_start);
  }
  if (hx) cudaFreeHost(hx);
  if (hy) cudaFreeHost(hy);
}

using namespace fgb;

extern "C" {

fgb_status fgb_faust_create(fgb_ctx* ctx, fgb_dtype dtype, int nfactors, const fgb_factor_desc* factors,
                            fgb_faust** out) {
  if (!ctx || !out) return FGB_ERR_INVALID_ARG;
  *out = nullptr;
  if (nfactors <= 0 || !factors) return fail(ctx, FGB_ERR_INVALID_ARG, "a Faust needs at least one factor");
  if (dtype_size(dtype) == 0) return fail(ctx, FGB_ERR_INVALID_ARG, "unknown dtype");
  for (int i = 0; i < nfactors; ++i) {
    FGB_TRY(validate_desc(ctx, dtype, factors[i]));
    if (i > 0 && factors[i - 1].cols != factors[i].rows)
      return fail(ctx, FGB_ERR_INVALID_ARG, "factor %d has %d rows, factor %d has %d columns", i, factors[i].rows,
                  i - 1, factors[i - 1].cols);
  }
  FGB_CUDA(ctx, cudaSetDevice(ctx->device));
  fgb_faust* F = new fgb_faust();
  F->ctx = ctx;
  F->dtype = dtype;
  F->f.resize(nfactors);
  for (int i = 0; i < nfactors; ++i) {
    fgb_status s = upload_factor(ctx, dtype, factors[i], F->f[i]);
    if (s != FGB_OK) {
      delete F;
      return s;
    }
  }
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    delete F;
    return cuda_check(ctx, e, "fgb_faust_create");
  }
  *out = F;
  return FGB_OK;
}

fgb_status fgb_faust_destroy(fgb_faust* F) {
  if (!F) return FGB_ERR_INVALID_ARG;
  cudaSetDevice(F->ctx->device);
  cudaStreamSynchronize(F->ctx->stream);
  delete F;
  return FGB_OK;
}

fgb_status fgb_faust_shape(const fgb_faust* F, int* rows, int* cols, int* nfactors) {
  if (!F) return FGB_ERR_INVALID_ARG;
  if (rows) *rows = F->f.front().rows;
  if (cols) *cols = F->f.back().cols;
  if (nfactors) *nfactors = (int)F->f.size();
  return FGB_OK;
}

fgb_status fgb_faust_mul(fgb_faust* F, const void* X, int ldx, int ncols, void* Y, int ldy, int mode) {
  if (!F) return FGB_ERR_INVALID_ARG;
  fgb_ctx* ctx = F->ctx;
  if (!X || !Y || ncols < 0) return fail(ctx, FGB_ERR_INVALID_ARG, "fgb_faust_mul: null operand");
  if (ldx < F->f.back().cols || ldy < F->f.front().rows)
    return fail(ctx, FGB_ERR_INVALID_ARG, "fgb_faust_mul: leading dimension smaller than the row count");
  if (ncols == 0) return FGB_OK;
  FGB_CUDA(ctx, cudaSetDevice(ctx->device));
  const bool csr = all_csr(F);
  bool fits = false;
  if (csr && (mode == 0 || mode == 3)) {
    bool ran = false;
    if (mode == 3 || F->f.size() > 1) FGB_TRY(bfly_chain(F, 'N', (int)F->f.size(), X, ldx, ncols, Y, ldy, mode == 3, &ran));
    if (ran) return FGB_OK;
    if (mode == 3) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "butterfly chain: not every factor is a butterfly factor");
  }
  if (csr && mode != 1 && rows_short(F, false)) {
    FGB_TRY(fused_desc(F));
    chain_fused(ctx, F->dtype, (const ChainDesc*)F->chain_desc, (int)F->f.size(), X, ldx, ncols, Y, ldy, max_dim(F),
                true, &fits);
  }
  if (mode == 2 && !fits)
    return fail(ctx, FGB_ERR_NOT_SUPPORTED,
                "fused chain: factors do not fit on chip, are not CSR or have rows of more than 16 entries");
  if (fits && (mode == 2 || (mode == 0 && F->f.size() > 1 && fused_pays(F, ncols))))
    return chain_fused(ctx, F->dtype, (const ChainDesc*)F->chain_desc, (int)F->f.size(), X, ldx, ncols, Y, ldy,
                       max_dim(F), false, nullptr);
  return mul_per_factor(F, X, ldx, ncols, Y, ldy);
}

fgb_status fgb_faust_mul_op(fgb_faust* F, char op, const void* X, int ldx, int ncols, void* Y, int ldy, int mode) {
  if (!F) return FGB_ERR_INVALID_ARG;
  if (op == 'N' || op == 'n') return fgb_faust_mul(F, X, ldx, ncols, Y, ldy, mode);
  fgb_ctx* ctx = F->ctx;
  if (op != 'T' && op != 't' && op != 'H' && op != 'h')
    return fail(ctx, FGB_ERR_INVALID_ARG, "fgb_faust_mul_op: op must be N, T or H");
  if (!X || !Y || ncols < 0) return fail(ctx, FGB_ERR_INVALID_ARG, "fgb_faust_mul_op: null operand");
  if (ldx < F->f.front().rows || ldy < F->f.back().cols)
    return fail(ctx, FGB_ERR_INVALID_ARG, "fgb_faust_mul_op: leading dimension smaller than the row count");
  if (!all_csr(F)) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "fgb_faust_mul_op: transposed products of CSR Fausts only");
  if (ncols == 0) return FGB_OK;
  FGB_CUDA(ctx, cudaSetDevice(ctx->device));
  // real scalars: the adjoint is the transpose
  for (auto& f : F->f)
    if (!f.has_t) FGB_TRY(csr_build_transpose(ctx, F->dtype, f));
  bool fits = false;
  int maxd = max_dim(F);
  if (mode == 0 || mode == 3) {
    bool ran = false;
    if (mode == 3 || F->f.size() > 1) FGB_TRY(bfly_chain(F, 'T', (int)F->f.size(), X, ldx, ncols, Y, ldy, mode == 3, &ran));
    if (ran) return FGB_OK;
    if (mode == 3) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "butterfly chain: not every factor is a butterfly factor");
  }
  if (mode != 1 && rows_short(F, true)) {
    FGB_TRY(fused_desc_t(F));
    chain_fused(ctx, F->dtype, (const ChainDesc*)F->chain_desc_t, (int)F->f.size(), X, ldx, ncols, Y, ldy, maxd, true,
                &fits);
  }
  if (mode == 2 && !fits) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "fused chain: factors do not fit on chip");
  if (fits && (mode == 2 || (mode == 0 && F->f.size() > 1 && fused_pays(F, ncols))))
    return chain_fused(ctx, F->dtype, (const ChainDesc*)F->chain_desc_t, (int)F->f.size(), X, ldx, ncols, Y, ldy,
                       maxd, false, nullptr);
  return mul_per_factor_t(F, X, ldx, ncols, Y, ldy);
}

fgb_status fgb_faust_mul_host(fgb_faust* F, const void* X, int ncols, void* Y) {
  if (!F) return FGB_ERR_INVALID_ARG;
  fgb_ctx* ctx = F->ctx;
  if (!X || !Y || ncols < 0) return fail(ctx, FGB_ERR_INVALID_ARG, "fgb_faust_mul_host: null operand");
  if (ncols == 0) return FGB_OK;
  FGB_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t es = dtype_size(F->dtype);
  const int rows = F->f.front().rows, inner = F->f.back().cols;
  const size_t xb = (size_t)inner * ncols * es, yb = (size_t)rows * ncols * es;
  size_t need = std::max(xb, yb);
  if (F->dxy_bytes < need) {
    dfree(F->dx);
    dfree(F->dy);
    F->dx = F->dy = nullptr;
    F->dxy_bytes = 0;
    FGB_TRY(dmalloc(ctx, &F->dx, need));
    FGB_TRY(dmalloc(ctx, &F->dy, need));
    F->dxy_bytes = need;
  }
  // Column chunks pipelined over three streams: the copy of chunk c + 1 in,
  // the product of chunk c and the copy of chunk c - 1 out overlap (host
  // buffers in pinned memory let the copy engines run beside the kernels).
  // Columns are independent, so the result does not depend on the chunking.
  int nchunk = 1;
  if (xb + yb >= ((size_t)32 << 20)) nchunk = (int)std::min<long>(4, std::max<long>(1, ncols / 512));
  if (nchunk == 1) {
    FGB_CUDA(ctx, cudaMemcpyAsync(F->dx, X, xb, cudaMemcpyHostToDevice, ctx->stream));
    FGB_TRY(fgb_faust_mul(F, F->dx, inner, ncols, F->dy, rows, 0));
    FGB_CUDA(ctx, cudaMemcpyAsync(Y, F->dy, yb, cudaMemcpyDeviceToHost, ctx->stream));
    FGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return check_kernel_err(ctx);
  }
  if (!F->s_in) {
    FGB_CUDA(ctx, cudaStreamCreateWithFlags(&F->s_in, cudaStreamNonBlocking));
    FGB_CUDA(ctx, cudaStreamCreateWithFlags(&F->s_out, cudaStreamNonBlocking));
    for (int c = 0; c < 4; ++c) {
      FGB_CUDA(ctx, cudaEventCreateWithFlags(&F->ev_in[c], cudaEventDisableTiming));
      FGB_CUDA(ctx, cudaEventCreateWithFlags(&F->ev_done[c], cudaEventDisableTiming));
    }
    FGB_CUDA(ctx, cudaEventCreateWithFlags(&F->ev_start, cudaEventDisableTiming));
  }
  // the copies start after the work already queued on the context's stream
  FGB_CUDA(ctx, cudaEventRecord(F->ev_start, ctx->stream));
  FGB_CUDA(ctx, cudaStreamWaitEvent(F->s_in, F->ev_start, 0));
  // whole 256-column tiles per chunk keep the BSR tensor-core path
  const int per = ((ncols + nchunk - 1) / nchunk + 255) / 256 * 256;
  for (int c = 0; c < nchunk; ++c) {
    const int c0 = c * per, nc = std::min(per, ncols - c0);
    if (nc <= 0) break;
    FGB_CUDA(ctx, cudaMemcpyAsync((char*)F->dx + es * (size_t)inner * c0, (const char*)X + es * (size_t)inner * c0,
                                  es * (size_t)inner * nc, cudaMemcpyHostToDevice, F->s_in));
    FGB_CUDA(ctx, cudaEventRecord(F->ev_in[c], F->s_in));
    FGB_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, F->ev_in[c], 0));
    FGB_TRY(fgb_faust_mul(F, (char*)F->dx + es * (size_t)inner * c0, inner, nc, (char*)F->dy + es * (size_t)rows * c0,
                          rows, 0));
    FGB_CUDA(ctx, cudaEventRecord(F->ev_done[c], ctx->stream));
    FGB_CUDA(ctx, cudaStreamWaitEvent(F->s_out, F->ev_done[c], 0));
    FGB_CUDA(ctx, cudaMemcpyAsync((char*)Y + es * (size_t)rows * c0, (const char*)F->dy + es * (size_t)rows * c0,
                                  es * (size_t)rows * nc, cudaMemcpyDeviceToHost, F->s_out));
  }
  FGB_CUDA(ctx, cudaStreamSynchronize(F->s_out));
  FGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return check_kernel_err(ctx);
}

fgb_status fgb_faust_spectral_norm(fgb_faust* F, int max_iter, double threshold, double* norm, int* flag) {
  if (!F || !norm) return FGB_ERR_INVALID_ARG;
  fgb_ctx* ctx = F->ctx;
  if (!all_csr(F)) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "spectral norm: CSR Fausts only");
  if (F->dtype != FGB_F64 && F->dtype != FGB_F32) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "spectral norm: F32/F64");
  if (max_iter <= 0) return fail(ctx, FGB_ERR_INVALID_ARG, "power_iteration :  nbr_iter_max <= 0");
  FGB_CUDA(ctx, cudaSetDevice(ctx->device));
  for (auto& f : F->f)
    if (!f.has_t) FGB_TRY(csr_build_transpose(ctx, F->dtype, f));
  double out = 0;
  int fl = 0;
  FGB_TRY(chain_spectral_norm_sync(ctx, F->dtype, F->f.data(), 0, (int)F->f.size(), max_iter, threshold, &out, &fl));
  *norm = out;
  if (flag) *flag = fl;
  return FGB_OK;
}

fgb_status fgb_faust_factor_info(const fgb_faust* F, int i, int* format, int* rows, int* cols, int* nnz) {
  if (!F || i < 0 || i >= (int)F->f.size()) return FGB_ERR_INVALID_ARG;
  const DevFactor& f = F->f[i];
  if (format) *format = f.format;
  if (rows) *rows = f.rows;
  if (cols) *cols = f.cols;
  if (nnz) *nnz = f.nnz;
  return FGB_OK;
}

fgb_status fgb_faust_factor_to_csr(fgb_faust* F, int i, int* host_rowptr, int* host_colind, void* host_values) {
  if (!F || i < 0 || i >= (int)F->f.size()) return FGB_ERR_INVALID_ARG;
  fgb_ctx* ctx = F->ctx;
  const DevFactor& f = F->f[i];
  if (f.format != FGB_CSR) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "factor is not CSR");
  FGB_CUDA(ctx, cudaSetDevice(ctx->device));
  FGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  FGB_CUDA(ctx, cudaMemcpy(host_rowptr, f.rowptr, sizeof(int) * (f.rows + 1), cudaMemcpyDeviceToHost));
  if (f.nnz) {
    FGB_CUDA(ctx, cudaMemcpy(host_colind, f.colind, sizeof(int) * f.nnz, cudaMemcpyDeviceToHost));
    FGB_CUDA(ctx, cudaMemcpy(host_values, f.val, dtype_size(F->dtype) * f.nnz, cudaMemcpyDeviceToHost));
  }
  return FGB_OK;
}

fgb_status fgb_faust_factor_to_bsr(fgb_faust* F, int i, int* host_browptr, int* host_bcolind, void* host_blocks) {
  if (!F || i < 0 || i >= (int)F->f.size()) return FGB_ERR_INVALID_ARG;
  fgb_ctx* ctx = F->ctx;
  const DevFactor& f = F->f[i];
  if (f.format != FGB_BSR) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "factor is not BSR");
  FGB_CUDA(ctx, cudaSetDevice(ctx->device));
  FGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  FGB_CUDA(ctx, cudaMemcpy(host_browptr, f.rowptr, sizeof(int) * (f.rows / f.bm + 1), cudaMemcpyDeviceToHost));
  if (f.nnz) {
    FGB_CUDA(ctx, cudaMemcpy(host_bcolind, f.colind, sizeof(int) * f.nnz, cudaMemcpyDeviceToHost));
    FGB_CUDA(ctx, cudaMemcpy(host_blocks, f.val, dtype_size(F->dtype) * (size_t)f.nnz * f.bm * f.bn,
                             cudaMemcpyDeviceToHost));
  }
  return FGB_OK;
}

fgb_status fgb_faust_factor_to_dense(fgb_faust* F, int i, void* host_dense) {
  if (!F || i < 0 || i >= (int)F->f.size() || !host_dense) return FGB_ERR_INVALID_ARG;
  fgb_ctx* ctx = F->ctx;
  const DevFactor& f = F->f[i];
  if (f.format != FGB_CSR) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "factor is not CSR");
  std::vector<int> rp(f.rows + 1), ci(std::max(1, f.nnz));
  const size_t es = dtype_size(F->dtype);
  std::vector<unsigned char> v(es * std::max(1, f.nnz));
  FGB_TRY(fgb_faust_factor_to_csr(F, i, rp.data(), ci.data(), v.data()));
  std::memset(host_dense, 0, es * (size_t)f.rows * f.cols);
  for (int r = 0; r < f.rows; ++r)
    for (int p = rp[r]; p < rp[r + 1]; ++p)
      std::memcpy((unsigned char*)host_dense + es * ((size_t)ci[p] * f.rows + r), v.data() + es * p, es);
  return FGB_OK;
}

}  // extern "C"
