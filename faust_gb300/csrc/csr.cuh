// csr.cuh — CSR x dense kernels shared by the Faust product and PALM.
//
// Every output entry follows the canonical row order of rowdot.cuh (a
// sequential fused multiply-add over the sparse operand's entries in stored
// order from +0 for rows of at most 16 entries; 16-entry chunks combined by a
// pairwise tree beyond), the order the oracle restates, so results are
// bit-identical to the CPU restatement.
#pragma once

#include "fgb_internal.cuh"

namespace fgb {

// Epilogue applied to each accumulated entry y(i,j):
//   EPI_STORE        y = acc
//   EPI_LAMBDA_MINUS y = (lambda * acc) - aux(i,j)      (PALM residual E)
//   EPI_D_MINUS      y = aux(i,j) - (alpha * acc)       (PALM gradient step)
enum { EPI_STORE = 0, EPI_LAMBDA_MINUS = 1, EPI_D_MINUS = 2 };

template <typename T>
struct Epi {
  int mode = EPI_STORE;
  const T* aux = nullptr;  // column-major, leading dimension ld_aux
  int ld_aux = 0;
  const T* scal = nullptr; // device scalar (lambda or alpha)
};

template <typename T>
__device__ __forceinline__ T epi_apply(const Epi<T>& e, T acc, long i, long j, T s) {
  if (e.mode == EPI_LAMBDA_MINUS) return subr(mulr(s, acc), e.aux[i + j * (long)e.ld_aux]);
  if (e.mode == EPI_D_MINUS) return subr(e.aux[i + j * (long)e.ld_aux], mulr(s, acc));
  return acc;
}

// Launch helpers (csr.cu).
// Y = S X  (S: rows x inner CSR; X: inner x ncols; Y: rows x ncols).
// max_row: longest row of S if known (rows of more than 16 entries run in a
// separate kernel), -1 when unknown; d_max_row: the same figure in device
// memory (or null), read by that kernel, which ends at once without long rows.
template <typename T>
fgb_status launch_csr_spmm(fgb_ctx* ctx, const int* rowptr, const int* colind, const T* val, int rows, int inner,
                           const T* X, int ldx, int ncols, T* Y, int ldy, const Epi<T>& epi, int max_row = -1,
                           const int* d_max_row = nullptr);
// Y = X S^T given the CSR of S (S: srows x scols; X: xrows x scols; Y: xrows x srows).
template <typename T>
fgb_status launch_dense_csrT(fgb_ctx* ctx, const T* X, int ldx, int xrows, const int* rowptr, const int* colind,
                             const T* val, int srows, int scols, T* Y, int ldy, const Epi<T>& epi, int max_row = -1,
                             const int* d_max_row = nullptr);
// Dense column-major (ld = rows) image of a CSR factor.
template <typename T>
fgb_status launch_csr_to_dense(fgb_ctx* ctx, const DevFactor& f, T* out);

struct ChainDesc {
  const int* rowptr;
  const int* colind;
  const void* val;
  int rows, cols;
};

}  // namespace fgb
