// prox.cuh — projections of a dense device matrix (ConstraintGeneric::project)
// and the dense -> CSR factor conversion used by palm4msa2.
#pragma once

#include "fgb_internal.cuh"

namespace fgb {

// Device state of one global top-k selection (prox_sp).
struct TopkState {
  unsigned long long prefix;  // bits of the threshold found so far
  unsigned long long mask;
  unsigned long long t;       // key of the k-th largest magnitude
  long long k_rem;            // rank still to find inside the current prefix
  long long G;                // #{key > t}
  long long E;                // #{key == t}
  long long tau;              // position of the k-th key >= t (linear order)
  int sel_case;               // 0 unique / keep all, 1 prefix rule, 2 heap order, 3 t == 0
  int status;
  unsigned blocks_done;
  unsigned pad;
};

// Scratch owned by a context-level prox workspace (sized for rows*cols).
struct ProxWork {
  long cap_elems = 0;
  int cap_rows = 0;
  TopkState* state = nullptr;
  unsigned* hist = nullptr;          // 2048 bins
  unsigned char* flags = nullptr;    // one byte per entry
  long long* chunk_cnt = nullptr;    // per-chunk counts (tau search / reductions)
  double* partials = nullptr;        // per-chunk reduction partials
  double* scal = nullptr;            // scalars: [0] = inverse norm (as FPP), [1] = norm
  int* row_cnt = nullptr;            // rows+1
  void* supp = nullptr;              // device copy of a support (SUPP)
  size_t supp_bytes = 0;
  void* heap = nullptr;              // heap of the tie replay when it does not fit on chip
  long heap_cap = 0;
  // pre-filtered tie replay (allocated on first use, only in workspaces made
  // by prox_work_reserve; a workspace built by hand keeps the one-block replay)
  int growable = 0;
  void* cand = nullptr;              // candidate (key, position) slots, one per entry
  long cand_cap = 0;
  unsigned long long* wbound = nullptr;  // per-window lower bounds of the k-th largest key
  int* wcount = nullptr;             // per-window candidate counts
  void* heap2 = nullptr;             // split heap (keys, positions) when it does not fit on chip
  long heap2_cap = 0;
  // single-launch radix select (workspaces made by prox_work_reserve): one
  // 2048-bin histogram per pass, then the grid barrier's two words and the
  // key-list counter; the key list of a small bucket
  unsigned* hist_passes = nullptr;
  unsigned long long* rs_list = nullptr;
  // split sum of squares of the normalisation (workspaces made by
  // prox_work_reserve): segment partials and per-lane masks (kept zero
  // between uses)
  double* sq_seg = nullptr;
  unsigned* sq_mask = nullptr;
  unsigned* sq_done = nullptr;  // segment blocks finished per chunk (kept zero between uses)
  long sq_chunks = 0;
  // the matrix whose non-zeros per row and column the normalisation counted
  // into row_cnt (consumed by the dense -> CSR conversion, which zeroes the
  // counts again), or null
  const void* counted = nullptr;
};

fgb_status prox_work_reserve(fgb_ctx* ctx, ProxWork& w, long elems, int rows);
void prox_work_free(ProxWork& w);

// Queues the projection of the dense rows x cols matrix M (column-major,
// ld = rows) in place.  supp_dev: device support for FGB_SUPP.  The first
// failure status is written to *d_status (device int) when not null.
template <typename T>
fgb_status launch_prox(fgb_ctx* ctx, ProxWork& w, const fgb_constraint& c, T* M, int rows, int cols,
                       const T* supp_dev, int* d_status);

// Queues dense -> CSR conversion of the non-zero entries of M into the
// factor f (capacity f.cap; more entries set *status) and, when f.t_* is set,
// the CSR of its transpose.  f.nnz is only known on the device afterwards
// (rowptr[rows]).
template <typename T>
fgb_status launch_dense_to_csr(fgb_ctx* ctx, ProxWork& w, const T* M, DevFactor& f, int* status);

}  // namespace fgb
