// palm_batched.cu — many independent palm4msa2 instances of uneven sizes in
// ONE persistent launch.
//
// Each CTA (256 threads) takes the next instance from a device work queue
// (instances are ordered by decreasing cost on the host) and runs the whole
// palm4msa2 loop for it with block-level versions of the single-instance
// kernels: the same floating-point order (sequential fma per product entry,
// 256-lane canonical reductions), so every instance is bit-identical to the
// oracle run of that instance.  Dense blocks live in a per-CTA workspace in
// global memory (L2-resident for small n); power-iteration vectors in shared
// memory.  Constraints: spcol, splin, splincol (k <= 64), normcol, normlin,
// supp.  CTAs per SM (1 to 3) come from the caller or from the table of the
// offline sweep (faust_gb300/tune_batched.py).
#include <algorithm>
#include <cstring>
#include <vector>

#include "fgb_internal.cuh"
#include "rowdot.cuh"

namespace fgb {
namespace bat {

constexpr int BT = 256;
constexpr int MAXJ = 16;
constexpr int KMAX = 64;

template <typename T>
struct Fac {
  int rows, cols, cap, pad;
  int* rowptr;
  int* colind;
  T* val;
  int* t_rowptr;
  int* t_colind;
  T* t_val;
};

template <typename T>
struct Cons {
  int kind, k, normalized, pos;
  double s;
  const T* supp;  // device, rows x cols (SUPP)
};

template <typename T>
struct Inst {
  int J, arows, acols, status;
  const T* A;
  double lambda;  // in: initial lambda; out: final lambda
  Fac<T> f[MAXJ];
  Cons<T> c[MAXJ];
  int nnz[MAXJ];  // out: entries of each factor
  long long cycles;  // out: SM clock cycles its CTA spent on the instance
};

template <typename T>
struct Slot {
  T* D;
  T* buf0;
  T* buf1;
  T* packed;  // MAXJ blocks of maxdim*maxdim
  unsigned char* flags;
  int* cnt;
};

struct Params {
  int nb_it, r2l, packing_RL, no_lambda, norm2_max_iter, constant_step, no_lambda_error, norm2_fp64;
  double norm2_threshold, step_size;
  long maxdim2;
  int ninst;
  int stage_elems;  // shared-memory staging area of a CTA, in elements of T
  int lambda_from_init;  // start from lambda = <A, S> / ||S||^2 of the initial factors
};

// ------------------------------------------------------------------ block ops
template <typename T>
__device__ __forceinline__ T bat_tree(T* lane) {
  return lane_tree_256(lane);
}

template <typename T>
__device__ void b_zero(T* p, long n) {
  for (long i = threadIdx.x; i < n; i += BT) p[i] = T(0);
}

template <typename T>
__device__ void b_csr_to_dense(const Fac<T>& f, T* out) {
  b_zero(out, (long)f.rows * f.cols);
  __syncthreads();
  for (int i = threadIdx.x; i < f.rows; i += BT)
    for (int p = f.rowptr[i]; p < f.rowptr[i + 1]; ++p) out[i + (long)f.colind[p] * f.rows] = f.val[p];
  __syncthreads();
}

enum { E_STORE = 0, E_LAMBDA = 1, E_DMINUS = 2 };

template <typename T>
__device__ __forceinline__ T b_epi(int mode, T acc, const T* aux, long idx, T s) {
  if (mode == E_LAMBDA) return subr(mulr(s, acc), aux[idx]);
  if (mode == E_DMINUS) return subr(aux[idx], mulr(s, acc));
  return acc;
}

// Shared-memory staging area of a CTA (elements of T).
template <typename T>
struct Stage {
  T* p;
  int elems;
};


// dst[r + c * ldd] = src[r + c * lds] for r < rows, c < cols (thread t takes
// the entries t, t + BT, ... of the column-major order; four loads issued
// before their stores).
template <typename T>
__device__ __forceinline__ void b_copy(T* dst, int ldd, const T* src, long lds, int rows, int cols) {
  const int dr = BT % rows, dc = BT / rows;
  int r = (int)threadIdx.x % rows, c = (int)threadIdx.x / rows;
  while (c < cols) {
    int r1 = r + dr, c1 = c + dc;
    if (r1 >= rows) {
      r1 -= rows;
      ++c1;
    }
    const T v0 = src[r + (long)c * lds];
    const bool has1 = c1 < cols;
    const T v1 = has1 ? src[r1 + (long)c1 * lds] : T(0);
    dst[r + c * ldd] = v0;
    if (has1) dst[r1 + c1 * ldd] = v1;
    r = r1 + dr;
    c = c1 + dc;
    if (r >= rows) {
      r -= rows;
      ++c;
    }
  }
}

// A CSR matrix as seen by a block op: in global memory, or copied into the
// staging area.
template <typename T>
struct Csr {
  const int* rp;
  const int* ci;
  const T* v;
};

// Copies the CSR of a factor (nrows rows) to the front of the staging area
// when it takes at most half of it, and shrinks sg to the rest.  The caller
// synchronizes before the copy is read.
template <typename T>
__device__ Csr<T> b_stage_csr(const int* rp, const int* ci, const T* v, int nrows, Stage<T>& sg) {
  const int nnz = rp[nrows];
  const size_t vb = ((size_t)nnz * sizeof(T) + 15) & ~(size_t)15;
  const size_t ib = ((size_t)(nrows + 1 + nnz) * sizeof(int) + 15) & ~(size_t)15;
  if (vb + ib > (size_t)sg.elems * sizeof(T) / 2) return Csr<T>{rp, ci, v};
  T* sv = sg.p;
  int* srp = reinterpret_cast<int*>(reinterpret_cast<char*>(sg.p) + vb);
  int* sci = srp + nrows + 1;
  for (int i = threadIdx.x; i <= nrows; i += BT) srp[i] = rp[i];
  for (int i = threadIdx.x; i < nnz; i += BT) {
    sci[i] = ci[i];
    sv[i] = v[i];
  }
  sg.p = reinterpret_cast<T*>(reinterpret_cast<char*>(sg.p) + vb + ib);
  sg.elems -= (int)((vb + ib) / sizeof(T));
  return Csr<T>{srp, sci, sv};
}

// 16 bytes of T from shared memory (G = 16 / sizeof(T) values).
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
  static constexpr int G = 4;
  __device__ static void load(const float* p, float* o) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
    o[3] = v.w;
  }
};
template <>
struct Vec16<double> {
  static constexpr int G = 2;
  __device__ static void load(const double* p, double* o) {
    const double2 v = *reinterpret_cast<const double2*>(p);
    o[0] = v.x;
    o[1] = v.y;
  }
};

// Y = S X   (S: rows x inner CSR, X: inner x ncols, Y: rows x ncols; lds = rows).
// S and a block of X's columns are staged in shared memory, the block stored
// row by row (stride sx) so that the G columns a thread owns are one 16-byte
// read per stored entry; each output entry is the sequential fma over its
// row's entries (rows of more than 16 entries: the chunked order of
// rowdot.cuh), G of them in flight per thread.
template <typename T>
__device__ __noinline__ void b_spmm(const int* rp, const int* ci, const T* v, int rows, int inner, const T* X, int ldx,
                                   int ncols, T* Y, int mode, const T* aux, T s, Stage<T> sg) {
  constexpr int G = Vec16<T>::G;
  const Csr<T> S = b_stage_csr<T>(rp, ci, v, rows, sg);
  // block width: a multiple of G, row stride padded off multiples of 32 words
  int cb = sg.elems / max(1, inner) - G;
  cb = max(G, min(cb, (ncols + G - 1) / G * G) / G * G);
  for (int j0 = 0; j0 < ncols; j0 += cb) {
    const int nc = min(cb, ncols - j0);
    const int ncp = (nc + G - 1) / G * G;
    const int sx = ncp + (((ncp * (int)sizeof(T)) % 128 == 0) ? G : 0);
    // stage: st[k * sx + c] = X[k, j0 + c] (zero beyond ncols)
    {
      // eight loads in flight per thread before their stores
      const int dk = BT % inner, dcol = BT / inner;
      int k = (int)threadIdx.x % inner, c = (int)threadIdx.x / inner;
      while (c < ncp) {
        T vv[8];
        int kk[8], cc[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          kk[u] = k;
          cc[u] = c;
          vv[u] = c < nc ? X[k + (long)(j0 + c) * ldx] : T(0);
          k += dk;
          c += dcol;
          if (k >= inner) {
            k -= inner;
            ++c;
          }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (cc[u] < ncp) sg.p[kk[u] * sx + cc[u]] = vv[u];
      }
    }
    __syncthreads();
    const int ng = ncp / G;
    const int di = BT % rows, dg = BT / rows;
    int i = (int)threadIdx.x % rows, g = (int)threadIdx.x / rows;
    for (; g < ng; i += di, g += dg, (i >= rows ? (i -= rows, ++g) : 0)) {
      T acc[G];
#pragma unroll
      for (int u = 0; u < G; ++u) acc[u] = T(0);
      const int p0 = S.rp[i], p1 = S.rp[i + 1];
      // the canonical row order (rowdot.cuh) on one code path for every row
      // length (a short row is a single chunk), so that long and short rows
      // of one warp do not run one after the other
      row_long_g<T, G, 10>(S.ci, S.v, p0, p1, sg.p + g * G, sx,
                           [](const T* q, T (&o)[G]) { Vec16<T>::load(q, o); }, acc);
#pragma unroll
      for (int u = 0; u < G; ++u) {
        const int c = g * G + u;
        if (c < nc) {
          const long idx = i + (long)(j0 + c) * rows;
          Y[idx] = b_epi(mode, acc[u], aux, idx, s);
        }
      }
    }
    __syncthreads();
  }
}

// Y = X S^T given the CSR of S (srows rows): y[r, c] = sum over row c of S.
// S and a block of X's rows (all xcols columns, column-major with a row
// stride padded to G) are staged in shared memory; a thread owns G
// consecutive rows of one output column.
template <typename T>
__device__ __noinline__ void b_dense_csrT(const T* X, int xrows, int xcols, const int* rp, const int* ci, const T* v,
                                         int srows, T* Y, int mode, const T* aux, T s, Stage<T> sg) {
  constexpr int G = Vec16<T>::G;
  const Csr<T> S = b_stage_csr<T>(rp, ci, v, srows, sg);
  int rb = sg.elems / max(1, xcols) - G;
  rb = max(G, min(rb, (xrows + G - 1) / G * G) / G * G);
  for (int r0 = 0; r0 < xrows; r0 += rb) {
    const int nr = min(rb, xrows - r0);
    const int nrp = (nr + G - 1) / G * G;
    {
      // eight loads in flight per thread before their stores
      const int dr = BT % nrp, dcol = BT / nrp;
      int rl = (int)threadIdx.x % nrp, col = (int)threadIdx.x / nrp;
      while (col < xcols) {
        T vv[8];
        int rr[8], cc[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          rr[u] = rl;
          cc[u] = col;
          vv[u] = (col < xcols && rl < nr) ? X[r0 + rl + (long)col * xrows] : T(0);
          rl += dr;
          col += dcol;
          if (rl >= nrp) {
            rl -= nrp;
            ++col;
          }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (cc[u] < xcols) sg.p[rr[u] + cc[u] * nrp] = vv[u];
      }
    }
    __syncthreads();
    const int ng = nrp / G;
    const int dg = BT % ng, dc = BT / ng;
    int g = (int)threadIdx.x % ng, c = (int)threadIdx.x / ng;
    for (; c < srows; g += dg, c += dc, (g >= ng ? (g -= ng, ++c) : 0)) {
      T acc[G];
#pragma unroll
      for (int u = 0; u < G; ++u) acc[u] = T(0);
      const int p0 = S.rp[c], p1 = S.rp[c + 1];
      // the canonical row order (rowdot.cuh) on one code path for every row
      // length (a short row is a single chunk), so that long and short rows
      // of one warp do not run one after the other
      row_long_g<T, G, 10>(S.ci, S.v, p0, p1, sg.p + g * G, nrp,
                           [](const T* q, T (&o)[G]) { Vec16<T>::load(q, o); }, acc);
#pragma unroll
      for (int u = 0; u < G; ++u) {
        const int rl = g * G + u;
        if (rl < nr) {
          const long idx = r0 + rl + (long)c * xrows;
          Y[idx] = b_epi(mode, acc[u], aux, idx, s);
        }
      }
    }
    __syncthreads();
  }
}

// Canonical sum of a[i]*b[i] over i < n (every thread gets the result).
template <typename T>
__device__ T b_cdot(const T* a, const T* b, long n, T* lane) {
  return block_cdot<T>(a, b, n, lane);
}

// ------------------------------------------------------------------ power iteration
// Op o of the operator F F^H (or F^H F) of F[lo..hi): returns the CSR to
// apply and its output length.
template <typename T>
__device__ __forceinline__ void pi_op(const Fac<T>* F, int lo, int hi, bool tall, int o, const int*& rp,
                                      const int*& ci, const T*& v, int& rows) {
  const int m = hi - lo;
  bool fwd;
  int idx;
  if (tall) {  // F^H F: F x applies F[hi-1] first, then the adjoints F[lo]^H ...
    fwd = o < m;
    idx = fwd ? hi - 1 - o : lo + (o - m);
  } else {  // F F^H: adjoints F[lo]^H first, then F[hi-1] ...
    fwd = o >= m;
    idx = fwd ? hi - 1 - (o - m) : lo + o;
  }
  const Fac<T>& f = F[idx];
  if (fwd) {
    rp = f.rowptr;
    ci = f.colind;
    v = f.val;
    rows = f.rows;
  } else {
    rp = f.t_rowptr;
    ci = f.t_colind;
    v = f.t_val;
    rows = f.cols;
  }
}

// TransformHelper::spectralNorm of F[lo..hi) by Faust::power_iteration; the
// same steps as k_power_iteration (power.cu), on one block.
template <typename T, typename TC>
__device__ __noinline__ double b_spectral_norm(const Fac<T>* F, int lo, int hi, int max_iter, TC thr, const TC* x0, TC* vbuf,
                                  int maxn, TC* lane, int* st) {
  __shared__ TC s_nrm, s_inv;
  if (hi <= lo) return 1.0;
  for (int i = lo; i < hi; ++i)
    if (F[i].rowptr[F[i].rows] == 0) return 0.0;
  const int rows = F[lo].rows, cols = F[hi - 1].cols;
  const bool tall = cols < rows;
  const int n = tall ? cols : rows;
  const int nops = 2 * (hi - lo);
  TC* bufs[3] = {vbuf, vbuf + maxn, vbuf + 2 * maxn};
  int xi = 0;
  for (int i = threadIdx.x; i < n; i += BT) bufs[0][i] = x0[i];
  __syncthreads();
  TC lam_old = TC(1), lam = TC(0);
  int it = 0;
  const TC athr = thr < TC(0) ? -thr : thr;
  auto absv = [](TC x) { return x < TC(0) ? -x : x; };
  while ((absv(subr(lam_old, lam)) > athr || absv(lam) <= athr) && it < max_iter) {
    ++it;
    lam_old = lam;
    TC* x = bufs[xi];
    const TC ss = b_cdot<TC>(x, x, n, lane);
    if (threadIdx.x == 0) {  // scalar FP64 work by one thread
      s_nrm = sqrtr(ss);
      s_inv = s_nrm == TC(0) ? TC(0) : divr(TC(1), s_nrm);
    }
    __syncthreads();
    const TC nrm = s_nrm;
    if (nrm == TC(0)) {
      if (threadIdx.x == 0) *st = FGB_ERR_ZERO_NORM;
      return 0.0;
    }
    const TC inv = s_inv;
    for (int i = threadIdx.x; i < n; i += BT) x[i] = mulr(x[i], inv);
    __syncthreads();
    int si = xi, di = (xi + 1) % 3;
    for (int o = 0; o < nops; ++o) {
      const int* rp;
      const int* ci;
      const T* v;
      int orow;
      pi_op(F, lo, hi, tall, o, rp, ci, v, orow);
      const TC* src = bufs[si];
      TC* dst = bufs[di];
      // the power iteration's row order (rowdot.cuh): long rows in chunks
      for (int r = threadIdx.x; r < orow; r += BT) {
        const int p0 = rp[r], p1 = rp[r + 1];
        if (p1 - p0 > ROW_CHUNK) {
          dst[r] = row_thread_long_inl<TC, T, 10>(ci, v, p0, p1, src, 1);
        } else {
          TC acc = TC(0);
#pragma unroll 4
          for (int p = p0; p < p1; ++p) acc = fmad((TC)v[p], src[ci[p]], acc);
          dst[r] = acc;
        }
      }
      __syncthreads();
      si = di;
      di = 3 - xi - si;
    }
    const TC* res = bufs[si];
    int nz = 0;
    for (int i = threadIdx.x; i < n; i += BT) nz |= (res[i] != TC(0));
    if (!__syncthreads_or(nz)) return 0.0;
    lam = b_cdot<TC>(x, res, n, lane);
    xi = si;
  }
  if (threadIdx.x == 0) {
    const TC r = sqrtr(lam);
    s_nrm = r < TC(0) ? -r : r;
  }
  __syncthreads();
  const double result = (double)s_nrm;
  __syncthreads();
  return result;
}

// ------------------------------------------------------------------ projections
__device__ __forceinline__ unsigned long long bkey(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffULL;
}
__device__ __forceinline__ unsigned long long bkey(float v) {
  return (unsigned long long)(__float_as_uint(v) & 0x7fffffffu);
}
template <typename T>
__device__ __forceinline__ T bpos(T v, int pos) {
  return (pos && v < T(0)) ? T(0) : v;
}

__device__ void b_heap_adjust(unsigned long long* hk, int* hi, int hole, int len, unsigned long long vk, int vi) {
  const int top = hole;
  int child = hole;
  while (child < (len - 1) / 2) {
    child = 2 * (child + 1);
    if (hk[child] > hk[child - 1]) child--;
    hk[hole] = hk[child];
    hi[hole] = hi[child];
    hole = child;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    hk[hole] = hk[child - 1];
    hi[hole] = hi[child - 1];
    hole = child - 1;
  }
  int parent = (hole - 1) / 2;
  while (hole > top && hk[parent] > vk) {
    hk[hole] = hk[parent];
    hi[hole] = hi[parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  hk[hole] = vk;
  hi[hole] = vi;
}

// The same adjustment on a heap whose entry j sits at hk[j * BT] (one heap
// per thread, interleaved in shared memory).
__device__ void b_heap_adjust_s(unsigned long long* hk, int* hi, int hole, int len, unsigned long long vk, int vi) {
  const int top = hole;
  int child = hole;
  while (child < (len - 1) / 2) {
    child = 2 * (child + 1);
    if (hk[child * BT] > hk[(child - 1) * BT]) child--;
    hk[hole * BT] = hk[child * BT];
    hi[hole * BT] = hi[child * BT];
    hole = child;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    hk[hole * BT] = hk[(child - 1) * BT];
    hi[hole * BT] = hi[(child - 1) * BT];
    hole = child - 1;
  }
  int parent = (hole - 1) / 2;
  while (hole > top && hk[parent * BT] > vk) {
    hk[hole * BT] = hk[parent * BT];
    hi[hole * BT] = hi[parent * BT];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  hk[hole * BT] = vk;
  hi[hole * BT] = vi;
}

// Per-line heap selection (std::partial_sort, |a| > |b|) of k entries, one
// thread per line.  The heaps live in the staging area when they fit (else
// in per-thread arrays); entries are read eight at a time.
template <typename T>
__device__ __noinline__ void b_line_topk(const T* M, int rows, int cols, bool by_col, int k, int pos, unsigned char* flags,
                            unsigned char bit, Stage<T> sg) {
  const int nl = by_col ? cols : rows, len = by_col ? rows : cols;
  const long step = by_col ? 1 : rows;
  const bool on_chip = (size_t)k * BT * 12 <= (size_t)sg.elems * sizeof(T);
  unsigned long long* shk = reinterpret_cast<unsigned long long*>(sg.p) + threadIdx.x;
  int* shi = reinterpret_cast<int*>(reinterpret_cast<unsigned long long*>(sg.p) + (size_t)k * BT) + threadIdx.x;
  for (int line = threadIdx.x; line < nl; line += BT) {
    const long base = by_col ? (long)line * rows : line;
    if (k >= len) {
      for (int e = 0; e < len; ++e) flags[base + e * step] |= bit;
      continue;
    }
    if (on_chip) {
      for (int e = 0; e < k; ++e) {
        shk[e * BT] = bkey(bpos(M[base + e * step], pos));
        shi[e * BT] = e;
      }
      if (k >= 2)
        for (int parent = (k - 2) / 2; parent >= 0; --parent)
          b_heap_adjust_s(shk, shi, parent, k, shk[parent * BT], shi[parent * BT]);
      int e = k;
      for (; e + 8 <= len; e += 8) {
        unsigned long long kk[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) kk[u] = bkey(bpos(M[base + (e + u) * step], pos));
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (kk[u] > shk[0]) b_heap_adjust_s(shk, shi, 0, k, kk[u], e + u);
      }
      for (; e < len; ++e) {
        const unsigned long long key = bkey(bpos(M[base + e * step], pos));
        if (key > shk[0]) b_heap_adjust_s(shk, shi, 0, k, key, e);
      }
      for (int q = 0; q < k; ++q) flags[base + (long)shi[q * BT] * step] |= bit;
    } else {
      unsigned long long hk[KMAX];
      int hi[KMAX];
      for (int e = 0; e < k; ++e) {
        hk[e] = bkey(bpos(M[base + e * step], pos));
        hi[e] = e;
      }
      if (k >= 2)
        for (int parent = (k - 2) / 2; parent >= 0; --parent) b_heap_adjust(hk, hi, parent, k, hk[parent], hi[parent]);
      for (int e = k; e < len; ++e) {
        const unsigned long long key = bkey(bpos(M[base + e * step], pos));
        if (key > hk[0]) b_heap_adjust(hk, hi, 0, k, key, e);
      }
      for (int q = 0; q < k; ++q) flags[base + (long)hi[q] * step] |= bit;
    }
  }
  __syncthreads();
}

template <typename T>
__device__ __noinline__ bool b_project(const Cons<T>& c, T* M, int rows, int cols, unsigned char* flags, T* lane, int* st,
                          Stage<T> sg) {
  const long N = (long)rows * cols;
  int pos = c.pos;
  if (c.kind == FGB_SPCOL || c.kind == FGB_SPLIN || c.kind == FGB_SPLINCOL) {
    if (c.kind == FGB_SPLINCOL) pos = 0;
    if (c.k <= 0) {
      b_zero(M, N);
    } else {
      if (c.kind != FGB_SPLIN) b_line_topk(M, rows, cols, true, min(c.k, rows), pos, flags, 1, sg);
      if (c.kind != FGB_SPCOL) b_line_topk(M, rows, cols, false, min(c.k, cols), pos, flags, 2, sg);
      for (long i = threadIdx.x; i < N; i += BT) {
        const T v = bpos(M[i], pos);
        M[i] = flags[i] ? v : T(0);
        flags[i] = 0;
      }
    }
  } else if (c.kind == FGB_NORMCOL || c.kind == FGB_NORMLIN) {
    if (c.s == 0) {
      b_zero(M, N);
    } else {
      const bool by_col = c.kind == FGB_NORMCOL;
      const int nl = by_col ? cols : rows, len = by_col ? rows : cols;
      for (int line = 0; line < nl; ++line) {
        auto at = [&](long e) -> long { return by_col ? (long)line * rows + e : e * rows + line; };
        T total = T(0);
        for (long c0 = 0; c0 < len; c0 += CR_CHUNK) {
          const long c1 = min((long)len, c0 + CR_CHUNK);
          T acc = T(0);
          for (long e = c0 + threadIdx.x; e < c1; e += CR_LANES) {
            const T v = bpos(M[at(e)], pos);
            acc = fmad(v, v, acc);
          }
          lane[threadIdx.x] = acc;
          total = addr(total, bat_tree(lane));
        }
        __shared__ T s_scal;
        if (threadIdx.x == 0) {
          T scal = sqrtr(total);
          if (scal != T(0)) scal = divr((T)c.s, scal);
          s_scal = scal;
        }
        __syncthreads();
        const T scal = s_scal;
        for (long e = threadIdx.x; e < len; e += BT) M[at(e)] = mulr(bpos(M[at(e)], pos), scal);
        __syncthreads();
      }
    }
  } else if (c.kind == FGB_SUPP) {
    for (long i = threadIdx.x; i < N; i += BT) M[i] = mulr(bpos(M[i], pos), c.supp[i]);
  } else {
    if (threadIdx.x == 0) *st = FGB_ERR_NOT_SUPPORTED;
    return false;
  }
  __syncthreads();
  if (c.normalized) {
    T total = T(0);
    for (long c0 = 0; c0 < N; c0 += CR_CHUNK) {
      const long c1 = min(N, c0 + CR_CHUNK);
      T acc = T(0);
      for (long i = c0 + threadIdx.x; i < c1; i += CR_LANES) acc = fmad(M[i], M[i], acc);
      lane[threadIdx.x] = acc;
      total = addr(total, bat_tree(lane));
    }
    __shared__ T s_n, s_inv2;
    if (threadIdx.x == 0) {
      s_n = sqrtr(total);
      s_inv2 = s_n == T(0) ? T(0) : (T)__ddiv_rn(1.0, (double)s_n);
    }
    __syncthreads();
    const T n = s_n;
    if (n == T(0)) {
      if (threadIdx.x == 0) *st = FGB_ERR_ZERO_NORM;
      return false;
    }
    const T inv = s_inv2;
    for (long i = threadIdx.x; i < N; i += BT) M[i] = mulr(M[i], inv);
    __syncthreads();
  }
  return true;
}

// dense -> CSR of the non-zero entries, then the transpose CSR.
template <typename T>
__device__ __noinline__ bool b_dense_to_csr(const T* M, Fac<T>& f, int* cnt, int* st) {
  __shared__ int part[BT];
  const int rows = f.rows, cols = f.cols;
  for (int i = threadIdx.x; i < rows; i += BT) {
    int c = 0;
    for (int j = 0; j < cols; ++j) c += M[i + (long)j * rows] != T(0);
    cnt[i] = c;
  }
  __syncthreads();
  const int per = (rows + BT - 1) / BT;
  const int r0 = threadIdx.x * per, r1 = min(rows, r0 + per);
  int s = 0;
  for (int r = r0; r < r1; ++r) s += cnt[r];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int u = 0; u < BT; ++u) {
      const int v = part[u];
      part[u] = run;
      run += v;
    }
    f.rowptr[rows] = run;
    if (run > f.cap) *st = FGB_ERR_INVALID_ARG;
  }
  __syncthreads();
  int run = part[threadIdx.x];
  for (int r = r0; r < r1; ++r) {
    f.rowptr[r] = run;
    run += cnt[r];
  }
  __syncthreads();
  if (f.rowptr[rows] > f.cap) return false;
  for (int i = threadIdx.x; i < rows; i += BT) {
    int p = f.rowptr[i];
    for (int j = 0; j < cols; ++j) {
      const T v = M[i + (long)j * rows];
      if (v != T(0)) {
        f.colind[p] = j;
        f.val[p] = v;
        ++p;
      }
    }
  }
  __syncthreads();
  // transpose: column counts, scan, ordered scatter (warp 0)
  const int nnz = f.rowptr[rows];
  for (int c = threadIdx.x; c <= cols; c += BT) cnt[c] = 0;
  __syncthreads();
  for (int p = threadIdx.x; p < nnz; p += BT) atomicAdd(&cnt[f.colind[p] + 1], 1);
  __syncthreads();
  const int cper = (cols + BT - 1) / BT;
  const int c0 = threadIdx.x * cper, c1 = min(cols, c0 + cper);
  s = 0;
  for (int c = c0; c < c1; ++c) s += cnt[c + 1];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int rr = 0;
    for (int u = 0; u < BT; ++u) {
      const int v = part[u];
      part[u] = rr;
      rr += v;
    }
    f.t_rowptr[cols] = rr;
  }
  __syncthreads();
  run = part[threadIdx.x];
  for (int c = c0; c < c1; ++c) {
    f.t_rowptr[c] = run;
    run += cnt[c + 1];
  }
  __syncthreads();
  for (int c = threadIdx.x; c < cols; c += BT) cnt[c] = f.t_rowptr[c];
  __syncthreads();
  if (threadIdx.x < 32) {
    const unsigned lane = threadIdx.x;
    for (int base = 0; base < nnz; base += 32) {
      const int p = base + (int)lane;
      const bool ok = p < nnz;
      int r = 0;
      if (ok) {
        int lo = 0, hi = rows - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (f.rowptr[mid] <= p) lo = mid;
          else hi = mid - 1;
        }
        r = lo;
      }
      const int c = ok ? f.colind[p] : -1 - (int)lane;
      const unsigned same = __match_any_sync(0xffffffffu, c);
      const int rank = __popc(same & ((1u << lane) - 1u));
      int slot = 0;
      if (ok) slot = cnt[c] + rank;
      __syncwarp();
      if (ok) {
        f.t_colind[slot] = r;
        f.t_val[slot] = f.val[p];
        if ((same >> lane) == 1u) cnt[c] = slot + 1;
      }
      __syncwarp();
    }
  }
  __syncthreads();
  return true;
}

// ------------------------------------------------------------------ one instance
// S = S_0 ... S_{J-1} as a dense block: the last factor's dense image, then
// the factors applied right to left (update_lambda's product without a
// packed operand).  Returns the buffer holding S.
template <typename T>
__device__ T* b_full_product(const Fac<T>* S, int J, T* const buf[2], int acols, Stage<T>& sg) {
  int cur = 0;
  b_csr_to_dense(S[J - 1], buf[cur]);
  for (int l = J - 2; l >= 0; --l) {
    b_spmm<T>(S[l].rowptr, S[l].colind, S[l].val, S[l].rows, S[l].cols, buf[cur], S[l].cols, acols, buf[cur ^ 1],
              E_STORE, nullptr, T(0), sg);
    cur ^= 1;
  }
  return buf[cur];
}

// <A, S> and ||S||_F^2 over N entries in the canonical order (256 lanes per
// chunk of 65536 entries, lane trees, chunk partials in order).
template <typename T>
__device__ void b_tr_ss(const T* A, const T* Smat, long N, T* lane, T& tr, T& ss) {
  tr = T(0);
  ss = T(0);
  for (long c0 = 0; c0 < N; c0 += CR_CHUNK) {
    const long c1 = min(N, c0 + CR_CHUNK);
    T a = T(0), s2 = T(0);
    for (long i = c0 + threadIdx.x; i < c1; i += CR_LANES) {
      a = fmad(A[i], Smat[i], a);
      s2 = fmad(Smat[i], Smat[i], s2);
    }
    lane[threadIdx.x] = a;
    tr = addr(tr, bat_tree(lane));
    lane[threadIdx.x] = s2;
    ss = addr(ss, bat_tree(lane));
  }
}

template <typename T, typename TN>
__device__ void run_instance(Inst<T>& I, const Slot<T>& W, const Params& P, const TN* x0, TN* vbuf, int maxn,
                             T* lane, TN* lane_n, Stage<T> sg) {
  const int J = I.J;
  Fac<T>* S = I.f;
  const bool r2l = P.r2l != 0;
  __shared__ int st;
  __shared__ T sh_c, sh_alpha;
  if (threadIdx.x == 0) st = 0;
  __syncthreads();
  T lam = (T)I.lambda;
  T* packed[MAXJ];
  for (int i = 0; i < J; ++i) packed[i] = W.packed + (long)i * P.maxdim2;
  T* buf[2] = {W.buf0, W.buf1};
  const int arows = I.arows, acols = I.acols;
  if (P.lambda_from_init) {
    // lambda = <A, S> / ||S||_F^2 of the seeded factors; an empty or NaN
    // product keeps the given lambda
    T tr, ss;
    b_tr_ss(I.A, b_full_product(S, J, buf, acols, sg), (long)arows * acols, lane, tr, ss);
    if (threadIdx.x == 0) {
      sh_c = sqrtr(ss);
      sh_alpha = (sh_c == T(0) || isnan(tr) || isnan(sh_c)) ? lam : divr(tr, mulr(sh_c, sh_c));
    }
    __syncthreads();
    lam = sh_alpha;
    __syncthreads();
  }
  for (int it = 0; it < P.nb_it; ++it) {
    // init_ite
    if (J >= 2) {
      if (!r2l) {
        b_csr_to_dense(S[J - 1], packed[J - 2]);
        for (int i = J - 3; i >= 0; --i)
          b_spmm<T>(S[i + 1].rowptr, S[i + 1].colind, S[i + 1].val, S[i + 1].rows, S[i + 1].cols, packed[i + 1], S[i + 1].cols, acols, packed[i], E_STORE, nullptr, T(0), sg);
      } else {
        b_csr_to_dense(S[0], packed[1]);
        for (int i = 2; i < J; ++i)
          b_dense_csrT<T>(packed[i - 1], arows, S[i - 1].rows, S[i - 1].t_rowptr, S[i - 1].t_colind, S[i - 1].t_val, S[i - 1].cols, packed[i], E_STORE, nullptr, T(0), sg);
      }
    }
    for (int step = 0; step < J; ++step) {
      const int f = r2l ? J - 1 - step : step;
      const Fac<T>& Sf = S[f];
      // step size (faust_palm4msa2020.hpp:563-617)
      T c;
      if (P.constant_step) {
        c = divr(T(1), (T)P.step_size);
      } else {
        const double nR = b_spectral_norm<T, TN>(S, f + 1, J, P.norm2_max_iter, (TN)P.norm2_threshold, x0, vbuf,
                                                 maxn, lane_n, &st);
        const double nL = b_spectral_norm<T, TN>(S, 0, f, P.norm2_max_iter, (TN)P.norm2_threshold, x0, vbuf, maxn,
                                                 lane_n, &st);
        __syncthreads();
        if (threadIdx.x == 0) {
          if (isnan(nR) || isnan(nL)) st = st ? st : FGB_ERR_NAN;
          if ((nR == 0.0 && (it > 0 || !r2l)) || (nL == 0.0 && (it > 0 || r2l))) st = st ? st : FGB_ERR_ZERO_NORM;
        }
        if (threadIdx.x == 0) {
          const double tnR = (double)(T)nR, tnL = (double)(T)nL, l = (double)lam;
          double cc = __dmul_rn(1.001, l);
          cc = __dmul_rn(cc, l);
          cc = __dmul_rn(cc, tnR);
          cc = __dmul_rn(cc, tnR);
          cc = __dmul_rn(cc, tnL);
          cc = __dmul_rn(cc, tnL);
          sh_c = (T)cc;
        }
        __syncthreads();
        c = sh_c;
      }
      if (threadIdx.x == 0) sh_alpha = divr(lam, c);
      __syncthreads();
      const T alpha = sh_alpha;
      __syncthreads();
      if (st) break;
      b_csr_to_dense(Sf, W.D);
      const bool hasL = f > 0, hasR = f + 1 < J;
      int cur = 0;
      if (!r2l) {
        if (hasR)
          b_spmm<T>(Sf.rowptr, Sf.colind, Sf.val, Sf.rows, Sf.cols, packed[f], Sf.cols, acols, buf[cur], f == 0 ? E_LAMBDA : E_STORE, I.A, lam, sg);
        else if (f == 0) {
          for (long i = threadIdx.x; i < (long)arows * acols; i += BT) buf[cur][i] = subr(mulr(lam, W.D[i]), I.A[i]);
          __syncthreads();
        } else {
          b_csr_to_dense(Sf, buf[cur]);
        }
        for (int l = f - 1; l >= 0; --l) {
          b_spmm<T>(S[l].rowptr, S[l].colind, S[l].val, S[l].rows, S[l].cols, buf[cur], S[l].cols, acols, buf[cur ^ 1], l == 0 ? E_LAMBDA : E_STORE, I.A, lam, sg);
          cur ^= 1;
        }
      } else {
        const int nR = J - 1 - f;
        if (hasL)
          b_dense_csrT<T>(packed[f], arows, Sf.rows, Sf.t_rowptr, Sf.t_colind, Sf.t_val, Sf.cols, buf[cur], nR == 0 ? E_LAMBDA : E_STORE, I.A, lam, sg);
        else if (nR == 0) {
          for (long i = threadIdx.x; i < (long)arows * acols; i += BT) buf[cur][i] = subr(mulr(lam, W.D[i]), I.A[i]);
          __syncthreads();
        } else {
          b_csr_to_dense(Sf, buf[cur]);
        }
        for (int l = f + 1; l < J; ++l) {
          b_dense_csrT<T>(buf[cur], arows, S[l].rows, S[l].t_rowptr, S[l].t_colind, S[l].t_val, S[l].cols, buf[cur ^ 1], l == J - 1 ? E_LAMBDA : E_STORE, I.A, lam, sg);
          cur ^= 1;
        }
      }
      // G = L^H E R^H with D - alpha G fused into the last product
      int rows = arows, cols = acols;
      const int nops = (J - 1 - f) + f;
      if (nops == 0) {
        for (long i = threadIdx.x; i < (long)Sf.rows * Sf.cols; i += BT)
          W.D[i] = subr(W.D[i], mulr(alpha, buf[cur][i]));
        __syncthreads();
      } else {
        int q = 0;
        auto left = [&](int l) {
          const bool last = ++q == nops;
          T* dst = last ? W.D : buf[cur ^ 1];
          b_spmm<T>(S[l].t_rowptr, S[l].t_colind, S[l].t_val, S[l].cols, S[l].rows, buf[cur], S[l].rows, cols, dst, last ? E_DMINUS : E_STORE, W.D, alpha, sg);
          rows = S[l].cols;
          if (!last) cur ^= 1;
        };
        auto right = [&](int l) {
          const bool last = ++q == nops;
          T* dst = last ? W.D : buf[cur ^ 1];
          b_dense_csrT<T>(buf[cur], rows, S[l].cols, S[l].rowptr, S[l].colind, S[l].val, S[l].rows, dst, last ? E_DMINUS : E_STORE, W.D, alpha, sg);
          cols = S[l].rows;
          if (!last) cur ^= 1;
        };
        if (!r2l) {
          for (int l = 0; l < f; ++l) left(l);
          for (int l = J - 1; l > f; --l) right(l);
        } else {
          for (int l = J - 1; l > f; --l) right(l);
          for (int l = 0; l < f; ++l) left(l);
        }
      }
      if (!b_project<T>(I.c[f], W.D, Sf.rows, Sf.cols, W.flags, lane, &st, sg)) break;
      if (!b_dense_to_csr<T>(W.D, S[f], W.cnt, &st)) break;
    }
    __syncthreads();
    if (st) break;
    if (!P.no_lambda) {
      // update_lambda: S_mat per the reuse rule (faust_palm4msa2020.hpp:449-468)
      T* Smat;
      const bool reuse = P.packing_RL || J <= 2;
      bool use_pR0 = false;
      if (J >= 2 && reuse) {
        const long lhs = (long)S[0].cols * S[1].rows;
        const long rhs = (long)S[J - 2].cols * S[J - 1].rows;
        use_pR0 = lhs < rhs;
      }
      if (J == 1) {
        b_csr_to_dense(S[0], buf[0]);
        Smat = buf[0];
      } else if (reuse && !r2l && use_pR0) {
        b_spmm<T>(S[0].rowptr, S[0].colind, S[0].val, S[0].rows, S[0].cols, packed[0], S[0].cols, acols, buf[0], E_STORE, nullptr, T(0), sg);
        Smat = buf[0];
      } else if (reuse && r2l && !use_pR0) {
        b_dense_csrT<T>(packed[J - 1], arows, S[J - 1].rows, S[J - 1].t_rowptr, S[J - 1].t_colind, S[J - 1].t_val, S[J - 1].cols, buf[0], E_STORE, nullptr, T(0), sg);
        Smat = buf[0];
      } else {
        Smat = b_full_product(S, J, buf, acols, sg);
      }
      T tr, ss;
      b_tr_ss(I.A, Smat, (long)arows * acols, lane, tr, ss);
      if (threadIdx.x == 0) {
        sh_c = sqrtr(ss);
        sh_alpha = (sh_c == T(0) || isnan(tr) || isnan(sh_c)) ? T(0) : divr(tr, mulr(sh_c, sh_c));
      }
      __syncthreads();
      const T nS = sh_c;
      const T lam_new = sh_alpha;
      __syncthreads();
      if (nS == T(0)) {
        if (!P.no_lambda_error) {
          if (threadIdx.x == 0) st = FGB_ERR_ZERO_NORM;
          break;
        }
      } else if (isnan(tr) || isnan(nS)) {
        if (!P.no_lambda_error) {
          if (threadIdx.x == 0) st = FGB_ERR_NAN;
          break;
        }
      } else {
        lam = lam_new;
      }
    }
    __syncthreads();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    I.status = st;
    I.lambda = (double)lam;
    for (int f = 0; f < J; ++f) I.nnz[f] = S[f].rowptr[S[f].rows];
  }
}

// MINB: resident CTAs per SM the register budget is cut for (2: up to 128
// registers a thread; 3: up to 80, with some spilling) -- the tuned table
// picks the CTAs per SM, and with it the variant.
template <typename T, typename TN, int MINB>
__global__ void __launch_bounds__(BT, MINB) k_palm_batched(Inst<T>* insts, const int* order, int* queue, Slot<T>* slots,
                                                        const __grid_constant__ Params P, const TN* x0, int maxn) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TN* vbuf = reinterpret_cast<TN*>(smem_raw);  // 3 * maxn
  TN* lane_n = vbuf + 3 * (long)maxn;
  // staging area 16-byte aligned after the vectors
  const size_t sg_off = ((3 * (size_t)maxn + BT) * sizeof(TN) + 15) & ~(size_t)15;
  Stage<T> sg{reinterpret_cast<T*>(smem_raw + sg_off), P.stage_elems};
  __shared__ T lane[BT];
  __shared__ int next;
  const Slot<T> W = slots[blockIdx.x];
  while (true) {
    if (threadIdx.x == 0) next = atomicAdd(queue, 1);
    __syncthreads();
    const int q = next;
    __syncthreads();
    if (q >= P.ninst) break;
    const long long c0 = clock64();
    run_instance<T, TN>(insts[order[q]], W, P, x0, vbuf, maxn, lane, lane_n, sg);
    if (threadIdx.x == 0) insts[order[q]].cycles = clock64() - c0;
  }
}

// Writes the seeded factor values: thread (i, q) stores
// scale * vals[i * V + q] at entry pos[q] of factor fac[q] of instance i and
// at slot tpos[q] of that factor's transpose.
template <typename T>
__global__ void k_seed_values(Inst<T>* insts, int ninst, int V, const T* __restrict__ vals, double scale,
                              const int* __restrict__ fac, const int* __restrict__ pos,
                              const int* __restrict__ tpos) {
  const long total = (long)ninst * V;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const int i = (int)(t / V), q = (int)(t % V);
    const T v = (T)(scale * (double)vals[t]);
    Fac<T>& F = insts[i].f[fac[q]];
    F.val[pos[q]] = v;
    F.t_val[tpos[q]] = v;
  }
}

}  // namespace bat

// ------------------------------------------------------------------ host driver
void free_factor(DevFactor& f);
long palm_factor_capacity(const fgb_constraint& c);
fgb_status pi_rand_device(fgb_ctx* ctx, int n, const int** d_rand);

template <typename T>
static fgb_status batched_impl(fgb_ctx* ctx, fgb_dtype dt, int nprob, const fgb_palm_problem* probs,
                               const fgb_palm_params* p, const fgb_batch_opts* opts, fgb_palm_result* res) {
  using namespace bat;
  if (nprob <= 0 || !probs || !p || !res) return fail(ctx, FGB_ERR_INVALID_ARG, "batched palm4msa2: bad arguments");
  int maxdim = 1, maxJ = 0;
  for (int i = 0; i < nprob; ++i) {
    const fgb_palm_problem& q = probs[i];
    if (q.nfacts <= 0 || q.nfacts > MAXJ) return fail(ctx, FGB_ERR_INVALID_ARG, "instance %d: 1..%d factors", i, MAXJ);
    if (!q.A || !q.cons) return fail(ctx, FGB_ERR_INVALID_ARG, "instance %d: null A or constraints", i);
    if (q.cons[0].rows != q.rows || q.cons[q.nfacts - 1].cols != q.cols)
      return fail(ctx, FGB_ERR_INVALID_ARG, "instance %d: constraint shapes do not match A", i);
    for (int f = 0; f < q.nfacts; ++f) {
      const fgb_constraint& c = q.cons[f];
      if (f > 0 && q.cons[f - 1].cols != c.rows)
        return fail(ctx, FGB_ERR_INVALID_ARG, "instance %d: factor %d shape mismatch", i, f);
      const bool line = c.kind == FGB_SPCOL || c.kind == FGB_SPLIN || c.kind == FGB_SPLINCOL;
      if (!(line || c.kind == FGB_NORMCOL || c.kind == FGB_NORMLIN || c.kind == FGB_SUPP))
        return fail(ctx, FGB_ERR_NOT_SUPPORTED, "batched palm4msa2: constraint kind %d not supported", c.kind);
      if (line && c.k > KMAX && c.k < std::max(c.rows, c.cols))
        return fail(ctx, FGB_ERR_NOT_SUPPORTED, "batched palm4msa2: per-line k <= %d", KMAX);
      if (c.kind == FGB_SUPP && !c.supp) return fail(ctx, FGB_ERR_INVALID_ARG, "SUPP without support");
      if ((c.kind == FGB_NORMCOL || c.kind == FGB_NORMLIN) && c.s < 0)
        return fail(ctx, FGB_ERR_INVALID_ARG, "Faust::prox_normcol : s < 0 ");
      maxdim = std::max(maxdim, std::max(c.rows, c.cols));
    }
    maxJ = std::max(maxJ, q.nfacts);
  }
  if (p->norm2_max_iter <= 0 && !p->constant_step_size)
    return fail(ctx, FGB_ERR_INVALID_ARG, "power_iteration :  nbr_iter_max <= 0");
  FGB_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t es = sizeof(T);
  const long md2 = (long)maxdim * maxdim;
  // slots (one device block for all of them)
  int per_sm = opts && opts->ctas_per_sm > 0 ? std::min(opts->ctas_per_sm, 3) : 2;
  int nslots = std::min(nprob, per_sm * ctx->sm_count);
  std::vector<void*> allocs;
  auto alloc = [&](void** q, size_t b) -> fgb_status {
    fgb_status s = dmalloc(ctx, q, b);
    if (s == FGB_OK) allocs.push_back(*q);
    return s;
  };
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  fgb_status s = FGB_OK;
  std::vector<Slot<T>> hs(nslots);
  {
    const size_t dense = al(es * md2);
    const size_t slot_bytes = 3 * dense + al(es * md2 * std::max(1, maxJ)) + al((size_t)md2) +
                              al(sizeof(int) * (maxdim + 2));
    unsigned char* base = nullptr;
    s = alloc((void**)&base, slot_bytes * nslots);
    for (int i = 0; i < nslots && s == FGB_OK; ++i) {
      unsigned char* q = base + slot_bytes * i;
      hs[i].D = reinterpret_cast<T*>(q);
      q += dense;
      hs[i].buf0 = reinterpret_cast<T*>(q);
      q += dense;
      hs[i].buf1 = reinterpret_cast<T*>(q);
      q += dense;
      hs[i].packed = reinterpret_cast<T*>(q);
      q += al(es * md2 * std::max(1, maxJ));
      hs[i].flags = q;
      q += al((size_t)md2);
      hs[i].cnt = reinterpret_cast<int*>(q);
    }
    // the projections expect cleared flags
    if (s == FGB_OK) s = cuda_check(ctx, cudaMemsetAsync(base, 0, slot_bytes * nslots, ctx->stream), "memset");
  }
  // instances and their factors: every factor array of every instance in one
  // device block, filled from one host image with a single copy
  std::vector<Inst<T>> hi(nprob);
  std::vector<std::vector<DevFactor>> facs(nprob);
  std::vector<std::pair<const void*, T*>> supp_cache;
  std::vector<std::pair<double, int>> cost(nprob);
  // host CSR (and transpose) of every initial factor: the given dense
  // matrix, or palm4msa2's default (zeros for the first factor updated,
  // identity for the others)
  struct HostCSR {
    std::vector<int> rp, ci, trp, tci;
    std::vector<T> vv, tvv;
    long cap = 0;
    size_t off = 0;
  };
  std::vector<std::vector<HostCSR>> hc(nprob);
  // Seeding from device values: every instance shares the structure of the
  // SUPP supports (stored entries = the support, values written on the
  // device by k_seed_values), built once from the first problem.
  const bool seed = opts && opts->init_values;
  std::vector<HostCSR> seed_csr;
  std::vector<int> seed_fac, seed_pos, seed_tpos;
  if (seed) {
    const fgb_palm_problem& q0 = probs[0];
    for (int i = 1; i < nprob; ++i) {
      if (probs[i].nfacts != q0.nfacts)
        return fail(ctx, FGB_ERR_INVALID_ARG, "seeded batch: instance %d has another factor count", i);
      for (int f = 0; f < q0.nfacts; ++f) {
        const fgb_constraint &a = probs[i].cons[f], &b = q0.cons[f];
        if (a.kind != FGB_SUPP || a.supp != b.supp || a.rows != b.rows || a.cols != b.cols)
          return fail(ctx, FGB_ERR_INVALID_ARG, "seeded batch: instance %d factor %d differs from instance 0's "
                      "SUPP constraint", i, f);
      }
    }
    seed_csr.resize(q0.nfacts);
    for (int f = 0; f < q0.nfacts; ++f) {
      const fgb_constraint& c = q0.cons[f];
      if (c.kind != FGB_SUPP) return fail(ctx, FGB_ERR_INVALID_ARG, "seeded batch: SUPP constraints only");
      HostCSR& H = seed_csr[f];
      const T* d = (const T*)c.supp;
      H.rp.assign(c.rows + 1, 0);
      for (int r = 0; r < c.rows; ++r) {
        for (int col = 0; col < c.cols; ++col)
          if (d[(size_t)col * c.rows + r] != T(0)) {
            H.ci.push_back(col);
            H.vv.push_back(T(0));
          }
        H.rp[r + 1] = (int)H.ci.size();
      }
      H.trp.assign(c.cols + 1, 0);
      H.tci.resize(H.ci.size());
      H.tvv.assign(H.ci.size(), T(0));
      for (int col : H.ci) H.trp[col + 1]++;
      for (int col = 0; col < c.cols; ++col) H.trp[col + 1] += H.trp[col];
      std::vector<int> fill(H.trp.begin(), H.trp.end() - 1);
      for (int r = 0; r < c.rows; ++r)
        for (int pp = H.rp[r]; pp < H.rp[r + 1]; ++pp) {
          const int slot = fill[H.ci[pp]]++;
          H.tci[slot] = r;
          seed_fac.push_back(f);
          seed_pos.push_back(pp);
          seed_tpos.push_back(slot);
        }
    }
    if ((long)seed_fac.size() != (long)opts->values_per_instance)
      return fail(ctx, FGB_ERR_INVALID_ARG, "seeded batch: %d values per instance given, the supports hold %zu",
                  opts->values_per_instance, seed_fac.size());
  }
  size_t pool_bytes = 0;
  for (int i = 0; i < nprob; ++i) {
    const fgb_palm_problem& q = probs[i];
    hc[i].resize(q.nfacts);
    for (int f = 0; f < q.nfacts; ++f) {
      const fgb_constraint& c = q.cons[f];
      HostCSR& H = hc[i][f];
      if (seed) {
        H = seed_csr[f];
        H.cap = std::max<long>(palm_factor_capacity(c), (long)H.ci.size());
        H.off = pool_bytes;
        pool_bytes += al(sizeof(int) * (c.rows + 1)) + al(sizeof(int) * (c.cols + 1)) + 2 * al(sizeof(int) * H.cap) +
                      2 * al(es * H.cap);
        continue;
      }
      H.rp.assign(c.rows + 1, 0);
      if (q.init_facts) {
        const T* d = (const T*)q.init_facts[f];
        for (int r = 0; r < c.rows; ++r) {
          for (int col = 0; col < c.cols; ++col) {
            const T v = d[(size_t)col * c.rows + r];
            if (v != T(0)) {
              H.ci.push_back(col);
              H.vv.push_back(v);
            }
          }
          H.rp[r + 1] = (int)H.ci.size();
        }
      } else {
        const bool zero = p->is_update_way_R2L ? (f == q.nfacts - 1) : (f == 0);
        for (int r = 0; r < c.rows; ++r) {
          if (!zero && r < c.cols) {
            H.ci.push_back(r);
            H.vv.push_back(T(1));
          }
          H.rp[r + 1] = (int)H.ci.size();
        }
      }
      H.trp.assign(c.cols + 1, 0);
      H.tci.resize(H.ci.size());
      H.tvv.resize(H.ci.size());
      for (int col : H.ci) H.trp[col + 1]++;
      for (int col = 0; col < c.cols; ++col) H.trp[col + 1] += H.trp[col];
      std::vector<int> fill(H.trp.begin(), H.trp.end() - 1);
      for (int r = 0; r < c.rows; ++r)
        for (int pp = H.rp[r]; pp < H.rp[r + 1]; ++pp) {
          const int slot = fill[H.ci[pp]]++;
          H.tci[slot] = r;
          H.tvv[slot] = H.vv[pp];
        }
      H.cap = std::max<long>(palm_factor_capacity(c), (long)H.ci.size());
      H.off = pool_bytes;
      pool_bytes += al(sizeof(int) * (c.rows + 1)) + al(sizeof(int) * (c.cols + 1)) + 2 * al(sizeof(int) * H.cap) +
                    2 * al(es * H.cap);
    }
  }
  unsigned char* pool = nullptr;
  if (s == FGB_OK) s = dmalloc(ctx, (void**)&pool, std::max<size_t>(pool_bytes, 256));
  std::shared_ptr<void> pool_owner;
  if (s == FGB_OK) pool_owner = std::shared_ptr<void>(pool, [](void* q) { dfree(q); });
  std::vector<unsigned char> img(pool_bytes, 0);
  for (int i = 0; i < nprob && s == FGB_OK; ++i) {
    const fgb_palm_problem& q = probs[i];
    Inst<T>& I = hi[i];
    std::memset(&I, 0, sizeof(I));
    I.J = q.nfacts;
    I.arows = q.rows;
    I.acols = q.cols;
    I.A = (const T*)q.A;
    I.lambda = q.init_lambda;
    facs[i].resize(q.nfacts);
    double cst = 0;
    for (int f = 0; f < q.nfacts && s == FGB_OK; ++f) {
      const fgb_constraint& c = q.cons[f];
      HostCSR& H = hc[i][f];
      DevFactor& F = facs[i][f];
      F.format = FGB_CSR;
      F.rows = c.rows;
      F.cols = c.cols;
      F.cap = (int)H.cap;
      F.nnz = (int)H.ci.size();
      const long cap = H.cap;
      const std::vector<int>&rp = H.rp, &ci = H.ci, &trp = H.trp, &tci = H.tci;
      const std::vector<T>&vv = H.vv, &tvv = H.tvv;
      // carve the pool and write the host image
      size_t o = H.off;
      auto place = [&](const void* src, size_t bytes, size_t room) {
        if (bytes) std::memcpy(img.data() + o, src, bytes);
        void* d = pool + o;
        o += al(room);
        return d;
      };
      F.rowptr = (int*)place(rp.data(), sizeof(int) * rp.size(), sizeof(int) * (c.rows + 1));
      F.t_rowptr = (int*)place(trp.data(), sizeof(int) * trp.size(), sizeof(int) * (c.cols + 1));
      F.colind = (int*)place(ci.data(), sizeof(int) * ci.size(), sizeof(int) * cap);
      F.t_colind = (int*)place(tci.data(), sizeof(int) * tci.size(), sizeof(int) * cap);
      F.val = place(vv.data(), es * vv.size(), es * cap);
      F.t_val = place(tvv.data(), es * tvv.size(), es * cap);
      F.has_t = true;
      I.f[f] = Fac<T>{F.rows, F.cols, F.cap, 0, F.rowptr, F.colind, (T*)F.val, F.t_rowptr, F.t_colind, (T*)F.t_val};
      Cons<T>& C = I.c[f];
      C.kind = c.kind;
      C.k = (int)std::min<long long>(c.k, 1 << 30);
      C.normalized = p->no_normalization ? 0 : c.normalized;
      C.pos = c.pos;
      C.s = c.s;
      C.supp = nullptr;
      if (c.kind == FGB_SUPP) {
        T* d = nullptr;
        for (auto& e : supp_cache)
          if (e.first == c.supp) d = e.second;
        if (!d) {
          s = alloc((void**)&d, es * (size_t)c.rows * c.cols);
          if (s != FGB_OK) break;
          cudaMemcpy(d, c.supp, es * (size_t)c.rows * c.cols, cudaMemcpyHostToDevice);
          supp_cache.push_back({c.supp, d});
        }
        C.supp = d;
      }
      cst += (double)c.rows * c.cols;
    }
    cost[i] = {-(cst * q.nfacts), i};
  }
  if (s == FGB_OK && pool_bytes)
    s = cuda_check(ctx, cudaMemcpy(pool, img.data(), pool_bytes, cudaMemcpyHostToDevice), "batched upload");
  if (s == FGB_OK) s = cuda_check(ctx, cudaGetLastError(), "batched upload");
  Inst<T>* d_inst = nullptr;
  Slot<T>* d_slots = nullptr;
  int* d_order = nullptr;
  int* d_queue = nullptr;
  const int* rnd = nullptr;
  if (s == FGB_OK) s = alloc((void**)&d_inst, sizeof(Inst<T>) * nprob);
  if (s == FGB_OK) s = alloc((void**)&d_slots, sizeof(Slot<T>) * nslots);
  if (s == FGB_OK) s = alloc((void**)&d_order, sizeof(int) * nprob);
  if (s == FGB_OK) s = alloc((void**)&d_queue, sizeof(int));
  if (s == FGB_OK) s = pi_rand_device(ctx, maxdim, &rnd);
  if (s == FGB_OK) {
    std::sort(cost.begin(), cost.end());
    std::vector<int> order(nprob);
    for (int i = 0; i < nprob; ++i) order[i] = cost[i].second;
    cudaMemcpy(d_inst, hi.data(), sizeof(Inst<T>) * nprob, cudaMemcpyHostToDevice);
    cudaMemcpy(d_slots, hs.data(), sizeof(Slot<T>) * nslots, cudaMemcpyHostToDevice);
    cudaMemcpy(d_order, order.data(), sizeof(int) * nprob, cudaMemcpyHostToDevice);
    s = cuda_check(ctx, cudaGetLastError(), "batched upload");
  }
  int* d_seed = nullptr;
  const int V = seed ? opts->values_per_instance : 0;
  if (s == FGB_OK && seed) {
    s = alloc((void**)&d_seed, sizeof(int) * 3 * (size_t)V);
    if (s == FGB_OK) {
      std::vector<int> tab;
      tab.reserve(3 * (size_t)V);
      tab.insert(tab.end(), seed_fac.begin(), seed_fac.end());
      tab.insert(tab.end(), seed_pos.begin(), seed_pos.end());
      tab.insert(tab.end(), seed_tpos.begin(), seed_tpos.end());
      s = cuda_check(ctx, cudaMemcpy(d_seed, tab.data(), sizeof(int) * tab.size(), cudaMemcpyHostToDevice), "seed");
    }
  }
  if (s == FGB_OK) {
    Params P;
    std::memset(&P, 0, sizeof(P));
    P.nb_it = p->nb_it;
    P.r2l = p->is_update_way_R2L;
    P.packing_RL = p->packing_RL;
    P.no_lambda = p->no_lambda;
    P.norm2_max_iter = p->norm2_max_iter;
    P.constant_step = p->constant_step_size;
    P.no_lambda_error = p->no_lambda_error;
    P.norm2_fp64 = p->norm2_fp64;
    P.norm2_threshold = p->norm2_threshold;
    P.step_size = p->step_size;
    P.maxdim2 = md2;
    P.ninst = nprob;
    P.lambda_from_init = opts ? opts->lambda_from_init : 0;
    const bool fp64n = sizeof(T) == 8 || p->norm2_fp64;
    // power-iteration vectors, their reduction lanes, then the staging area
    // of the block products (a share of the SM's shared memory per CTA)
    const size_t vec_bytes = ((3 * (size_t)maxdim + BT) * (fp64n ? 8 : 4) + 15) & ~(size_t)15;
    const size_t per_cta = std::min<size_t>(ctx->smem_optin ? ctx->smem_optin : 227 * 1024,
                                            (size_t)(228 * 1024) / per_sm - 2048);
    const size_t stage_bytes = per_cta > vec_bytes + 8192 + 4096 ? per_cta - vec_bytes - 8192 : 4096;
    P.stage_elems = (int)std::min<size_t>(stage_bytes / es, std::max<size_t>((size_t)md2, 4 * (16 / es) * (size_t)maxdim));
    // the block products need 2 * G * maxdim entries of the staging area
    // after a factor's CSR (which takes at most half of it); G = 16 / sizeof(T)
    if ((size_t)P.stage_elems < 4 * (16 / es) * (size_t)maxdim)
      s = fail(ctx, FGB_ERR_NOT_SUPPORTED, "batched palm4msa2: dimension %d too large for %d CTAs per SM", maxdim,
               per_sm);
    const size_t smem = vec_bytes + (size_t)P.stage_elems * es;
    const bool three = per_sm >= 3;
    auto kern_d = three ? k_palm_batched<T, double, 3> : k_palm_batched<T, double, 2>;
    auto kern_f = three ? k_palm_batched<T, float, 3> : k_palm_batched<T, float, 2>;
    if (s == FGB_OK) s = smem_opt_in(ctx, fp64n ? (const void*)kern_d : (const void*)kern_f, smem);
    // The launch sequence: queue reset, seeding (when asked), the persistent
    // kernel, captured as one CUDA graph and launched as a unit.  It runs on
    // the context's stream, or on a private stream when the context uses the
    // legacy default stream (which cannot be captured; the uploads above are
    // synchronous, so nothing of the caller's is pending).  The call reads
    // its results back, so a stream that is being captured is refused.
    cudaStream_t ls = ctx->stream, priv = nullptr;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (s == FGB_OK && ls) s = cuda_check(ctx, cudaStreamIsCapturing(ls, &cap), "capture status");
    if (s == FGB_OK && cap != cudaStreamCaptureStatusNone)
      s = fail(ctx, FGB_ERR_NOT_SUPPORTED, "batched palm4msa2 reads its results back: not inside a stream capture");
    if (s == FGB_OK && !ls) {
      s = cuda_check(ctx, cudaStreamCreateWithFlags(&priv, cudaStreamNonBlocking), "stream");
      ls = priv;
    }
    auto enqueue = [&]() -> cudaError_t {
      cudaError_t e = cudaMemsetAsync(d_queue, 0, sizeof(int), ls);
      if (e != cudaSuccess) return e;
      if (seed) {
        const long total = (long)nprob * V;
        const int grid = (int)std::min<long>((total + 255) / 256, 8L * ctx->sm_count);
        k_seed_values<T><<<grid, 256, 0, ls>>>(d_inst, nprob, V, (const T*)opts->init_values,
                                               opts->init_values_scale, d_seed, d_seed + V, d_seed + 2 * V);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
      }
      if (fp64n)
        kern_d<<<nslots, BT, smem, ls>>>(d_inst, d_order, d_queue, d_slots, P, ctx->x0_d, maxdim);
      else
        kern_f<<<nslots, BT, smem, ls>>>(d_inst, d_order, d_queue, d_slots, P, ctx->x0_f, maxdim);
      return cudaGetLastError();
    };
    if (s == FGB_OK) {
      cudaGraph_t graph = nullptr;
      cudaGraphExec_t exec = nullptr;
      cudaError_t e = cudaStreamBeginCapture(ls, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        const cudaError_t e1 = enqueue();
        e = cudaStreamEndCapture(ls, &graph);
        if (e == cudaSuccess) e = e1;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
      if (e == cudaSuccess) e = cudaGraphLaunch(exec, ls);
      if (e == cudaSuccess) e = cudaStreamSynchronize(ls);
      if (exec) cudaGraphExecDestroy(exec);
      if (graph) cudaGraphDestroy(graph);
      s = cuda_check(ctx, e, "batched palm graph");
      if (s == FGB_OK) ctx->launches.fetch_add(seed ? 2 : 1);
    }
    if (priv) cudaStreamDestroy(priv);
  }
  if (s == FGB_OK) {
    cudaMemcpy(hi.data(), d_inst, sizeof(Inst<T>) * nprob, cudaMemcpyDeviceToHost);
    for (int i = 0; i < nprob; ++i) {
      res[i].lambda = hi[i].lambda;
      res[i].status = hi[i].status;
      res[i].cycles = hi[i].cycles;
      fgb_faust* F = new fgb_faust();
      F->ctx = ctx;
      F->dtype = dt;
      F->f = facs[i];
      F->pool = pool_owner;
      for (int f = 0; f < (int)F->f.size(); ++f) F->f[f].nnz = hi[i].nnz[f];
      facs[i].clear();
      res[i].faust = F;
    }
  }
  // factors not handed out are views into the pool (released with its owner)
  facs.clear();
  for (void* q : allocs) dfree(q);
  return s;
}

}  // namespace fgb

using namespace fgb;

extern "C" fgb_status fgb_palm4msa2_batched(fgb_ctx* ctx, fgb_dtype dtype, int nprob, const fgb_palm_problem* probs,
                                            const fgb_palm_params* params, const fgb_batch_opts* opts,
                                            fgb_palm_result* results) {
  if (!ctx) return FGB_ERR_INVALID_ARG;
  if (dtype == FGB_F32) return batched_impl<float>(ctx, dtype, nprob, probs, params, opts, results);
  if (dtype == FGB_F64) return batched_impl<double>(ctx, dtype, nprob, probs, params, opts, results);
  return fail(ctx, FGB_ERR_NOT_SUPPORTED, "batched palm4msa2: F32 or F64");
}
