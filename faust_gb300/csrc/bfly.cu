// bfly.cu — fused chain kernel for Fausts whose factors all have butterfly
// supports (faust_butterfly.hpp:459-492, butterfly_support): factor S of
// size n (a power of two) with stride h stores, in row r, the two entries at
// columns r & ~h and r | h (in that order).  Rows r and r ^ h read the same
// two inputs, so a thread that holds the 2^g rows spanned by g strides can
// apply up to g consecutive factors in registers and touch shared memory
// once per g factors instead of once per factor:
//
//   pass = up to G consecutive factors (application order) with at most G
//          distinct strides; orbit = base + any subset of those strides;
//   per pass every thread loads its orbits' rows of the column tile from
//   shared memory, applies the factors in registers, stores them back (or,
//   in the last pass, to Y); one block barrier per pass.
//
// Entry order is the library's canonical one: out[r] = fma(v1, x[r|h],
// fma(v0, x[r&~h], +0)) with (v0, v1) row r's stored values in order, so the
// result is bit-identical to the per-factor CSR product.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "csr.cuh"
#include "fgb_internal.cuh"

namespace fgb {

constexpr int BF_MAXS = 64;   // factors per chain
constexpr int BF_G = 3;       // largest number of strides per pass the plan holds
constexpr int BF_THREADS = 256;

struct BflyPlan {
  int n, nsteps, npasses;
  const void* val[BF_MAXS];   // step s (application order): 2 values per row
  int stride[BF_MAXS];
  int pass_first[BF_MAXS], pass_n[BF_MAXS], pass_g[BF_MAXS];
  int pass_bit[BF_MAXS][BF_G];  // orbit strides of the pass, ascending
};

template <typename T>
struct V2;
template <>
struct V2<float> {
  using type = float2;
};
template <>
struct V2<double> {
  using type = double2;
};

template <typename T, int TC>
__device__ __forceinline__ void ld_row(const T* p, T (&x)[TC]) {
  if constexpr (TC * sizeof(T) == 16) {
    if constexpr (sizeof(T) == 4) {
      const float4 v = *reinterpret_cast<const float4*>(p);
      x[0] = v.x, x[1] = v.y, x[2] = v.z, x[3] = v.w;
    } else {
      const double2 v = *reinterpret_cast<const double2*>(p);
      x[0] = v.x, x[1] = v.y;
    }
  } else {
#pragma unroll
    for (int t = 0; t < TC; ++t) x[t] = p[t];
  }
}

template <typename T, int TC>
__device__ __forceinline__ void st_row(T* p, const T (&x)[TC]) {
  if constexpr (TC * sizeof(T) == 16) {
    if constexpr (sizeof(T) == 4)
      *reinterpret_cast<float4*>(p) = make_float4(x[0], x[1], x[2], x[3]);
    else
      *reinterpret_cast<double2*>(p) = make_double2(x[0], x[1]);
  } else {
#pragma unroll
    for (int t = 0; t < TC; ++t) p[t] = x[t];
  }
}

// 16-byte row slot of matrix row r in the shared tile: the low three bits
// are XORed with higher ones so that the rows one warp touches in a pass
// (r = base + j * 2^b for consecutive orbit bases) fall in distinct bank
// groups whatever the pass strides are.
__device__ __forceinline__ int bf_slot(int r) { return r ^ (((r >> 3) ^ (r >> 6) ^ (r >> 9) ^ (r >> 12)) & 7); }

// Rows of orbit o in pass ps: o with a zero inserted at every orbit stride,
// plus every subset of the strides.
template <int G>
__device__ __forceinline__ void bf_rows(const BflyPlan& p, int ps, int o, int (&row)[1 << G]) {
  const int g = p.pass_g[ps];
  int bit[G];
#pragma unroll
  for (int b = 0; b < G; ++b) bit[b] = b < g ? p.pass_bit[ps][b] : 0;
  int base = o;
#pragma unroll
  for (int b = 0; b < G; ++b)
    if (b < g) base = ((base & ~(bit[b] - 1)) << 1) | (base & (bit[b] - 1));
#pragma unroll
  for (int k = 0; k < (1 << G); ++k) {
    int r = base;
#pragma unroll
    for (int b = 0; b < G; ++b)
      if ((k >> b) & 1) r += bit[b];
    row[k] = r;
  }
}

// The values of every factor of pass ps for the rows of one orbit.
template <typename T, int G>
__device__ __forceinline__ void bf_load_vals(const BflyPlan& p, int ps, const int (&row)[1 << G],
                                             typename V2<T>::type (&v)[G][1 << G]) {
  using T2 = typename V2<T>::type;
  const int g = p.pass_g[ps], ns = p.pass_n[ps], first = p.pass_first[ps];
#pragma unroll
  for (int s = 0; s < G; ++s) {
    const T2* vs = reinterpret_cast<const T2*>(p.val[first + (s < ns ? s : 0)]);
#pragma unroll
    for (int k = 0; k < (1 << G); ++k)
      if (s < ns && k < (1 << g)) v[s][k] = __ldg(vs + row[k]);
  }
}

// One block per column tile of TC columns; 256 threads.  Each thread walks
// its (pass, orbit) items in order and loads the values of its next item
// before working on the current one, so the L2 latency of the values
// overlaps the shared-memory work (also across the pass barrier: values do
// not depend on the tile).
template <typename T, int TC, int G>
__global__ void __launch_bounds__(BF_THREADS, sizeof(T) == 4 ? 3 : 2)
    k_bfly_chain(const __grid_constant__ BflyPlan p, const T* __restrict__ X, int ldx, int ncols, T* __restrict__ Y,
                 int ldy) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* tile = reinterpret_cast<T*>(smem_raw);  // n slots of TC values
  using T2 = typename V2<T>::type;
  const int n = p.n;
  const int j0 = blockIdx.x * TC;
  const int tid = threadIdx.x;
  // first item's values in flight while the tile is staged
  int nps = 0;
  while (nps < p.npasses && tid >= (n >> p.pass_g[nps])) ++nps;
  int nrow[1 << G];
  T2 vn[G][1 << G];
  if (nps < p.npasses) {
    bf_rows<G>(p, nps, tid, nrow);
    bf_load_vals<T, G>(p, nps, nrow, vn);
  }
  for (int r = tid; r < n; r += blockDim.x) {
    T x[TC];
#pragma unroll
    for (int t = 0; t < TC; ++t) x[t] = (j0 + t < ncols) ? X[r + (long)(j0 + t) * ldx] : T(0);
    st_row<T, TC>(tile + (long)bf_slot(r) * TC, x);
  }
  __syncthreads();
  for (int ps = 0; ps < p.npasses; ++ps) {
    const int g = p.pass_g[ps], first = p.pass_first[ps], ns = p.pass_n[ps];
    const bool last = ps + 1 == p.npasses;
    const int orbits = n >> g;
    int bit[G];
#pragma unroll
    for (int b = 0; b < G; ++b) bit[b] = b < g ? p.pass_bit[ps][b] : 0;
    for (int o = tid; o < orbits; o += blockDim.x) {
      int row[1 << G];
      T2 v[G][1 << G];
#pragma unroll
      for (int k = 0; k < (1 << G); ++k) row[k] = nrow[k];
#pragma unroll
      for (int s = 0; s < G; ++s)
#pragma unroll
        for (int k = 0; k < (1 << G); ++k) v[s][k] = vn[s][k];
      // next item: the next orbit of this pass, else the first of a later pass
      {
        int qo = o + blockDim.x, qp = ps;
        if (qo >= orbits) {
          qp = ps + 1;
          qo = tid;
          while (qp < p.npasses && tid >= (n >> p.pass_g[qp])) ++qp;
        }
        if (qp < p.npasses) {
          bf_rows<G>(p, qp, qo, nrow);
          bf_load_vals<T, G>(p, qp, nrow, vn);
        }
      }
      T xs[1 << G][TC];
#pragma unroll
      for (int k = 0; k < (1 << G); ++k)
        if (k < (1 << g)) ld_row<T, TC>(tile + (long)bf_slot(row[k]) * TC, xs[k]);
#pragma unroll
      for (int s = 0; s < G; ++s) {
        if (s >= ns) break;
        const int h = p.stride[first + s];
#pragma unroll
        for (int b = 0; b < G; ++b) {
          if (b >= g || bit[b] != h) continue;
#pragma unroll
          for (int k = 0; k < (1 << G); ++k) {
            if (((k >> b) & 1) || k >= (1 << g)) continue;
            const int k1 = k | (1 << b);
#pragma unroll
            for (int t = 0; t < TC; ++t) {
              const T a = xs[k][t], c = xs[k1][t];
              xs[k][t] = fmad(v[s][k].y, c, fmad(v[s][k].x, a, T(0)));
              xs[k1][t] = fmad(v[s][k1].y, c, fmad(v[s][k1].x, a, T(0)));
            }
          }
        }
      }
      if (last) {
#pragma unroll
        for (int k = 0; k < (1 << G); ++k) {
          if (k >= (1 << g)) continue;
#pragma unroll
          for (int t = 0; t < TC; ++t)
            if (j0 + t < ncols) Y[row[k] + (long)(j0 + t) * ldy] = xs[k][t];
        }
      } else {
#pragma unroll
        for (int k = 0; k < (1 << G); ++k)
          if (k < (1 << g)) st_row<T, TC>(tile + (long)bf_slot(row[k]) * TC, xs[k]);
      }
    }
    if (!last) __syncthreads();
  }
}

// ------------------------------------------------------------------ detection
// bad[q] = 1 unless factor q is a butterfly factor of stride h[q].
__global__ void k_bfly_detect(const int* __restrict__ rowptr, const int* __restrict__ colind, int n,
                              int* __restrict__ bad, int* __restrict__ hout) {
  const int h = colind[1] - colind[0];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *hout = h;
    if (h <= 0 || h >= n || (h & (h - 1)) || rowptr[n] != 2 * n) *bad = 1;
  }
  if (h <= 0 || h >= n) return;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    if (rowptr[r] != 2 * r || colind[2 * r] != (r & ~h) || colind[2 * r + 1] != (r | h)) *bad = 1;
  }
}

// Caches DevFactor::bfly (stride, or 0) for every factor of F.
static fgb_status bfly_detect(fgb_faust* F) {
  fgb_ctx* ctx = F->ctx;
  const int J = (int)F->f.size();
  bool need = false;
  for (auto& f : F->f) need = need || f.bfly < 0;
  if (!need) return FGB_OK;
  std::vector<int> cand(J, 0);
  int ncand = 0;
  for (int q = 0; q < J; ++q) {
    const DevFactor& f = F->f[q];
    const bool shape = f.format == FGB_CSR && f.rows == f.cols && f.rows >= 2 && (f.rows & (f.rows - 1)) == 0 &&
                       f.nnz == 2 * f.rows;
    cand[q] = shape;
    ncand += shape;
  }
  if (ncand) {
    int* d = nullptr;
    FGB_TRY(dmalloc(ctx, (void**)&d, sizeof(int) * 2 * J));
    FGB_CUDA(ctx, cudaMemsetAsync(d, 0, sizeof(int) * 2 * J, ctx->stream));
    for (int q = 0; q < J; ++q) {
      if (!cand[q]) continue;
      const DevFactor& f = F->f[q];
      const int g = std::max(1, std::min(2 * ctx->sm_count, (f.rows + 255) / 256));
      k_bfly_detect<<<g, 256, 0, ctx->stream>>>(f.rowptr, f.colind, f.rows, d + q, d + J + q);
      FGB_LAUNCHED(ctx);
    }
    std::vector<int> h(2 * J);
    cudaError_t e = cudaMemcpyAsync(h.data(), d, sizeof(int) * 2 * J, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    dfree(d);
    if (e != cudaSuccess) return cuda_check(ctx, e, "butterfly detection");
    for (int q = 0; q < J; ++q) F->f[q].bfly = (cand[q] && !h[q]) ? h[J + q] : 0;
  } else {
    for (auto& f : F->f) f.bfly = 0;
  }
  return FGB_OK;
}

template <typename T, int G>
static void build_plan(fgb_faust* F, char op, int nfac, BflyPlan& p) {
  const int J = (int)F->f.size();
  p.n = F->f[0].rows;
  p.nsteps = nfac;
  // application order: G_{nfac-1} first, with G_q = S_q (op N) or S_{J-1-q}^T
  for (int s = 0; s < nfac; ++s) {
    const int q = nfac - 1 - s;
    const DevFactor& f = F->f[op == 'N' ? q : J - 1 - q];
    p.val[s] = op == 'N' ? f.val : f.t_val;
    p.stride[s] = f.bfly;
  }
  p.npasses = 0;
  for (int s = 0; s < nfac;) {
    const int ps = p.npasses++;
    int bits[BF_G], nb = 0, cnt = 0;
    while (s < nfac && cnt < G) {
      bool have = false;
      for (int b = 0; b < nb; ++b) have = have || bits[b] == p.stride[s];
      if (!have) {
        if (nb == G) break;
        bits[nb++] = p.stride[s];
      }
      ++cnt;
      ++s;
    }
    std::sort(bits, bits + nb);
    p.pass_first[ps] = s - cnt;
    p.pass_n[ps] = cnt;
    p.pass_g[ps] = nb;
    for (int b = 0; b < BF_G; ++b) p.pass_bit[ps][b] = b < nb ? bits[b] : 0;
  }
}

template <typename T, int TC, int G>
static fgb_status launch_bfly(fgb_faust* F, char op, int nfac, const T* X, int ldx, int ncols, T* Y, int ldy) {
  fgb_ctx* ctx = F->ctx;
  BflyPlan p;
  build_plan<T, G>(F, op, nfac, p);
  const size_t smem = (size_t)p.n * TC * sizeof(T);
  auto kern = k_bfly_chain<T, TC, G>;
  if (smem > 48 * 1024)
    FGB_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int tiles = (ncols + TC - 1) / TC;
  kern<<<tiles, BF_THREADS, smem, ctx->stream>>>(p, X, ldx, ncols, Y, ldy);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

// Runs G_0 ... G_{nfac-1} X with the butterfly kernel when every factor of the
// chain is a butterfly factor and the column tile fits in shared memory;
// *ran tells whether it did.  force: also for few column tiles.
fgb_status bfly_chain(fgb_faust* F, char op, int nfac, const void* X, int ldx, int ncols, void* Y, int ldy,
                      bool force, bool* ran) {
  *ran = false;
  fgb_ctx* ctx = F->ctx;
  if (F->dtype != FGB_F32 && F->dtype != FGB_F64) return FGB_OK;
  if (nfac < 1 || nfac > BF_MAXS || ncols <= 0) return FGB_OK;
  FGB_TRY(bfly_detect(F));
  const int J = (int)F->f.size();
  for (int q = 0; q < nfac; ++q)
    if (F->f[op == 'N' ? q : J - 1 - q].bfly <= 0) return FGB_OK;
  const int n = F->f[0].rows;
  for (auto& f : F->f)
    if (f.rows != n) return FGB_OK;
  for (int q = 0; q < nfac; ++q) {
    const DevFactor& f = F->f[op == 'N' ? q : J - 1 - q];
    if (op != 'N' && !f.has_t) return FGB_OK;
    // pairs of values are read as one 2-element vector
    if ((uintptr_t)(op == 'N' ? f.val : f.t_val) % (2 * dtype_size(F->dtype))) return FGB_OK;
  }
  const size_t cap = std::min<size_t>(ctx->smem_optin ? ctx->smem_optin : 227 * 1024, 200 * 1024);
  if ((size_t)n * 16 > cap) return FGB_OK;  // one 16-byte row per matrix row
  const int tc = 16 / (int)dtype_size(F->dtype);
  const long tiles = (ncols + tc - 1) / tc;
  if (!force && tiles < ctx->sm_count) return FGB_OK;
  *ran = true;
  if (F->dtype == FGB_F32)
    return launch_bfly<float, 4, 2>(F, op, nfac, (const float*)X, ldx, ncols, (float*)Y, ldy);
  return launch_bfly<double, 2, 2>(F, op, nfac, (const double*)X, ldx, ncols, (double*)Y, ldy);
}

}  // namespace fgb
