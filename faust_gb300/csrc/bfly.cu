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
constexpr int BF_G = 3;       // stride slots per pass in the plan (two are used)
constexpr int BF_THREADS = 256;

struct BflyPlan {
  int n, nsteps, npasses;
  const void* val[BF_MAXS];   // step s (application order): 2 values per row
  int stride[BF_MAXS];
  int pass_first[BF_MAXS], pass_n[BF_MAXS], pass_g[BF_MAXS];
  int pass_bit[BF_MAXS][BF_G];  // orbit strides of the pass, ascending
  int step_bit[BF_MAXS];        // index of step s's stride among its pass's strides
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

// 16-byte row slot of matrix row r in the shared tile.  Its low three bits
// are XORed with (r3, r4, r3 ^ r4), so that the eight rows one quarter-warp
// touches (eight consecutive orbits, same position in the orbit) land in
// distinct bank groups for every pass stride pair of n = 4096 except
// (1, 8), a lone 2, and (2, 2^j) with j >= 4, which are 2-way.
__device__ __forceinline__ int bf_slot(int r) { return r ^ ((0x3650 >> (((r >> 3) & 3) << 2)) & 7); }

// One orbit of a pass with two strides (rows base, +b0, +b1, +b0+b1) or one
// stride (rows base, +b0), and the values of the pass's factors on its rows.
template <typename T>
struct BfItem {
  int row[4];
  typename V2<T>::type v[2][4];
};

template <typename T>
__device__ __forceinline__ void bf_item(const BflyPlan& p, int ps, int o, BfItem<T>& it) {
  using T2 = typename V2<T>::type;
  const int g = p.pass_g[ps], ns = p.pass_n[ps], first = p.pass_first[ps];
  const int b0 = p.pass_bit[ps][0], b1 = p.pass_bit[ps][1];
  int base = ((o & ~(b0 - 1)) << 1) | (o & (b0 - 1));
  if (g == 2) base = ((base & ~(b1 - 1)) << 1) | (base & (b1 - 1));
  it.row[0] = base;
  it.row[1] = base + b0;
  it.row[2] = base + b1;
  it.row[3] = base + b0 + b1;
  const T2* v0 = reinterpret_cast<const T2*>(p.val[first]);
  const T2* v1 = reinterpret_cast<const T2*>(p.val[first + (ns > 1 ? 1 : 0)]);
  if (g == 2) {
#pragma unroll
    for (int k = 0; k < 4; ++k) it.v[0][k] = __ldg(v0 + it.row[k]);
#pragma unroll
    for (int k = 0; k < 4; ++k) it.v[1][k] = __ldg(v1 + it.row[k]);
  } else {
    it.v[0][0] = __ldg(v0 + it.row[0]);
    it.v[0][1] = __ldg(v0 + it.row[1]);
    if (ns > 1) {
      it.v[1][0] = __ldg(v1 + it.row[0]);
      it.v[1][1] = __ldg(v1 + it.row[1]);
    }
  }
}

// One factor on the rows of an orbit: pairs (k, k | 2^b) of local rows.
template <typename T, int TC, int B>
__device__ __forceinline__ void bf_stage(T (&xs)[4][TC], const typename V2<T>::type (&v)[4]) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if ((k >> B) & 1) continue;
    const int k1 = k | (1 << B);
#pragma unroll
    for (int t = 0; t < TC; ++t) {
      const T a = xs[k][t], c = xs[k1][t];
      xs[k][t] = fmad(v[k].y, c, fmad(v[k].x, a, T(0)));
      xs[k1][t] = fmad(v[k1].y, c, fmad(v[k1].x, a, T(0)));
    }
  }
}

// One block per column tile of TC columns, BF_THREADS threads, two strides
// per pass.  Each thread walks its (pass, orbit) items in order and loads the
// values of its next item before working on the current one, so their L2
// latency overlaps the shared-memory work (also across the pass barrier:
// values do not depend on the tile).
template <typename T, int TC>
__global__ void __launch_bounds__(BF_THREADS, sizeof(T) == 4 ? 3 : 2)
    k_bfly_chain(const __grid_constant__ BflyPlan p, const T* __restrict__ X, int ldx, int ncols, T* __restrict__ Y,
                 int ldy) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* tile = reinterpret_cast<T*>(smem_raw);  // n slots of TC values
  const int n = p.n;
  const int j0 = blockIdx.x * TC;
  const int tid = threadIdx.x;
  int nps = 0;
  while (nps < p.npasses && tid >= (n >> p.pass_g[nps])) ++nps;
  BfItem<T> nx;
  if (nps < p.npasses) bf_item<T>(p, nps, tid, nx);
  for (int r = tid; r < n; r += BF_THREADS) {
    T x[TC];
#pragma unroll
    for (int t = 0; t < TC; ++t) x[t] = (j0 + t < ncols) ? X[r + (long)(j0 + t) * ldx] : T(0);
    st_row<T, TC>(tile + (long)bf_slot(r) * TC, x);
  }
  __syncthreads();
  for (int ps = 0; ps < p.npasses; ++ps) {
    const int g = p.pass_g[ps], ns = p.pass_n[ps], first = p.pass_first[ps];
    const bool last = ps + 1 == p.npasses;
    const int orbits = n >> g;
    const int sb0 = p.step_bit[first], sb1 = p.step_bit[first + (ns > 1 ? 1 : 0)];
    for (int o = tid; o < orbits; o += BF_THREADS) {
      const BfItem<T> it = nx;
      {
        int qo = o + BF_THREADS, qp = ps;
        if (qo >= orbits) {
          qp = ps + 1;
          qo = tid;
          while (qp < p.npasses && tid >= (n >> p.pass_g[qp])) ++qp;
        }
        if (qp < p.npasses) bf_item<T>(p, qp, qo, nx);
      }
      T xs[4][TC];
      if (g == 2) {
#pragma unroll
        for (int k = 0; k < 4; ++k) ld_row<T, TC>(tile + (long)bf_slot(it.row[k]) * TC, xs[k]);
        if (sb0 == 0) bf_stage<T, TC, 0>(xs, it.v[0]);
        else bf_stage<T, TC, 1>(xs, it.v[0]);
        if (ns > 1) {
          if (sb1 == 0) bf_stage<T, TC, 0>(xs, it.v[1]);
          else bf_stage<T, TC, 1>(xs, it.v[1]);
        }
      } else {
        // one stride: local rows 0 and 1 only
#pragma unroll
        for (int k = 0; k < 2; ++k) ld_row<T, TC>(tile + (long)bf_slot(it.row[k]) * TC, xs[k]);
#pragma unroll
        for (int s = 0; s < 2; ++s) {
          if (s >= ns) break;
#pragma unroll
          for (int t = 0; t < TC; ++t) {
            const T a = xs[0][t], c = xs[1][t];
            xs[0][t] = fmad(it.v[s][0].y, c, fmad(it.v[s][0].x, a, T(0)));
            xs[1][t] = fmad(it.v[s][1].y, c, fmad(it.v[s][1].x, a, T(0)));
          }
        }
      }
      const int kn = g == 2 ? 4 : 2;
      if (last) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          if (k >= kn) continue;
#pragma unroll
          for (int t = 0; t < TC; ++t)
            if (j0 + t < ncols) Y[it.row[k] + (long)(j0 + t) * ldy] = xs[k][t];
        }
      } else {
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (k < kn) st_row<T, TC>(tile + (long)bf_slot(it.row[k]) * TC, xs[k]);
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

// Passes of at most two consecutive factors (application order) with at most
// two distinct strides.
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
    const int cnt = (s + 1 < nfac) ? 2 : 1;
    int bits[2] = {p.stride[s], cnt > 1 ? p.stride[s + 1] : 0};
    int nb = (cnt > 1 && bits[1] != bits[0]) ? 2 : 1;
    if (nb == 2 && bits[1] < bits[0]) std::swap(bits[0], bits[1]);
    p.pass_first[ps] = s;
    p.pass_n[ps] = cnt;
    p.pass_g[ps] = nb;
    p.pass_bit[ps][0] = bits[0];
    p.pass_bit[ps][1] = nb == 2 ? bits[1] : 0;
    p.pass_bit[ps][2] = 0;
    for (int u = 0; u < cnt; ++u) p.step_bit[s + u] = p.stride[s + u] == bits[0] ? 0 : 1;
    s += cnt;
  }
}

template <typename T, int TC>
static fgb_status launch_bfly(fgb_faust* F, char op, int nfac, const T* X, int ldx, int ncols, T* Y, int ldy) {
  fgb_ctx* ctx = F->ctx;
  BflyPlan p;
  build_plan(F, op, nfac, p);
  const size_t smem = (size_t)p.n * TC * sizeof(T);
  auto kern = k_bfly_chain<T, TC>;
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
    return launch_bfly<float, 4>(F, op, nfac, (const float*)X, ldx, ncols, (float*)Y, ldy);
  return launch_bfly<double, 2>(F, op, nfac, (const double*)X, ldx, ncols, (double*)Y, ldy);
}

}  // namespace fgb
