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

// ------------------------------------------------- radix kernel (FP32)
// The full chain of an n = 2^L butterfly Faust applied in one of its two
// natural orders: strides 1, 2, ..., n/2 in application order (F X with the
// factors of butterfly_support, whose factor i has stride n / 2^(i+1)) or
// n/2, ..., 1 (F^T X).  With the strides known at compile time a pass takes
// PG consecutive factors: an orbit is the R = 2^PG rows base + {0..R-1} << lb,
// held in registers for 4 columns, and every shared-memory address is a
// per-thread base plus an immediate.  The first pass reads X from global
// memory and the last writes Y, so the tile makes ceil(L/PG) - 1 trips
// through shared memory.
//
// Shared tile: row r at 16-byte slot r + (r >> PG) (one pad slot per 2^PG
// rows).  slot(base | off) = slot(base) + slot(off) for disjoint bits, and
// the 8 rows one quarter-warp touches land in distinct bank groups for the
// aligned stride groups of n = 4096.
//
// Factor values are read from a copy laid out in the kernel's order
// (k_br_layout): for pass P, step j, row pair h and orbit o, one float4
// holding (v0, v1) of the pair's two rows, orbits innermost, so each warp
// load is 512 contiguous bytes.
constexpr int BR_TC = 4;
constexpr int BR_MAXT = 256;
#ifndef FGB_BR_PG
#define FGB_BR_PG 4
#endif
constexpr int BR_PG = FGB_BR_PG;

template <int L, bool ASC, int PG>
struct BrShape {
  static constexpr int n = 1 << L;
  static constexpr int NP = (L + PG - 1) / PG;
  static constexpr int T = (n >> PG) < BR_MAXT ? (n >> PG) : BR_MAXT;
  __host__ __device__ static constexpr int g(int P) { return L - PG * P < PG ? L - PG * P : PG; }
  __host__ __device__ static constexpr int lb(int P) { return ASC ? PG * P : L - PG * P - g(P); }
  __host__ __device__ static constexpr int slot(int r) { return r + (r >> PG); }
  // float4 offset of pass P's values
  __host__ __device__ static constexpr long voff(int P) { return P == 0 ? 0 : voff(P - 1) + (long)g(P - 1) * (n / 2); }
  __host__ __device__ static constexpr int base(int P, int o) {
    return (o & ((1 << lb(P)) - 1)) | ((o >> lb(P)) << (lb(P) + g(P)));
  }
};

struct BrSrc {
  const float2* val[32];  // step s (application order): (v0, v1) per row
};

template <int L, bool ASC, int PG>
__global__ void k_br_layout(const __grid_constant__ BrSrc src, float4* __restrict__ out) {
  using S = BrShape<L, ASC, PG>;
  const long total = (long)L * (S::n / 2);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    int P = 0;
    long rem = i;
    while (rem >= (long)S::g(P) * (S::n / 2)) rem -= (long)S::g(P++) * (S::n / 2);
    const int lb = S::lb(P), R = 1 << S::g(P), orb = S::n >> S::g(P);
    const int o = (int)(rem % orb), jh = (int)(rem / orb);
    const int j = jh / (R / 2), h = jh % (R / 2);
    const int base = S::base(P, o);
    const float2* v = src.val[PG * P + j];
    const float2 a = v[base + ((2 * h) << lb)], b = v[base + ((2 * h + 1) << lb)];
    out[i] = make_float4(a.x, a.y, b.x, b.y);
  }
}

struct BrArgs {
  const float4* vals;  // k_br_layout order
  const float* X;
  float* Y;
  int ldx, ldy, ncols;
};

// R consecutive floats at p (R = 2, 4, 8 or 16; p aligned to min(R, 4) floats).
template <int R>
__device__ __forceinline__ void br_ld_run(const float* p, float (&v)[R]) {
  if constexpr (R == 2) {
    const float2 a = __ldcs(reinterpret_cast<const float2*>(p));
    v[0] = a.x, v[1] = a.y;
  } else {
#pragma unroll
    for (int q = 0; q < R / 4; ++q) {
      const float4 a = __ldcs(reinterpret_cast<const float4*>(p) + q);
      v[4 * q] = a.x, v[4 * q + 1] = a.y, v[4 * q + 2] = a.z, v[4 * q + 3] = a.w;
    }
  }
}

template <int R>
__device__ __forceinline__ void br_st_run(float* p, const float (&v)[R]) {
  if constexpr (R == 2) {
    __stcs(reinterpret_cast<float2*>(p), make_float2(v[0], v[1]));
  } else {
#pragma unroll
    for (int q = 0; q < R / 4; ++q)
      __stcs(reinterpret_cast<float4*>(p) + q, make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]));
  }
}

// Values of step j of pass P on the R rows of orbit o.
template <int R, int ORB>
__device__ __forceinline__ void br_vals(const float4* __restrict__ pv, int o, float2 (&v)[R]) {
#pragma unroll
  for (int h = 0; h < R / 2; ++h) {
    const float4 a = __ldg(pv + h * ORB + o);
    v[2 * h] = make_float2(a.x, a.y);
    v[2 * h + 1] = make_float2(a.z, a.w);
  }
}

// One factor on an orbit's rows: pairs (k, k | 2^B) of local rows.
template <int R, int B>
__device__ __forceinline__ void br_stage(float (&x)[R][BR_TC], const float2 (&v)[R]) {
#pragma unroll
  for (int k = 0; k < R; ++k) {
    if ((k >> B) & 1) continue;
    const int k1 = k | (1 << B);
#pragma unroll
    for (int t = 0; t < BR_TC; ++t) {
      const float a = x[k][t], c = x[k1][t];
      x[k][t] = fmad(v[k].y, c, fmad(v[k].x, a, 0.0f));
      x[k1][t] = fmad(v[k1].y, c, fmad(v[k1].x, a, 0.0f));
    }
  }
}

// Steps J.. of a pass (local bit of step J's stride: J ascending, G-1-J
// descending), the values of step J+1 loaded before step J's arithmetic.
template <bool ASC, int G, int R, int ORB, int J>
__device__ __forceinline__ void br_steps(const float4* __restrict__ pv, int o, float (&x)[R][BR_TC],
                                         float2 (&v)[R]) {
  float2 vn[R];
  if constexpr (J + 1 < G) br_vals<R, ORB>(pv + (J + 1) * (R / 2) * ORB, o, vn);
  br_stage<R, ASC ? J : G - 1 - J>(x, v);
  if constexpr (J + 1 < G) {
#pragma unroll
    for (int k = 0; k < R; ++k) v[k] = vn[k];
    br_steps<ASC, G, R, ORB, J + 1>(pv, o, x, v);
  }
}

template <int L, bool ASC, int PG, int P>
__device__ __forceinline__ void br_pass(const BrArgs& a, float* tile, int tid, int j0, bool full) {
  using S = BrShape<L, ASC, PG>;
  constexpr int G = S::g(P), LB = S::lb(P), R = 1 << G;
  constexpr int ORB = S::n >> G;
  constexpr int OPT = ORB / S::T;
  constexpr bool FIRST = P == 0, LAST = P == S::NP - 1;
  const float4* pv = a.vals + S::voff(P);
#pragma unroll 1
  for (int u = 0; u < OPT; ++u) {
    const int o = tid + u * S::T;
    const int base = S::base(P, o);
    float2 v[R];
    br_vals<R, ORB>(pv, o, v);
    float x[R][BR_TC];
    if constexpr (FIRST) {
      if constexpr (LB == 0) {
#pragma unroll
        for (int t = 0; t < BR_TC; ++t) {
          float c[R];
          if (full || j0 + t < a.ncols) {
            br_ld_run<R>(a.X + (long)(j0 + t) * a.ldx + base, c);
          } else {
#pragma unroll
            for (int k = 0; k < R; ++k) c[k] = 0.0f;
          }
#pragma unroll
          for (int k = 0; k < R; ++k) x[k][t] = c[k];
        }
      } else {
#pragma unroll
        for (int t = 0; t < BR_TC; ++t) {
          const float* xc = a.X + (long)(j0 + t) * a.ldx + base;
#pragma unroll
          for (int k = 0; k < R; ++k) x[k][t] = (full || j0 + t < a.ncols) ? __ldcs(xc + (k << LB)) : 0.0f;
        }
      }
    } else {
      const float* s = tile + S::slot(base) * BR_TC;
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const float4 q = *reinterpret_cast<const float4*>(s + S::slot(k << LB) * BR_TC);
        x[k][0] = q.x, x[k][1] = q.y, x[k][2] = q.z, x[k][3] = q.w;
      }
    }
    br_steps<ASC, G, R, ORB, 0>(pv, o, x, v);
    if constexpr (LAST) {
      if constexpr (LB == 0) {
#pragma unroll
        for (int t = 0; t < BR_TC; ++t) {
          if (!full && j0 + t >= a.ncols) continue;
          float c[R];
#pragma unroll
          for (int k = 0; k < R; ++k) c[k] = x[k][t];
          br_st_run<R>(a.Y + (long)(j0 + t) * a.ldy + base, c);
        }
      } else {
#pragma unroll
        for (int t = 0; t < BR_TC; ++t) {
          if (!full && j0 + t >= a.ncols) continue;
          float* yc = a.Y + (long)(j0 + t) * a.ldy + base;
#pragma unroll
          for (int k = 0; k < R; ++k) __stcs(yc + (k << LB), x[k][t]);
        }
      }
    } else {
      float* s = tile + S::slot(base) * BR_TC;
#pragma unroll
      for (int k = 0; k < R; ++k)
        *reinterpret_cast<float4*>(s + S::slot(k << LB) * BR_TC) = make_float4(x[k][0], x[k][1], x[k][2], x[k][3]);
    }
  }
  if constexpr (!LAST) {
    __syncthreads();
    br_pass<L, ASC, PG, P + 1>(a, tile, tid, j0, full);
  }
}

// One block per tile of BR_TC columns.
template <int L, bool ASC, int PG>
__global__ void __launch_bounds__(BrShape<L, ASC, PG>::T, PG >= 4 ? 2 : 3) k_bfly_radix(const __grid_constant__ BrArgs a) {
  extern __shared__ __align__(16) float br_tile[];
  const int j0 = blockIdx.x * BR_TC;
  br_pass<L, ASC, PG, 0>(a, br_tile, threadIdx.x, j0, j0 + BR_TC <= a.ncols);
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

template <int L, bool ASC>
static fgb_status launch_radix(fgb_faust* F, int slot, const BflyPlan& p, BrArgs a) {
  using S = BrShape<L, ASC, BR_PG>;
  fgb_ctx* ctx = F->ctx;
  if (!F->brv[slot]) {
    BrSrc src;
    for (int s = 0; s < L; ++s) src.val[s] = reinterpret_cast<const float2*>(p.val[s]);
    void* d = nullptr;
    FGB_TRY(dmalloc(ctx, &d, sizeof(float) * 2 * (size_t)L * S::n));
    const long total = (long)L * (S::n / 2);
    const int g = (int)std::min<long>(4L * ctx->sm_count, (total + 255) / 256);
    k_br_layout<L, ASC, BR_PG><<<g, 256, 0, ctx->stream>>>(src, reinterpret_cast<float4*>(d));
    FGB_LAUNCHED(ctx);
    F->brv[slot] = d;
  }
  a.vals = reinterpret_cast<const float4*>(F->brv[slot]);
  auto kern = k_bfly_radix<L, ASC, BR_PG>;
  const size_t smem = (size_t)S::slot(S::n) * BR_TC * sizeof(float);
  if (smem > 48 * 1024)
    FGB_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int tiles = (a.ncols + BR_TC - 1) / BR_TC;
  kern<<<tiles, S::T, smem, ctx->stream>>>(a);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

// The radix kernel when the plan is the whole chain of an FP32 butterfly
// Faust with 2^8 <= n <= 2^12 in one of the two natural stride orders and
// every pointer and leading dimension allows its 16-byte accesses; *ran
// tells whether it ran.
static fgb_status try_radix(fgb_faust* F, char op, const BflyPlan& p, const float* X, int ldx, int ncols, float* Y,
                            int ldy, bool* ran) {
  *ran = false;
  int L = 0;
  while ((1 << L) < p.n) ++L;
  if (L < 8 || L > 12 || p.nsteps != L || (int)F->f.size() != L) return FGB_OK;
  bool asc = true, desc = true;
  for (int s = 0; s < L; ++s) {
    asc = asc && p.stride[s] == (1 << s);
    desc = desc && p.stride[s] == (1 << (L - 1 - s));
  }
  if (!asc && !desc) return FGB_OK;
  if ((uintptr_t)X % 16 || (uintptr_t)Y % 16 || ldx % 4 || ldy % 4) return FGB_OK;
  BrArgs a;
  a.vals = nullptr;
  a.X = X, a.Y = Y, a.ldx = ldx, a.ldy = ldy, a.ncols = ncols;
  *ran = true;
  const int slot = op == 'N' ? 0 : 1;
  switch (L * 2 + (asc ? 1 : 0)) {
    case 17: return launch_radix<8, true>(F, slot, p, a);
    case 16: return launch_radix<8, false>(F, slot, p, a);
    case 19: return launch_radix<9, true>(F, slot, p, a);
    case 18: return launch_radix<9, false>(F, slot, p, a);
    case 21: return launch_radix<10, true>(F, slot, p, a);
    case 20: return launch_radix<10, false>(F, slot, p, a);
    case 23: return launch_radix<11, true>(F, slot, p, a);
    case 22: return launch_radix<11, false>(F, slot, p, a);
    case 25: return launch_radix<12, true>(F, slot, p, a);
    default: return launch_radix<12, false>(F, slot, p, a);
  }
}

template <typename T, int TC>
static fgb_status launch_bfly(fgb_faust* F, char op, int nfac, const T* X, int ldx, int ncols, T* Y, int ldy) {
  fgb_ctx* ctx = F->ctx;
  BflyPlan p;
  build_plan(F, op, nfac, p);
  if constexpr (sizeof(T) == 4) {
    bool ran = false;
    FGB_TRY(try_radix(F, op, p, X, ldx, ncols, Y, ldy, &ran));
    if (ran) return FGB_OK;
  }
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
