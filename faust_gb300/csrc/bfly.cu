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
#include "tc_common.cuh"

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
// The full chain of an n = 2^L butterfly Faust (1024 <= n <= 4096) applied in
// one of its two natural orders: strides 1, 2, ..., n/2 in application order
// (F X with the factors of butterfly_support, whose factor i has stride
// n / 2^(i+1)) or n/2, ..., 1 (F^T X).  With the strides known at compile
// time a pass takes four consecutive factors: an orbit is the 16 rows
// base + {0..15} << lb, held in registers for the tile's 4 columns, and every
// shared-memory address is a per-thread base plus an immediate.  A 4096-row
// chain is three passes and two barriers.
//
// Shared tile: column-major, column c at word c * CW, row r at word
// r + 16 (r >> 8) (a 64-byte pad every 256 rows), CW = 4 (mod 32).  X arrives
// by bulk asynchronous copies of 256-row runs (one per run and column, on an
// mbarrier with a bounded wait), so no thread loads it.  Conflict-free
// accesses: a pass whose rows are contiguous (lb = 0) reads 16-byte vectors
// and lane l takes the columns in the order rotated by (l >> 1) & 3 (CW = 4
// puts the columns 16 bytes apart in the banks); the pad moves rows r and
// r + 256 16 banks apart for the scalar accesses of the lb = 4 pass.  The
// last pass writes Y from registers (lb > 0: every warp store is 128
// contiguous bytes) or through the tile and bulk stores (lb = 0).
//
// Factor values are read from a copy laid out in the kernel's order
// (k_br_layout): for pass P, step j, butterfly pair h of the step's stage and
// orbit o, one float4 holding (v0, v1) of the pair's two rows, orbits
// innermost, so each warp load is 512 contiguous bytes and a pair's values
// arrive in one load.
constexpr int BR_TC = 4;
constexpr int BR_MAXT = 256;
constexpr int BR_PG = 4;

template <int L, bool ASC>
struct BrShape {
  static constexpr int PG = BR_PG;
  static constexpr int n = 1 << L;
  static constexpr int NP = (L + PG - 1) / PG;
  static constexpr int T = (n >> PG) < BR_MAXT ? (n >> PG) : BR_MAXT;
  static constexpr int NRUN = n / 256;                     // 256-row runs per column
  static constexpr int CW = (n + 16 * NRUN + 31) / 32 * 32 + 4;  // column stride (words)
  static constexpr size_t SMEM = (size_t)BR_TC * CW * 4 + 16;   // tile + mbarrier
  __host__ __device__ static constexpr int g(int P) { return L - PG * P < PG ? L - PG * P : PG; }
  __host__ __device__ static constexpr int lb(int P) { return ASC ? PG * P : L - PG * P - g(P); }
  __host__ __device__ static constexpr int word(int r) { return r + 16 * (r >> 8); }
  // float4 offset of pass P's values
  __host__ __device__ static constexpr long voff(int P) { return P == 0 ? 0 : voff(P - 1) + (long)g(P - 1) * (n / 2); }
  __host__ __device__ static constexpr int base(int P, int o) {
    return (o & ((1 << lb(P)) - 1)) | ((o >> lb(P)) << (lb(P) + g(P)));
  }
};

struct BrSrc {
  const float2* val[32];  // step s (application order): (v0, v1) per row
};

template <int L, bool ASC>
__global__ void k_br_layout(const __grid_constant__ BrSrc src, float4* __restrict__ out) {
  using S = BrShape<L, ASC>;
  const long total = (long)L * (S::n / 2);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    int P = 0;
    long rem = i;
    while (rem >= (long)S::g(P) * (S::n / 2)) rem -= (long)S::g(P++) * (S::n / 2);
    const int lb = S::lb(P), R = 1 << S::g(P), orb = S::n >> S::g(P);
    const int o = (int)(rem % orb), jh = (int)(rem / orb);
    const int j = jh / (R / 2), h = jh % (R / 2);
    const int base = S::base(P, o);
    // the h-th pair (k, k | 2^B) of step j's stage, B its local bit
    const int B = ASC ? j : S::g(P) - 1 - j;
    const int k = ((h >> B) << (B + 1)) | (h & ((1 << B) - 1)), k1 = k | (1 << B);
    const float2* v = src.val[S::PG * P + j];
    const float2 a = v[base + (k << lb)], b = v[base + (k1 << lb)];
    out[i] = make_float4(a.x, a.y, b.x, b.y);
  }
}

struct BrArgs {
  const float4* vals;  // k_br_layout order
  const float* X;
  float* Y;
  int ldx, ldy, ncols;
  int* err;            // set when the bounded wait for the tile runs out
};

// R contiguous words at p (R = 2, 4, 8 or 16; p aligned to min(R, 4) words).
template <int R>
__device__ __forceinline__ void br_lds_run(const float* p, float (&v)[R]) {
  if constexpr (R == 2) {
    const float2 a = *reinterpret_cast<const float2*>(p);
    v[0] = a.x, v[1] = a.y;
  } else {
#pragma unroll
    for (int q = 0; q < R / 4; ++q) {
      const float4 a = *(reinterpret_cast<const float4*>(p) + q);
      v[4 * q] = a.x, v[4 * q + 1] = a.y, v[4 * q + 2] = a.z, v[4 * q + 3] = a.w;
    }
  }
}

template <int R>
__device__ __forceinline__ void br_sts_run(float* p, const float (&v)[R]) {
  if constexpr (R == 2) {
    *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
  } else {
#pragma unroll
    for (int q = 0; q < R / 4; ++q)
      *(reinterpret_cast<float4*>(p) + q) = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
  }
}

// Items of a thread: (pass P, orbit round U); an item applies the pass's G
// steps to orbit o = tid + U * T, i.e. NPAIR = G * R / 2 butterfly pairs whose
// value float4s sit at pv + i * ORB + o (i = step * R / 2 + pair).  A ring of
// D value loads runs ahead of the arithmetic across steps, items and passes
// (values do not depend on the tile).
template <int L, bool ASC, int P>
struct BrItem {
  using S = BrShape<L, ASC>;
  static constexpr int G = S::g(P), LB = S::lb(P), R = 1 << G;
  static constexpr int ORB = S::n >> G;
  static constexpr int OPT = ORB / S::T;
  static constexpr int NPAIR = G * R / 2;
};

template <int L, bool ASC, int P = 0>
__host__ __device__ constexpr int br_min_pairs() {
  if constexpr (P + 1 < BrShape<L, ASC>::NP) {
    constexpr int a = BrItem<L, ASC, P>::NPAIR, b = br_min_pairs<L, ASC, P + 1>();
    return a < b ? a : b;
  } else {
    return BrItem<L, ASC, P>::NPAIR;
  }
}

template <int L, bool ASC>
__host__ __device__ constexpr int br_ring() {
  return br_min_pairs<L, ASC>() < 8 ? br_min_pairs<L, ASC>() : 8;
}

// Value float4 of pair i of item (P, U) for thread tid.
template <int L, bool ASC, int P, int U>
__device__ __forceinline__ float4 br_val(const float4* __restrict__ vals, int tid, int i) {
  using I = BrItem<L, ASC, P>;
  return __ldg(vals + BrShape<L, ASC>::voff(P) + (long)i * I::ORB + tid + U * BrShape<L, ASC>::T);
}

// C0: pairs of the thread's earlier items; pair i of this item is in ring
// slot (C0 + i) % D.
template <int L, bool ASC, int P, int U, int D, int C0>
__device__ __forceinline__ void br_item(const BrArgs& a, float* tile, int tid, int j0, float4 (&ring)[D]) {
  using S = BrShape<L, ASC>;
  using I = BrItem<L, ASC, P>;
  constexpr int G = I::G, LB = I::LB, R = I::R, NPAIR = I::NPAIR;
  constexpr bool LAST_PASS = P == S::NP - 1;
  constexpr bool LAST_ITEM = LAST_PASS && U + 1 == I::OPT;
  constexpr int NP2 = U + 1 < I::OPT ? P : P + 1;  // next item
  constexpr int NU2 = U + 1 < I::OPT ? U + 1 : 0;
  const int o = tid + U * S::T;
  const int base = S::base(P, o);
  // contiguous rows: columns in an order rotated per lane pair
  const int rot = LB == 0 ? (tid >> 1) & 3 : 0;
  float x[R][BR_TC];
  const float* rowp = tile + S::word(base);
#pragma unroll
  for (int t = 0; t < BR_TC; ++t) {
    const float* cp = rowp + ((t + rot) & 3) * S::CW;
    if constexpr (LB == 0) {
      float c[R];
      br_lds_run<R>(cp, c);
#pragma unroll
      for (int k = 0; k < R; ++k) x[k][t] = c[k];
    } else {
#pragma unroll
      for (int k = 0; k < R; ++k) x[k][t] = cp[S::word(k << LB)];
    }
  }
#pragma unroll
  for (int i = 0; i < NPAIR; ++i) {
    const int slot = (C0 + i) % D;
    const float4 w = ring[slot];
    if (i + D < NPAIR) {
      ring[slot] = br_val<L, ASC, P, U>(a.vals, tid, i + D);
    } else if constexpr (!LAST_ITEM) {
      ring[slot] = br_val<L, ASC, NP2, NU2>(a.vals, tid, i + D - NPAIR);
    }
    const int J = i / (R / 2), h = i % (R / 2);
    const int B = ASC ? J : G - 1 - J;
    const int k = ((h >> B) << (B + 1)) | (h & ((1 << B) - 1)), k1 = k | (1 << B);
#pragma unroll
    for (int t = 0; t < BR_TC; ++t) {
      const float p0 = x[k][t], p1 = x[k1][t];
      x[k][t] = fmad(w.y, p1, fmad(w.x, p0, 0.0f));
      x[k1][t] = fmad(w.w, p1, fmad(w.z, p0, 0.0f));
    }
  }
  if constexpr (LAST_PASS && LB > 0) {
#pragma unroll
    for (int t = 0; t < BR_TC; ++t) {
      if (j0 + t >= a.ncols) continue;
      float* yc = a.Y + (long)(j0 + t) * a.ldy + base;
#pragma unroll
      for (int k = 0; k < R; ++k) __stcs(yc + (k << LB), x[k][t]);
    }
  } else {
    float* wp = tile + S::word(base);
#pragma unroll
    for (int t = 0; t < BR_TC; ++t) {
      float* cp = wp + ((t + rot) & 3) * S::CW;
      if constexpr (LB == 0) {
        float c[R];
#pragma unroll
        for (int k = 0; k < R; ++k) c[k] = x[k][t];
        br_sts_run<R>(cp, c);
      } else {
#pragma unroll
        for (int k = 0; k < R; ++k) cp[S::word(k << LB)] = x[k][t];
      }
    }
  }
  if constexpr (!LAST_ITEM) {
    if constexpr (NP2 != P) __syncthreads();
    br_item<L, ASC, NP2, NU2, D, C0 + NPAIR>(a, tile, tid, j0, ring);
  }
}

__device__ __forceinline__ void br_bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   tc::su32(dst)),
               "l"(src), "r"(bytes), "r"(tc::su32(bar))
               : "memory");
}

__device__ __forceinline__ void br_bulk_store(void* dst, const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(tc::su32(src)),
               "r"(bytes)
               : "memory");
}

// One block per tile of BR_TC columns.
template <int L, bool ASC>
__global__ void __launch_bounds__(BrShape<L, ASC>::T, 2) k_bfly_radix(const __grid_constant__ BrArgs a) {
  using S = BrShape<L, ASC>;
  extern __shared__ __align__(128) float br_tile[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(br_tile + BR_TC * S::CW);
  const int tid = threadIdx.x;
  const int j0 = blockIdx.x * BR_TC;
  const int nc = min(BR_TC, a.ncols - j0);
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid < 32) {
    if (tid == 0) tc::mbar_expect_tx(bar, (uint32_t)(nc * S::n * 4));
    __syncwarp();
    for (int i = tid; i < nc * S::NRUN; i += 32) {
      const int c = i / S::NRUN, g = i % S::NRUN;
      br_bulk_load(br_tile + c * S::CW + S::word(g * 256), a.X + (long)(j0 + c) * a.ldx + g * 256, 1024, bar);
    }
  }
  // the first value loads go out while the tile is in flight
  constexpr int D = br_ring<L, ASC>();
  float4 ring[D];
#pragma unroll
  for (int i = 0; i < D; ++i) ring[i] = br_val<L, ASC, 0, 0>(a.vals, tid, i);
  bool ok = false;
  for (unsigned i = 0; i < tc::WAIT_LIMIT; ++i)
    if (tc::mbar_try_wait(bar, 0)) {
      ok = true;
      break;
    }
  if (__syncthreads_or(!ok)) {
    if (tid == 0) {
      atomicExch(a.err, 1);
      // the copies in flight land before the shared memory is released
      for (unsigned i = 0; i < tc::WAIT_LIMIT && !tc::mbar_try_wait(bar, 0); ++i) {
      }
    }
    return;
  }
  br_item<L, ASC, 0, 0, D, 0>(a, br_tile, tid, j0, ring);
  if constexpr (S::lb(S::NP - 1) == 0) {
    // the last pass left Y's tile in shared memory
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid < 32) {
      for (int i = tid; i < nc * S::NRUN; i += 32) {
        const int c = i / S::NRUN, g = i % S::NRUN;
        br_bulk_store(a.Y + (long)(j0 + c) * a.ldy + g * 256, br_tile + c * S::CW + S::word(g * 256), 1024);
      }
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    }
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

template <int L, bool ASC>
static fgb_status launch_radix(fgb_faust* F, int slot, const BflyPlan& p, BrArgs a) {
  using S = BrShape<L, ASC>;
  fgb_ctx* ctx = F->ctx;
  if (!F->brv[slot]) {
    BrSrc src;
    for (int s = 0; s < L; ++s) src.val[s] = reinterpret_cast<const float2*>(p.val[s]);
    void* d = nullptr;
    FGB_TRY(dmalloc(ctx, &d, sizeof(float) * 2 * (size_t)L * S::n));
    const long total = (long)L * (S::n / 2);
    const int g = (int)std::min<long>(4L * ctx->sm_count, (total + 255) / 256);
    k_br_layout<L, ASC><<<g, 256, 0, ctx->stream>>>(src, reinterpret_cast<float4*>(d));
    FGB_LAUNCHED(ctx);
    F->brv[slot] = d;
  }
  a.vals = reinterpret_cast<const float4*>(F->brv[slot]);
  FGB_TRY(kernel_err_word(ctx, &a.err));
  auto kern = k_bfly_radix<L, ASC>;
  FGB_TRY(smem_opt_in(ctx, (const void*)kern, S::SMEM));
  const int tiles = (a.ncols + BR_TC - 1) / BR_TC;
  kern<<<tiles, S::T, S::SMEM, ctx->stream>>>(a);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

// The radix kernel when the plan is the whole chain of an FP32 butterfly
// Faust with 1024 <= n <= 4096 in one of the two natural stride orders and
// every pointer and leading dimension allows its 16-byte accesses; *ran
// tells whether it ran.
static fgb_status try_radix(fgb_faust* F, char op, const BflyPlan& p, const float* X, int ldx, int ncols, float* Y,
                            int ldy, bool* ran) {
  *ran = false;
  int L = 0;
  while ((1 << L) < p.n) ++L;
  if (L < 10 || L > 12 || p.nsteps != L || (int)F->f.size() != L) return FGB_OK;
  bool asc = true, desc = true;
  for (int s = 0; s < L; ++s) {
    asc = asc && p.stride[s] == (1 << s);
    desc = desc && p.stride[s] == (1 << (L - 1 - s));
  }
  if (!asc && !desc) return FGB_OK;
  if ((uintptr_t)X % 16 || (uintptr_t)Y % 16 || ldx % 4 || ldy % 4) return FGB_OK;
  BrArgs a;
  a.vals = nullptr;
  a.err = nullptr;
  a.X = X, a.Y = Y, a.ldx = ldx, a.ldy = ldy, a.ncols = ncols;
  *ran = true;
  const int slot = op == 'N' ? 0 : 1;
  switch (L * 2 + (asc ? 1 : 0)) {
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
  FGB_TRY(smem_opt_in(ctx, (const void*)kern, smem));
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
