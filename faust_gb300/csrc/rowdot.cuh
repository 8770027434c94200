// rowdot.cuh — the canonical order of a sparse row times a dense vector.
//
// A product entry y = sum_p val[p] * x(colind[p]) runs over the row's stored
// entries in order, cut into chunks of ROW_CHUNK entries: each chunk is a
// sequential fma from +0, and the chunk partials P_0 .. P_{M-1} are added by
// the recursive-halving pairwise tree (at stride s = 1, 2, 4, ...:
// Q_l += Q_{l+s} for l = 0 mod 2s and l + s < M).  A row of at most ROW_CHUNK
// entries is one sequential fma chain.  The oracle restates the same order
// (row_dot).
//
// On GB300 one FP64 FMA warp instruction issues every 64 cycles per
// scheduler, predicated or not, so a long row summed by one chain costs 64
// cycles per entry; with the chunks a long row splits over warps (aligned
// groups of chunks are subtrees of the tree) and over lanes.
#pragma once

#include "fgb_internal.cuh"

namespace fgb {

constexpr int ROW_CHUNK = 16;
constexpr int PI_CHUNK = ROW_CHUNK;

// Binary-counter merge of tree leaves arriving in order: level b holds the
// sum of 2^b consecutive leaves.  Pushing leaf number `count` (0-based)
// merges it with the occupied levels given by the bits of count (older +
// newer), which reproduces the recursive-halving tree; finish() combines the
// remaining levels from the lowest (newest) up.
template <typename T, int LEVELS, bool FLAT = false>
struct TreeAcc {
  T lv[LEVELS];
  __device__ __forceinline__ void push(int count, T v) {
    if (FLAT) {
      // branch-free over the levels (keeps lv in registers where the early
      // exit below would put it in local memory)
      const int land = __ffs(~count) - 1;
#pragma unroll
      for (int b = 0; b < LEVELS; ++b) {
        if (b < land) v = addr(lv[b], v);
        if (b == land) lv[b] = v;
      }
      return;
    }
#pragma unroll
    for (int b = 0; b < LEVELS; ++b) {
      if ((count >> b) & 1) {
        v = addr(lv[b], v);
      } else {
        lv[b] = v;
        return;
      }
    }
  }
  __device__ __forceinline__ T finish(int count) const {
    T acc = T(0);
    bool have = false;
#pragma unroll
    for (int b = 0; b < LEVELS; ++b)
      if ((count >> b) & 1) {
        acc = have ? addr(lv[b], acc) : lv[b];
        have = true;
      }
    return acc;
  }
};

// G independent trees advanced together (the same leaf count): one thread
// computing a long row for G consecutive columns of a shared-memory tile.
template <typename T, int G, int LEVELS>
struct TreeAccG {
  T lv[LEVELS][G];
  __device__ __forceinline__ void push(int count, const T (&v)[G], T (&carry)[G]) {
#pragma unroll
    for (int u = 0; u < G; ++u) carry[u] = v[u];
#pragma unroll
    for (int b = 0; b < LEVELS; ++b) {
      if ((count >> b) & 1) {
#pragma unroll
        for (int u = 0; u < G; ++u) carry[u] = addr(lv[b][u], carry[u]);
      } else {
#pragma unroll
        for (int u = 0; u < G; ++u) lv[b][u] = carry[u];
        return;
      }
    }
  }
  __device__ __forceinline__ void finish(int count, T (&out)[G]) const {
    bool have = false;
#pragma unroll
    for (int b = 0; b < LEVELS; ++b)
      if ((count >> b) & 1) {
#pragma unroll
        for (int u = 0; u < G; ++u) out[u] = have ? addr(lv[b][u], out[u]) : lv[b][u];
        have = true;
      }
  }
};

// A row (any length; one chunk when short) for G consecutive columns: the dense
// operand of column u is x[colind * stride + u] (a row-major tile), loaded
// G at a time by LOAD(ptr, vals).
template <typename T, int G, int LEVELS, typename Load>
__device__ __forceinline__ void row_long_g(const int* __restrict__ ci, const T* __restrict__ val, int p0, int p1,
                                           const T* __restrict__ x, int stride, Load load, T (&out)[G]) {
  TreeAccG<T, G, LEVELS> t;
  int m = 0;
  int b = p0;
  // full chunks, unrolled
  for (; b + ROW_CHUNK <= p1; b += ROW_CHUNK, ++m) {
    T P[G];
#pragma unroll
    for (int u = 0; u < G; ++u) P[u] = T(0);
#pragma unroll
    for (int q = 0; q < ROW_CHUNK; ++q) {
      const T v = val[b + q];
      T xv[G];
      load(x + ci[b + q] * stride, xv);
#pragma unroll
      for (int u = 0; u < G; ++u) P[u] = fmad(v, xv[u], P[u]);
    }
    T carry[G];
    t.push(m, P, carry);
  }
  if (b < p1 || m == 0) {
    T P[G];
#pragma unroll
    for (int u = 0; u < G; ++u) P[u] = T(0);
    for (int p = b; p < p1; ++p) {
      const T v = val[p];
      T xv[G];
      load(x + ci[p] * stride, xv);
#pragma unroll
      for (int u = 0; u < G; ++u) P[u] = fmad(v, xv[u], P[u]);
    }
    if (m == 0) {
      // a row of one chunk: its partial is the result (the tree is not
      // touched, so short rows never reach its spilled levels)
#pragma unroll
      for (int u = 0; u < G; ++u) out[u] = P[u];
      return;
    }
    T carry[G];
    t.push(m++, P, carry);
  }
  t.finish(m, out);
}

// One thread, a row of more than ROW_CHUNK entries (below 2^LEVELS chunks);
// the dense operand is x[colind * stride].
template <typename TC, typename TF, int LEVELS>
__device__ __forceinline__ TC row_thread_long_inl(const int* __restrict__ ci, const TF* __restrict__ val, int p0,
                                                  int p1, const TC* __restrict__ x, long stride) {
  TreeAcc<TC, LEVELS> t;
  int m = 0;
  for (int b = p0; b < p1; b += ROW_CHUNK, ++m) {
    TC P = TC(0);
    const int e = min(p1, b + ROW_CHUNK);
    for (int p = b; p < e; ++p) P = fmad((TC)val[p], x[(long)ci[p] * stride], P);
    t.push(m, P);
  }
  return t.finish(m);
}

template <typename TC, typename TF>
__device__ __noinline__ TC row_thread_long(const int* __restrict__ ci, const TF* __restrict__ val, int p0, int p1,
                                           const TC* __restrict__ x, long stride) {
  return row_thread_long_inl<TC, TF, 16>(ci, val, p0, p1, x, stride);
}

// One thread, any row: short rows inline, long ones through the call above.
template <typename TC, typename TF>
__device__ __forceinline__ TC pi_row_thread(const int* __restrict__ ci, const TF* __restrict__ val, int p0, int p1,
                                            const TC* __restrict__ x) {
  if (p1 - p0 > ROW_CHUNK) return row_thread_long<TC, TF>(ci, val, p0, p1, x, 1);
  TC acc = TC(0);
  for (int p = p0; p < p1; ++p) acc = fmad((TC)val[p], x[ci[p]], acc);
  return acc;
}

// One warp (all 32 lanes), lane l working on chunks l, l + 32, ...: each
// round of 32 chunks is reduced by the tree over lanes, and the round sums
// merge as leaves of the same tree (a round is an aligned subtree of 32).
// Every lane returns the value.
template <typename TC, typename TF>
__device__ __forceinline__ TC pi_row_warp(const int* __restrict__ ci, const TF* __restrict__ val, int p0, int p1,
                                          const TC* __restrict__ x, int lane) {
  const unsigned FULL = 0xffffffffu;
  const int M = (p1 - p0 + PI_CHUNK - 1) / PI_CHUNK;
  TreeAcc<TC, 12> t;
  int nr = 0;
  for (int r0 = 0; r0 < M; r0 += 32, ++nr) {
    const int m = r0 + lane;
    TC P = TC(0);
    if (m < M) {
      const int b = p0 + m * PI_CHUNK, e = min(p1, b + PI_CHUNK);
      for (int p = b; p < e; ++p) P = fmad((TC)val[p], x[ci[p]], P);
    }
    const int K = min(32, M - r0);
#pragma unroll
    for (int s = 1; s < 32; s <<= 1) {
      const TC o = __shfl_down_sync(FULL, P, s);
      if ((lane & (2 * s - 1)) == 0 && lane + s < K) P = addr(P, o);
    }
    t.push(nr, __shfl_sync(FULL, P, 0));
  }
  return t.finish(nr);
}

// A long row split over the NW warps of a block, one output per lane (a
// column of X, or a row of X for X S^T): warp w computes the roots of the
// chunk groups g = w, w + NW, ... (ROW_GROUP chunks each, an aligned subtree
// of the row's tree), the roots meet in shared memory (roots: ROW_GROUPS x 32
// values) and warp 0 merges them in order; rounds of ROW_GROUPS groups are
// aligned subtrees again.  The value is returned in warp 0 (other warps get
// 0).  Every thread of the block must call it with the same row.
constexpr int ROW_GROUP = 4;
constexpr int ROW_GROUPS = 64;

template <typename T, int NW, typename Gather>
__device__ __forceinline__ T row_block_long(const T* __restrict__ val, const int* __restrict__ colind, int p0,
                                            int p1, Gather gather, T* roots, int lane, int warp) {
  const int M = (p1 - p0 + ROW_CHUNK - 1) / ROW_CHUNK;
  const int NG = (M + ROW_GROUP - 1) / ROW_GROUP;
  TreeAcc<T, 16, true> top;
  int nround = 0;
  for (int g0 = 0; g0 < NG; g0 += ROW_GROUPS, ++nround) {
    const int ng = min(ROW_GROUPS, NG - g0);
    for (int gl = warp; gl < ng; gl += NW) {
      TreeAcc<T, 3, true> t;
      int m = 0;
#pragma unroll 1
      for (int c = 0; c < ROW_GROUP; ++c) {
        const int b = p0 + ((g0 + gl) * ROW_GROUP + c) * ROW_CHUNK;
        if (b >= p1) break;
        const int n = min(ROW_CHUNK, p1 - b);
        T v[ROW_CHUNK], x[ROW_CHUNK];
#pragma unroll
        for (int u = 0; u < ROW_CHUNK; ++u) {
          v[u] = u < n ? __ldg(val + b + u) : T(0);
          x[u] = u < n ? gather(__ldg(colind + b + u)) : T(0);
        }
        T P = T(0);
#pragma unroll
        for (int u = 0; u < ROW_CHUNK; ++u)
          if (u < n) P = fmad(v[u], x[u], P);
        t.push(m++, P);
      }
      roots[gl * 32 + lane] = t.finish(m);
    }
    __syncthreads();
    if (warp == 0) {
      TreeAcc<T, 7, true> r;
      for (int gl = 0; gl < ng; ++gl) r.push(gl, roots[gl * 32 + lane]);
      top.push(nround, r.finish(ng));
    }
    __syncthreads();
  }
  return warp == 0 ? top.finish(nround) : T(0);
}

}  // namespace fgb
