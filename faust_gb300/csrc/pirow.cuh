// pirow.cuh — the power iteration's sparse-row order.
//
// Inside the power iteration (one right-hand vector) a row of S x runs over
// the row's stored entries in order, cut into chunks of PI_CHUNK entries:
// each chunk is a sequential fma from +0, and the chunk partials
// P_0 .. P_{M-1} are added by the recursive-halving pairwise tree (at stride
// s = 1, 2, 4, ...: Q_l += Q_{l+s} for l = 0 mod 2s and l + s < M).  A row of
// at most PI_CHUNK entries is one sequential fma chain.  The oracle restates
// the same order (pi_row_dot).
//
// On GB300 one FP64 FMA warp instruction issues every 64 cycles per
// scheduler, so a long row done by one thread costs 64 cycles per entry; the
// chunks let a warp run it as up to 32 chains of 16 entries and a five-level
// tree.
#pragma once

#include "fgb_internal.cuh"

namespace fgb {

constexpr int PI_CHUNK = 16;

// Binary-counter merge of tree leaves arriving in order: level b holds the
// sum of 2^b consecutive leaves.  Pushing leaf number `count` (0-based)
// merges it with the occupied levels given by the bits of count (older + newer),
// which reproduces the recursive-halving tree; finish() combines the
// remaining levels from the lowest (newest) up.
template <typename T, int LEVELS>
struct TreeAcc {
  T lv[LEVELS];
  __device__ __forceinline__ void push(int count, T v) {
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

// One thread, a row of more than PI_CHUNK entries (below 2^16 chunks).
template <typename TC, typename TF>
__device__ __noinline__ TC pi_row_thread_long(const int* __restrict__ ci, const TF* __restrict__ val, int p0, int p1,
                                              const TC* __restrict__ x) {
  TreeAcc<TC, 16> t;
  int m = 0;
  for (int b = p0; b < p1; b += PI_CHUNK, ++m) {
    TC P = TC(0);
    const int e = min(p1, b + PI_CHUNK);
    for (int p = b; p < e; ++p) P = fmad((TC)val[p], x[ci[p]], P);
    t.push(m, P);
  }
  return t.finish(m);
}

// One thread, any row: short rows inline, long ones through the call above.
template <typename TC, typename TF>
__device__ __forceinline__ TC pi_row_thread(const int* __restrict__ ci, const TF* __restrict__ val, int p0, int p1,
                                            const TC* __restrict__ x) {
  if (p1 - p0 > PI_CHUNK) return pi_row_thread_long<TC, TF>(ci, val, p0, p1, x);
  TC acc = TC(0);
  for (int p = p0; p < p1; ++p) acc = fmad((TC)val[p], x[ci[p]], acc);
  return acc;
}

// One warp (all 32 lanes), lane l working on chunks l, l + 32, ...: each
// round of 32 chunks is reduced by the tree over lanes, and the round sums
// merge as leaves of the same tree (a round is an aligned subtree of 32).
// Every lane returns the value.
template <typename TC, typename TF>
__device__ __noinline__ TC pi_row_warp(const int* __restrict__ ci, const TF* __restrict__ val, int p0, int p1,
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

}  // namespace fgb
