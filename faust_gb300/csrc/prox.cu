// prox.cu — projections (faust_prox.hpp) of a dense device matrix, all
// decisions taken on the device so that a palm4msa2 iteration can be replayed
// as a CUDA graph.
//
// Global top-k (prox_sp) reproduces the support std::partial_sort selects
// with the comparator |a| > |b| (faust_prox.hpp:52-69), ties included:
//  1. radix select on magnitude keys gives t (the k-th largest |v|),
//     G = #{|v| > t} and E = #{|v| == t};
//  2. if G + E == k the set is unique; if t == 0 the tied entries are zeros
//     and drop out of the sparse factor whichever are chosen;
//  3. otherwise, with tau the position where the running count of |v| >= t
//     reaches k: when no |v| > t lies after tau, heap selection keeps exactly
//     the entries |v| >= t at positions <= tau (every such entry entered the
//     heap before its minimum reached t, and none was evicted afterwards);
//  4. otherwise the heap itself decides which ties stay: one block replays the
//     selection (make_heap on the first k entries, then each later entry
//     larger than the heap top replaces it through the hole-to-leaf
//     adjustment and sift-up of the standard heap), after a parallel filter
//     that drops entries not larger than the top at the start of each chunk.
// Per-row / per-column top-k (prox_splin / prox_spcol) replay the same heap
// selection per line, one thread per line.
#include <algorithm>
#include <cstring>

#include "prox.cuh"

namespace fgb {

constexpr int PX_THREADS = 256;
constexpr int RS_MAX_PASSES = 6;  // passes of the single-launch radix select
constexpr int RS_LIST_CAP = 32768;  // bucket size the radix select finishes in one block
constexpr int LINE_KMAX = 64;
constexpr int SQ_SEG = 16;                                // segments of a lane's values
constexpr int SQ_PER = (int)(CR_CHUNK / CR_LANES / SQ_SEG);  // values per segment

__device__ __forceinline__ unsigned long long mag_key(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffULL;
}
__device__ __forceinline__ unsigned long long mag_key(float v) {
  return (unsigned long long)(__float_as_uint(v) & 0x7fffffffu);
}
__device__ __forceinline__ unsigned long long raw_bits(double v) { return (unsigned long long)__double_as_longlong(v); }
__device__ __forceinline__ unsigned long long raw_bits(float v) { return __float_as_uint(v); }
template <typename T>
__device__ __forceinline__ T pos_adj(T v, int pos) {
  return (pos && v < T(0)) ? T(0) : v;
}

// Magnitude key of pos_adj(v, pos) by integer operations only (v < 0 is a
// set sign bit on a non-zero, non-NaN value), so that the scans issue no
// floating-point instruction.
__device__ __forceinline__ unsigned long long sel_key(double v, int pos) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned long long m = b & 0x7fffffffffffffffULL;
  return (pos && (b >> 63) && m != 0 && m <= 0x7ff0000000000000ULL) ? 0ULL : m;
}
__device__ __forceinline__ unsigned long long sel_key(float v, int pos) {
  const unsigned b = __float_as_uint(v);
  const unsigned m = b & 0x7fffffffu;
  return (pos && (b >> 31) && m != 0 && m <= 0x7f800000u) ? 0ULL : (unsigned long long)m;
}

// ------------------------------------------------------------------ workspace
fgb_status prox_work_reserve(fgb_ctx* ctx, ProxWork& w, long elems, int rows) {
  if (w.cap_elems >= elems && w.cap_rows >= rows && w.state) return FGB_OK;
  prox_work_free(w);
  FGB_TRY(dmalloc(ctx, (void**)&w.state, sizeof(TopkState)));
  FGB_TRY(dmalloc(ctx, (void**)&w.hist, sizeof(unsigned) * 2048));
  FGB_TRY(dmalloc(ctx, (void**)&w.flags, (size_t)std::max(1L, elems)));
  const long nchunks = (elems + 8191) / 8192 + 2;
  FGB_TRY(dmalloc(ctx, (void**)&w.chunk_cnt, sizeof(long long) * 2 * nchunks));
  FGB_TRY(dmalloc(ctx, (void**)&w.partials, sizeof(double) * (elems / CR_CHUNK + 2)));
  FGB_TRY(dmalloc(ctx, (void**)&w.scal, sizeof(double) * 4));
  FGB_TRY(dmalloc(ctx, (void**)&w.row_cnt, sizeof(int) * (rows + 2)));
  FGB_CUDA(ctx, cudaMemsetAsync(w.row_cnt, 0, sizeof(int) * (rows + 2), ctx->stream));
  FGB_CUDA(ctx, cudaMemsetAsync(w.flags, 0, (size_t)std::max(1L, elems), ctx->stream));
  FGB_CUDA(ctx, cudaMemsetAsync(w.hist, 0, sizeof(unsigned) * 2048, ctx->stream));
  FGB_TRY(dmalloc(ctx, (void**)&w.hist_passes, sizeof(unsigned) * (RS_MAX_PASSES * 2048 + 8)));
  FGB_CUDA(ctx, cudaMemsetAsync(w.hist_passes, 0, sizeof(unsigned) * (RS_MAX_PASSES * 2048 + 8), ctx->stream));
  FGB_TRY(dmalloc(ctx, (void**)&w.rs_list, sizeof(unsigned long long) * RS_LIST_CAP));
  w.sq_chunks = (elems + CR_CHUNK - 1) / CR_CHUNK;
  FGB_TRY(dmalloc(ctx, (void**)&w.sq_seg, sizeof(double) * (size_t)std::max(1L, w.sq_chunks) * SQ_SEG * CR_LANES));
  FGB_TRY(dmalloc(ctx, (void**)&w.sq_mask, sizeof(unsigned) * (size_t)std::max(1L, w.sq_chunks) * CR_LANES));
  FGB_CUDA(ctx, cudaMemsetAsync(w.sq_mask, 0, sizeof(unsigned) * (size_t)std::max(1L, w.sq_chunks) * CR_LANES,
                                ctx->stream));
  FGB_TRY(dmalloc(ctx, (void**)&w.sq_done, sizeof(unsigned) * (size_t)std::max(1L, w.sq_chunks)));
  FGB_CUDA(ctx, cudaMemsetAsync(w.sq_done, 0, sizeof(unsigned) * (size_t)std::max(1L, w.sq_chunks), ctx->stream));
  w.cap_elems = elems;
  w.cap_rows = rows;
  w.growable = 1;
  return FGB_OK;
}

void prox_work_free(ProxWork& w) {
  dfree(w.state);
  dfree(w.hist);
  dfree(w.hist_passes);
  w.hist_passes = nullptr;
  dfree(w.rs_list);
  dfree(w.flags);
  dfree(w.chunk_cnt);
  dfree(w.partials);
  dfree(w.scal);
  dfree(w.row_cnt);
  dfree(w.supp);
  dfree(w.heap);
  dfree(w.cand);
  dfree(w.wbound);
  dfree(w.wcount);
  dfree(w.heap2);
  dfree(w.sq_seg);
  dfree(w.sq_mask);
  dfree(w.sq_done);
  w = ProxWork();
}

// ------------------------------------------------------------------ radix select
// One pass over an 11-bit (or shorter) digit of the magnitude keys whose
// higher bits equal the prefix found so far; the last block to finish picks
// the bucket holding the k_rem-th largest key.
template <typename T>
__global__ void __launch_bounds__(PX_THREADS)
    k_radix_pass(const T* __restrict__ M, long N, int pos, int shift, int bits, TopkState* st,
                 unsigned* __restrict__ hist) {
  __shared__ unsigned sh[2048];
  __shared__ int is_last;
  const int nb = 1 << bits;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const unsigned long long prefix = st->prefix, mask = st->mask;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    const unsigned long long key = sel_key(M[i], pos);
    if ((key & mask) == prefix) atomicAdd(&sh[(key >> shift) & (nb - 1)], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) is_last = (atomicAdd(&st->blocks_done, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    sh[i] = __ldcg(&hist[i]);
    hist[i] = 0;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    const int per = nb / 32;
    unsigned long long s = 0;
    for (int j = 0; j < per; ++j) s += sh[nb - 1 - (lane * per + j)];
    unsigned long long incl = s;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const unsigned long long excl = incl - s;
    const long long krem = st->k_rem;
    const unsigned ball = __ballot_sync(0xffffffffu, (long long)excl < krem && krem <= (long long)incl);
    const int L = ball ? __ffs(ball) - 1 : -1;
    if (lane == L) {
      unsigned long long cum = excl;
      for (int j = 0; j < per; ++j) {
        const int b = nb - 1 - (lane * per + j);
        const unsigned long long h = sh[b];
        if ((long long)(cum + h) >= krem) {
          st->G += (long long)cum;
          st->k_rem = krem - (long long)cum;
          st->prefix = prefix | ((unsigned long long)b << shift);
          st->mask = mask | ((unsigned long long)(nb - 1) << shift);
          st->E = (long long)h;
          break;
        }
        cum += h;
      }
    }
    if (L < 0 && lane == 0) st->status = FGB_ERR_INVALID_ARG;
  }
  if (threadIdx.x == 0) st->blocks_done = 0;
}

// ------------------------------------------------------------------ radix select, one launch
// All the passes of the radix select in one cooperative launch: per pass,
// every block histograms its share of the keys that match the prefix, adds
// its bins to the pass's global histogram, waits at a grid barrier, and then
// every block reads the histogram and picks the bucket itself (the same
// choice everywhere), so only one barrier per pass is needed (the clearing
// of the histograms is described at k_radix_select).  The barrier wait is
// bounded: on time-out the state's status is set to FGB_ERR_TIMEOUT.
__device__ __forceinline__ bool rs_grid_barrier(unsigned* bar, unsigned nblocks, int* s_ok) {
  __syncthreads();
  if (threadIdx.x == 0) {
    bool ok = true;
    volatile unsigned* gen = bar + 1;
    const unsigned g0 = *gen;
    __threadfence();
    if (atomicAdd(&bar[0], 1u) == nblocks - 1) {
      bar[0] = 0;
      __threadfence();
      atomicAdd(&bar[1], 1u);
    } else {
      long spins = 0;
      while (*gen == g0) {
        if (++spins > (1L << 21)) {
          ok = false;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    *s_ok = ok;
  }
  __syncthreads();
  return *s_ok != 0;
}

struct RsShared {
  unsigned long long prefix, mask;
  long long krem, G, E;
  int ok, bad;
  unsigned long long wsum[PX_THREADS / 32];
};

// The bucket of the histogram sh[0..nb) holding the k_rem-th largest key,
// found by every block alike: thread t owns bins nb-1-t*per .. nb-per-t*per
// (descending), a block scan of their sums finds the owner, which walks its
// bins and narrows the prefix.  Every thread of the block calls.
__device__ __forceinline__ void rs_pick(const unsigned* sh, int nb, int shift, unsigned long long prefix,
                                        unsigned long long mask, RsShared& s) {
  const int per = nb / PX_THREADS;  // 8, 2 or 1
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  unsigned long long sum = 0;
  for (int j = 0; j < per; ++j) sum += sh[nb - 1 - (t * per + j)];
  unsigned long long incl = sum;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s.wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    unsigned long long w = lane < PX_THREADS / 32 ? s.wsum[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < PX_THREADS / 32) s.wsum[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  incl += warp ? s.wsum[warp - 1] : 0ULL;
  const unsigned long long excl = incl - sum;
  const long long krem = s.krem;
  const long long total = (long long)s.wsum[PX_THREADS / 32 - 1];
  __syncthreads();  // everyone has read s.krem before the owner updates it
  if ((long long)excl < krem && krem <= (long long)incl) {
    unsigned long long cum = excl;
    for (int j = 0; j < per; ++j) {
      const int b = nb - 1 - (t * per + j);
      const unsigned long long h = sh[b];
      if ((long long)(cum + h) >= krem) {
        s.G += (long long)cum;
        s.krem = krem - (long long)cum;
        s.prefix = prefix | ((unsigned long long)b << shift);
        s.mask = mask | ((unsigned long long)(nb - 1) << shift);
        s.E = (long long)h;
        break;
      }
      cum += h;
    }
  }
  if (t == 0 && total < krem) s.bad = 1;
  __syncthreads();
}

// Pass p of the grid histograms the keys matching the prefix of passes
// 0..p-1.  Pass 0 matches every key and its bins cluster (they are the
// exponent bits), so its shared-memory increments are aggregated per warp.
// When the bucket chosen so far holds at most RS_LIST_CAP keys and passes
// remain, the pass also appends those keys to `list`; after its barrier
// block 0 alone runs the remaining passes over the list (the other blocks
// return), which replaces the last full scans and barriers by block-local
// passes over a few thousand keys.  The list counter is the word after the
// barrier's two; block 0 clears it and the histograms of passes 1.. at the
// start (no block touches them before the first barrier), histogram p-1
// after barrier p.  Block 0 also resets the selection state the later
// kernels read (k comes as an argument), so no separate reset launch is
// needed.
template <typename T>
__global__ void __launch_bounds__(PX_THREADS)
    k_radix_select(const T* __restrict__ M, long N, int pos, int npass, long long k, TopkState* st, unsigned* hists,
                   unsigned long long* __restrict__ list) {
  __shared__ unsigned sh[2048];
  __shared__ RsShared s;
  unsigned* bar = hists + RS_MAX_PASSES * 2048;
  unsigned* list_n = bar + 2;
  const int shifts8[6] = {52, 41, 30, 19, 8, 0}, bits8[6] = {11, 11, 11, 11, 11, 8};
  const int shifts4[3] = {20, 9, 0}, bits4[3] = {11, 11, 9};
  if (threadIdx.x == 0) {
    s.prefix = 0;
    s.mask = 0;
    s.krem = k;
    s.G = 0;
    s.E = 0;
    s.bad = 0;
  }
  if (blockIdx.x == 0) {
    for (int i = threadIdx.x; i < (RS_MAX_PASSES - 1) * 2048; i += blockDim.x) hists[2048 + i] = 0;
    if (threadIdx.x == 0) {
      // the state fields later kernels read (no block writes the state
      // before its first barrier)
      *list_n = 0;
      st->t = 0;
      st->tau = 0;
      st->sel_case = 0;
      st->status = 0;
      st->blocks_done = 0;
    }
  }
  bool timed_out = false, tail = false;
  int p = 0;
  for (; p < npass; ++p) {
    const int shift = sizeof(T) == 8 ? shifts8[p] : shifts4[p];
    const int bits = sizeof(T) == 8 ? bits8[p] : bits4[p];
    const int nb = 1 << bits;
    unsigned* hist = hists + p * 2048;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) sh[i] = 0;
    __syncthreads();
    const unsigned long long prefix = s.prefix, mask = s.mask;
    const bool collect = p > 0 && p + 1 < npass && s.E <= RS_LIST_CAP;
    {
      // eight keys per thread in flight before their atomics
      const long stride = (long)gridDim.x * blockDim.x;
      long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
      if (p == 0) {
        for (; i + 7 * stride < N; i += 8 * stride) {
          unsigned long long key[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) key[u] = sel_key(M[i + u * stride], pos);
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const unsigned b = (unsigned)(key[u] >> shift) & (unsigned)(nb - 1);
            const unsigned peers = __match_any_sync(__activemask(), b);
            if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&sh[b], (unsigned)__popc(peers));
          }
        }
        for (; i < N; i += stride) atomicAdd(&sh[(sel_key(M[i], pos) >> shift) & (nb - 1)], 1u);
      } else {
        for (; i + 7 * stride < N; i += 8 * stride) {
          unsigned long long key[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) key[u] = sel_key(M[i + u * stride], pos);
#pragma unroll
          for (int u = 0; u < 8; ++u)
            if ((key[u] & mask) == prefix) {
              atomicAdd(&sh[(key[u] >> shift) & (nb - 1)], 1u);
              if (collect) {
                const unsigned at = atomicAdd(list_n, 1u);
                if (at < (unsigned)RS_LIST_CAP) list[at] = key[u];
              }
            }
        }
        for (; i < N; i += stride) {
          const unsigned long long key = sel_key(M[i], pos);
          if ((key & mask) == prefix) {
            atomicAdd(&sh[(key >> shift) & (nb - 1)], 1u);
            if (collect) {
              const unsigned at = atomicAdd(list_n, 1u);
              if (at < (unsigned)RS_LIST_CAP) list[at] = key;
            }
          }
        }
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nb; i += blockDim.x)
      if (sh[i]) atomicAdd(&hist[i], sh[i]);
    __threadfence();
    if (!rs_grid_barrier(bar, gridDim.x, &s.ok)) timed_out = true;
    if (p > 0 && blockIdx.x == 0)
      for (int i = threadIdx.x; i < 2048; i += blockDim.x) hists[(p - 1) * 2048 + i] = 0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) sh[i] = __ldcg(&hist[i]);
    __syncthreads();
    rs_pick(sh, nb, shift, prefix, mask, s);
    if (collect) {
      ++p;
      tail = true;
      break;
    }
  }
  if (tail && blockIdx.x == 0) {
    const unsigned n = min(__ldcg(list_n), (unsigned)RS_LIST_CAP);
    for (; p < npass; ++p) {
      const int shift = sizeof(T) == 8 ? shifts8[p] : shifts4[p];
      const int bits = sizeof(T) == 8 ? bits8[p] : bits4[p];
      const int nb = 1 << bits;
      for (int i = threadIdx.x; i < nb; i += blockDim.x) sh[i] = 0;
      __syncthreads();
      const unsigned long long prefix = s.prefix, mask = s.mask;
      for (unsigned i = threadIdx.x; i < n; i += blockDim.x) {
        const unsigned long long key = __ldcg(&list[i]);
        if ((key & mask) == prefix) atomicAdd(&sh[(key >> shift) & (nb - 1)], 1u);
      }
      __syncthreads();
      rs_pick(sh, nb, shift, prefix, mask, s);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->prefix = s.prefix;
    st->mask = s.mask;
    st->k_rem = s.krem;
    st->G = s.G;
    st->E = s.E;
    if (s.bad) atomicCAS(&st->status, 0, (int)FGB_ERR_INVALID_ARG);
  }
  if (timed_out && threadIdx.x == 0) atomicCAS(&st->status, 0, (int)FGB_ERR_TIMEOUT);
  // The last block to leave clears the barrier's arrival count.  After a
  // barrier time-out the late blocks' arrivals can leave it non-zero, and
  // the next launch on this workspace would then release a barrier early.
  // Every block has passed all its barriers once it counts itself out here.
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&bar[3], 1u) == gridDim.x - 1) {
      bar[0] = 0;
      bar[3] = 0;
      __threadfence();
    }
  }
}

// The same selection with every thread's keys held in registers (at most
// RS_KREG per thread, i.e. N <= grid threads * RS_KREG; one block per SM, so
// that fewer blocks meet at each grid barrier and merge their histograms):
// each full pass reads registers instead of the matrix.  Once the chosen bucket holds at
// most RS_TAIL_CAP keys, every block appends its keys of that bucket to the
// list straight from its registers and counts itself in; block 0 alone
// waits for all the blocks (a one-sided, bounded wait) and finishes the
// remaining digits from the list staged in shared memory.  The histograms,
// bucket picks and outputs are those of k_radix_select.
constexpr int RS_KREG = 32;
constexpr int RS_TAIL_CAP = 4096;

template <typename T>
__global__ void __launch_bounds__(PX_THREADS, 1)
    k_radix_select_reg(const T* __restrict__ M, long N, int pos, int npass, long long k, TopkState* st,
                       unsigned* hists, unsigned long long* __restrict__ list) {
  __shared__ unsigned sh[2048];
  __shared__ RsShared s;
  __shared__ unsigned long long tl[RS_TAIL_CAP];
  unsigned* bar = hists + RS_MAX_PASSES * 2048;
  unsigned* list_n = bar + 2;
  unsigned* arrived = bar + 4;  // blocks whose keys are in the list
  const int shifts8[6] = {52, 41, 30, 19, 8, 0}, bits8[6] = {11, 11, 11, 11, 11, 8};
  const int shifts4[3] = {20, 9, 0}, bits4[3] = {11, 11, 9};
  if (threadIdx.x == 0) {
    s.prefix = 0;
    s.mask = 0;
    s.krem = k;
    s.G = 0;
    s.E = 0;
    s.bad = 0;
  }
  if (blockIdx.x == 0) {
    for (int i = threadIdx.x; i < (RS_MAX_PASSES - 1) * 2048; i += blockDim.x) hists[2048 + i] = 0;
    if (threadIdx.x == 0) {
      // (no block touches these before the first barrier)
      *list_n = 0;
      *arrived = 0;
      st->t = 0;
      st->tau = 0;
      st->sel_case = 0;
      st->status = 0;
      st->blocks_done = 0;
    }
  }
  // the thread's keys, in the order of the strided scans
  const long stride = (long)gridDim.x * blockDim.x;
  const long i0 = blockIdx.x * (long)blockDim.x + threadIdx.x;
  unsigned long long key[RS_KREG];
  int nk = 0;
#pragma unroll
  for (int u = 0; u < RS_KREG; ++u) {
    const long i = i0 + u * stride;
    key[u] = i < N ? sel_key(M[i], pos) : 0ULL;
    nk += i < N;
  }
  bool timed_out = false, tail = false;
  int p = 0;
  for (; p < npass; ++p) {
    const int shift = sizeof(T) == 8 ? shifts8[p] : shifts4[p];
    const int bits = sizeof(T) == 8 ? bits8[p] : bits4[p];
    const int nb = 1 << bits;
    unsigned* hist = hists + p * 2048;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) sh[i] = 0;
    __syncthreads();
    const unsigned long long prefix = s.prefix, mask = s.mask;
    if (p == 0) {
#pragma unroll
      for (int u = 0; u < RS_KREG; ++u)
        if (u < nk) {
          const unsigned b = (unsigned)(key[u] >> shift) & (unsigned)(nb - 1);
          const unsigned peers = __match_any_sync(__activemask(), b);
          if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&sh[b], (unsigned)__popc(peers));
        }
    } else {
#pragma unroll
      for (int u = 0; u < RS_KREG; ++u)
        if (u < nk && (key[u] & mask) == prefix) atomicAdd(&sh[(key[u] >> shift) & (nb - 1)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nb; i += blockDim.x)
      if (sh[i]) atomicAdd(&hist[i], sh[i]);
    __threadfence();
    if (!rs_grid_barrier(bar, gridDim.x, &s.ok)) timed_out = true;
    if (p > 0 && blockIdx.x == 0)
      for (int i = threadIdx.x; i < 2048; i += blockDim.x) hists[(p - 1) * 2048 + i] = 0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) sh[i] = __ldcg(&hist[i]);
    __syncthreads();
    rs_pick(sh, nb, shift, prefix, mask, s);
    if (p + 1 < npass && s.E <= RS_TAIL_CAP) {
      tail = true;
      break;
    }
  }
  if (tail) {
    // the keys of the bucket just chosen (s.E of them over the grid)
    const unsigned long long prefix = s.prefix, mask = s.mask;
#pragma unroll
    for (int u = 0; u < RS_KREG; ++u)
      if (u < nk && (key[u] & mask) == prefix) {
        const unsigned at = atomicAdd(list_n, 1u);
        if (at < (unsigned)RS_TAIL_CAP) list[at] = key[u];
      }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(arrived, 1u);
    if (blockIdx.x == 0) {
      if (threadIdx.x == 0) {
        volatile unsigned* arr = arrived;
        long spins = 0;
        bool ok = true;
        while (*arr < gridDim.x) {
          if (++spins > (1L << 21)) {
            ok = false;
            break;
          }
          __nanosleep(64);
        }
        __threadfence();
        s.ok = ok;
      }
      __syncthreads();
      if (!s.ok) timed_out = true;
      // every block has read histogram p: clear it for the next launch
      for (int i = threadIdx.x; i < 2048; i += blockDim.x) hists[p * 2048 + i] = 0;
      const unsigned n = min(__ldcg(list_n), (unsigned)RS_TAIL_CAP);
      for (unsigned i = threadIdx.x; i < n; i += blockDim.x) tl[i] = __ldcg(&list[i]);
      for (++p; p < npass; ++p) {
        const int shift = sizeof(T) == 8 ? shifts8[p] : shifts4[p];
        const int bits = sizeof(T) == 8 ? bits8[p] : bits4[p];
        const int nb = 1 << bits;
        for (int i = threadIdx.x; i < nb; i += blockDim.x) sh[i] = 0;
        __syncthreads();
        const unsigned long long pf = s.prefix, mk = s.mask;
        for (unsigned i = threadIdx.x; i < n; i += blockDim.x) {
          const unsigned long long kk = tl[i];
          if ((kk & mk) == pf) atomicAdd(&sh[(kk >> shift) & (nb - 1)], 1u);
        }
        __syncthreads();
        rs_pick(sh, nb, shift, pf, mk, s);
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->prefix = s.prefix;
    st->mask = s.mask;
    st->k_rem = s.krem;
    st->G = s.G;
    st->E = s.E;
    if (s.bad) atomicCAS(&st->status, 0, (int)FGB_ERR_INVALID_ARG);
  }
  if (timed_out && threadIdx.x == 0) atomicCAS(&st->status, 0, (int)FGB_ERR_TIMEOUT);
  // the last block to leave clears the barrier's arrival count (as in
  // k_radix_select)
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&bar[3], 1u) == gridDim.x - 1) {
      bar[0] = 0;
      bar[3] = 0;
      __threadfence();
    }
  }
}

// ------------------------------------------------------------------ tie case
// Decides the tie case; for ties with t > 0 finds tau and whether an entry
// |v| > t lies after it.
template <typename T>
__global__ void __launch_bounds__(PX_THREADS)
    k_tie_case(const T* __restrict__ M, long N, int pos, long chunk, TopkState* st, long long* __restrict__ cnt) {
  __shared__ int is_last;
  __shared__ long long s_ge[PX_THREADS], s_gt[PX_THREADS];
  __shared__ long long c_target, c_base_gt, c_idx;
  const unsigned long long t = st->prefix;
  const long long k_rem = st->k_rem, E = st->E, G = st->G;
  if (E == k_rem || t == 0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->t = t;
      st->sel_case = (E == k_rem) ? 0 : 3;
    }
    return;
  }
  const long k = G + k_rem;
  // per-chunk counts of keys >= t and > t
  const long c0 = blockIdx.x * chunk, c1 = min(N, c0 + chunk);
  long long ge = 0, gt = 0;
  for (long i = c0 + threadIdx.x; i < c1; i += blockDim.x) {
    const unsigned long long key = sel_key(M[i], pos);
    ge += key >= t;
    gt += key > t;
  }
  s_ge[threadIdx.x] = ge;
  s_gt[threadIdx.x] = gt;
  __syncthreads();
  for (int s = PX_THREADS / 2; s >= 1; s >>= 1) {
    if (threadIdx.x < s) {
      s_ge[threadIdx.x] += s_ge[threadIdx.x + s];
      s_gt[threadIdx.x] += s_gt[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    cnt[2 * blockIdx.x] = s_ge[0];
    cnt[2 * blockIdx.x + 1] = s_gt[0];
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) is_last = (atomicAdd(&st->blocks_done, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  if (threadIdx.x == 0) {
    long long cum_ge = 0, cum_gt = 0;
    long idx = -1;
    for (long b = 0; b < gridDim.x; ++b) {
      const long long g = __ldcg(&cnt[2 * b]), h = __ldcg(&cnt[2 * b + 1]);
      if (cum_ge + g >= k) {
        idx = b;
        break;
      }
      cum_ge += g;
      cum_gt += h;
    }
    c_idx = idx;
    c_target = k - cum_ge;  // rank of tau inside the chunk (1-based)
    c_base_gt = cum_gt;
  }
  __syncthreads();
  if (c_idx < 0) {
    if (threadIdx.x == 0) st->status = FGB_ERR_INVALID_ARG;
    return;
  }
  // exact tau inside chunk c_idx: each thread takes a contiguous slice
  const long b0 = c_idx * chunk, b1 = min(N, b0 + chunk);
  const long len = b1 - b0, per = (len + PX_THREADS - 1) / PX_THREADS;
  const long s0 = b0 + threadIdx.x * per, s1 = min(b1, s0 + per);
  ge = 0;
  gt = 0;
  for (long i = s0; i < s1; ++i) {
    const unsigned long long key = sel_key(M[i], pos);
    ge += key >= t;
    gt += key > t;
  }
  s_ge[threadIdx.x] = ge;
  s_gt[threadIdx.x] = gt;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long run_ge = 0, run_gt = 0;
    int who = -1;
    for (int u = 0; u < PX_THREADS; ++u) {
      if (run_ge + s_ge[u] >= c_target) {
        who = u;
        break;
      }
      run_ge += s_ge[u];
      run_gt += s_gt[u];
    }
    s_ge[0] = who;
    s_gt[0] = run_ge;
    s_gt[1] = run_gt;
    if (who < 0) st->status = FGB_ERR_INVALID_ARG;
  }
  __syncthreads();
  if ((long long)threadIdx.x == s_ge[0]) {
    long long run_ge = s_gt[0], run_gt = s_gt[1];
    for (long i = s0; i < s1; ++i) {
      const unsigned long long key = sel_key(M[i], pos);
      run_ge += key >= t;
      run_gt += key > t;
      if (run_ge == c_target) {
        const long long gt_before = c_base_gt + run_gt;
        st->tau = i;
        st->t = t;
        st->sel_case = (gt_before == G) ? 1 : 2;
        break;
      }
    }
  }
  if (threadIdx.x == 0) st->blocks_done = 0;
}

// ------------------------------------------------------------------ heap replay
// A heap node: magnitude key and position, read and written as one 16-byte
// shared-memory access.
struct __align__(16) HNode {
  unsigned long long key;
  long long idx;
};

struct HeapView {
  HNode* n;
};

// Standard binary-heap adjustment with the comparator "larger key first":
// move the hole to a leaf along the child preferred by the comparator (the
// left child only when it is strictly preferred), then sift the value up.
__device__ void heap_adjust(HeapView h, int hole, int len, HNode v) {
  const int top = hole;
  int child = hole;
  while (child < (len - 1) / 2) {
    child = 2 * (child + 1);
    const HNode r = h.n[child], l = h.n[child - 1];
    if (r.key > l.key) {
      h.n[hole] = l;
      child--;
    } else {
      h.n[hole] = r;
    }
    hole = child;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    h.n[hole] = h.n[child - 1];
    hole = child - 1;
  }
  int parent = (hole - 1) / 2;
  while (hole > top) {
    const HNode pn = h.n[parent];
    if (!(pn.key > v.key)) break;
    h.n[hole] = pn;
    hole = parent;
    parent = (hole - 1) / 2;
  }
  h.n[hole] = v;
}

// The same adjustment with a two-level lookahead: both children and all
// their children are read in one batch of independent shared-memory loads,
// so the descent takes one round trip per two levels.  The moves are exactly
// those of heap_adjust.
__host__ __device__ inline void heap_adjust2(HeapView h, int hole, int len, HNode v) {
  const int top = hole;
  const int lim = (len - 1) / 2;
  int child = hole;
  while (child < lim) {
    const int r1 = 2 * (child + 1), l1 = r1 - 1;
    const HNode nr = h.n[r1], nl = h.n[l1];
    const bool rhas = r1 < lim, lhas = l1 < lim;
    HNode rr, rl, lr, ll;
    if (rhas) {
      rr = h.n[2 * (r1 + 1)];
      rl = h.n[2 * (r1 + 1) - 1];
    }
    if (lhas) {
      lr = h.n[2 * (l1 + 1)];
      ll = h.n[2 * (l1 + 1) - 1];
    }
    int c = r1;
    HNode cn = nr;
    bool chas = rhas;
    HNode gr = rr, gl = rl;
    if (nr.key > nl.key) {
      c = l1;
      cn = nl;
      chas = lhas;
      gr = lr;
      gl = ll;
    }
    h.n[hole] = cn;
    hole = c;
    child = c;
    if (!chas) break;
    const int r2 = 2 * (c + 1);
    int c2 = r2;
    HNode c2n = gr;
    if (gr.key > gl.key) {
      c2 = r2 - 1;
      c2n = gl;
    }
    h.n[hole] = c2n;
    hole = c2;
    child = c2;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    h.n[hole] = h.n[child - 1];
    hole = child - 1;
  }
  int parent = (hole - 1) / 2;
  while (hole > top) {
    const HNode pn = h.n[parent];
    if (!(pn.key > v.key)) break;
    h.n[hole] = pn;
    hole = parent;
    parent = (hole - 1) / 2;
  }
  h.n[hole] = v;
}

constexpr int HR_CHUNK = 8192;
constexpr int HR_PER = HR_CHUNK / PX_THREADS;  // 32 entries per thread

template <typename T>
__global__ void __launch_bounds__(PX_THREADS)
    k_heap_replay(const T* __restrict__ M, long N, int pos, int k, TopkState* st, unsigned char* __restrict__ flags,
                  HNode* gheap, int use_smem) {
  if (st->sel_case != 2) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int warp_tot[PX_THREADS / 32];
  __shared__ int s_ncand;
  HNode* cand = reinterpret_cast<HNode*>(smem_raw);  // HR_CHUNK candidates
  HeapView h;
  h.n = use_smem ? cand + HR_CHUNK : gheap;
  for (int i = threadIdx.x; i < k; i += blockDim.x) h.n[i] = HNode{sel_key(M[i], pos), i};
  __syncthreads();
  if (threadIdx.x == 0 && k >= 2) {
    int parent = (k - 2) / 2;
    while (true) {
      heap_adjust2(h, parent, k, h.n[parent]);
      if (parent == 0) break;
      parent--;
    }
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (long c0 = k; c0 < N; c0 += HR_CHUNK) {
    const unsigned long long topk = h.n[0].key;
    const long c1 = min(N, c0 + HR_CHUNK);
    // parallel filter (a key not above the current top can never enter):
    // thread t looks at entries c0 + t + 256*u, keeping chunk order per warp
    // slice through a two-level scan
    unsigned long long kk[HR_PER];
    int cnt = 0;
    const long base = c0 + (long)threadIdx.x * HR_PER;
#pragma unroll
    for (int u = 0; u < HR_PER; ++u) {
      const long i = base + u;
      kk[u] = (i < c1) ? sel_key(M[i], pos) : 0ULL;
      cnt += (i < c1) && kk[u] > topk;
    }
    if (__syncthreads_count(cnt) == 0) continue;
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
      int run = 0;
      for (int w = 0; w < PX_THREADS / 32; ++w) {
        const int t = warp_tot[w];
        warp_tot[w] = run;
        run += t;
      }
      s_ncand = run;
    }
    __syncthreads();
    int off = warp_tot[warp] + incl - cnt;
#pragma unroll
    for (int u = 0; u < HR_PER; ++u) {
      const long i = base + u;
      if (i < c1 && kk[u] > topk) cand[off++] = HNode{kk[u], i};
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const int nc = s_ncand;
      unsigned long long top = h.n[0].key;
      for (int q = 0; q < nc; ++q) {
        const HNode c = cand[q];
        if (c.key > top) {
          heap_adjust2(h, 0, k, c);
          top = h.n[0].key;
        }
      }
    }
    __syncthreads();
  }
  const unsigned long long t = st->t;
  for (int i = threadIdx.x; i < k; i += blockDim.x)
    if (h.n[i].key == t) flags[h.n[i].idx] = 1;
}

// ------------------------------------------------------------------ tie replay with a parallel pre-filter
// The same selection as k_heap_replay, split so that only the sequential
// part stays on one SM:
//
//  1. k_rp_bounds (one block per window of the linear order): a lower bound
//     of the k-th largest key of the window, from two 12-bit histograms.
//  2. k_rp_filter (one block per window): an entry i >= k can enter the heap
//     only if its key exceeds the heap top at its arrival, and that top is at
//     least the k-th largest key of every earlier window and at least the
//     initial top (the smallest of the first k keys).  Entries above the
//     largest of those bounds are kept, in linear order, in the window's
//     own slot range of the candidate array.
//  3. k_rp_replay (one block): make_heap of the first k keys, level by level
//     in parallel (subtrees of one level are disjoint, so the order of
//     libstdc++'s loop does not matter among them), then one warp replays
//     every candidate against the live top.  A replacement of the top runs
//     __adjust_heap + __push_heap as a warp: the hole's path to a leaf
//     (the preferred child of each node, the left one only when its key is
//     strictly smaller) is found five levels per round from a ballot of the
//     preferences of a 31-node subtree, and because keys grow along that
//     path, the sift-up of the new key is one more ballot.
//
// Windows: [0, 2k), [2k, 4k), [4k, 8k), ... doubling up to wmax entries,
// then wmax entries each.
constexpr int RP_BLOCK = 512;
constexpr int RP_BINS = 4096;
constexpr int RP_STAGE = 2048;
constexpr int RP_MAXWIN = 1024;

// Entries of each heap array (keys, positions): node n at n + 1, padded so
// that reading the two children of any node below k (entries 2n + 2, 2n + 3)
// and the two-level look-ahead of rp_insert (up to 4 * lim + 7) stay inside.
__host__ __device__ inline long rp_key_len(long k) { return ((2 * k + 8) + 1) & ~1L; }

__host__ __device__ inline void rp_window(long i, long N, long k, long wmax, long* lo, long* hi) {
  long s = 0, len = 2 * k;
  long j = 0;
  while (j < i && len < wmax) {
    s += len;
    len = s < wmax ? s : wmax;
    ++j;
  }
  if (j < i) s += (i - j) * len;
  *lo = s < N ? s : N;
  *hi = s + len < N ? s + len : N;
}

static long rp_wmax(long N, long k) {
  long w = std::max(65536L, 2 * k);
  w = std::max(w, (N + 511) / 512);
  return (w + 255) / 256 * 256;
}

static int rp_window_count(long N, long k, long wmax) {
  int n = 0;
  long lo, hi;
  do {
    rp_window(n, N, k, wmax, &lo, &hi);
    ++n;
  } while (hi < N);
  return n;
}

// Block-wide (RP_BLOCK threads): the bin of the need-th largest key of a
// histogram with bins in increasing key order, and the count above it.
__device__ void rp_find_bin(const unsigned* hist, long need, int* s_bin, long* s_above, long* s_warp) {
  constexpr int PER = RP_BINS / RP_BLOCK;  // 8 bins per thread, thread 0 holds the top ones
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  long mine = 0;
  for (int q = 0; q < PER; ++q) mine += hist[RP_BINS - 1 - (t * PER + q)];
  long incl = mine;
  for (int o = 1; o < 32; o <<= 1) {
    const long y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (t == 0) {
    long run = 0;
    for (int w = 0; w < RP_BLOCK / 32; ++w) {
      const long x = s_warp[w];
      s_warp[w] = run;
      run += x;
    }
  }
  __syncthreads();
  const long before = s_warp[warp] + incl - mine;  // keys in higher bins than this thread's
  if (before < need && before + mine >= need) {
    long acc = before;
    for (int q = 0; q < PER; ++q) {
      const int b = RP_BINS - 1 - (t * PER + q);
      if (acc + hist[b] >= need) {
        *s_bin = b;
        *s_above = acc;
        break;
      }
      acc += hist[b];
    }
  }
  __syncthreads();
}

// Warp-aggregated shared-memory histogram increment (every lane calls it).
__device__ __forceinline__ void rp_hist_add(unsigned* hist, unsigned bin, bool valid) {
  const unsigned key = valid ? bin : 0xffffffffu;
  const unsigned same = __match_any_sync(0xffffffffu, key);
  const int lane = threadIdx.x & 31;
  if (valid && (__ffs(same) - 1) == lane) atomicAdd(&hist[bin], (unsigned)__popc(same));
}

template <typename T>
__global__ void __launch_bounds__(RP_BLOCK)
    k_rp_bounds(const T* __restrict__ M, long N, int pos, long k, long wmax, const TopkState* st,
                unsigned long long* __restrict__ wb) {
  if (st->sel_case != 2) return;
  __shared__ unsigned hist[RP_BINS];
  __shared__ int s_bin;
  __shared__ long s_above, s_warp[RP_BLOCK / 32];
  long lo, hi;
  rp_window(blockIdx.x, N, k, wmax, &lo, &hi);
  if (hi - lo < k) {
    if (threadIdx.x == 0) wb[blockIdx.x] = 0;
    return;
  }
  constexpr int KB = (int)sizeof(T) * 8;
  constexpr int S1 = KB - 12, S2 = KB - 24;
  unsigned long long bound = 0;
  long need = k;
  for (int pass = 0; pass < 2; ++pass) {
    for (int i = threadIdx.x; i < RP_BINS; i += RP_BLOCK) hist[i] = 0;
    if (threadIdx.x == 0) s_bin = 0;
    __syncthreads();
    for (long b0 = lo; b0 < hi; b0 += RP_BLOCK) {
      const long i = b0 + threadIdx.x;
      const bool in = i < hi;
      const unsigned long long key = in ? sel_key(M[i], pos) : 0ULL;
      const bool take = in && (pass == 0 || (key >> S1) == (bound >> S1));
      const unsigned bin = (unsigned)((pass == 0 ? key >> S1 : key >> S2) & (RP_BINS - 1));
      rp_hist_add(hist, bin, take);
    }
    __syncthreads();
    rp_find_bin(hist, need, &s_bin, &s_above, s_warp);
    if (pass == 0) {
      bound = (unsigned long long)s_bin << S1;
      need -= s_above;
    } else {
      bound |= (unsigned long long)s_bin << S2;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) wb[blockIdx.x] = bound;
}

template <typename T>
__global__ void __launch_bounds__(RP_BLOCK)
    k_rp_filter(const T* __restrict__ M, long N, int pos, long k, long wmax, const TopkState* st,
                const unsigned long long* __restrict__ wb, HNode* __restrict__ cand, int* __restrict__ wcnt) {
  if (st->sel_case != 2) return;
  constexpr int U = 8, NW = RP_BLOCK / 32;
  __shared__ unsigned long long s_min[NW];
  __shared__ unsigned long long s_bound;
  __shared__ int s_cnt[U * NW];
  __shared__ int s_total;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  long lo, hi;
  rp_window(blockIdx.x, N, k, wmax, &lo, &hi);
  // initial top: the smallest of the first k keys
  unsigned long long mn = ~0ULL;
  for (long i = t; i < k; i += RP_BLOCK) {
    const unsigned long long key = sel_key(M[i], pos);
    mn = key < mn ? key : mn;
  }
  for (int o = 16; o >= 1; o >>= 1) {
    const unsigned long long y = __shfl_xor_sync(0xffffffffu, mn, o);
    mn = y < mn ? y : mn;
  }
  if (lane == 0) s_min[warp] = mn;
  __syncthreads();
  if (t == 0) {
    unsigned long long b = ~0ULL;
    for (int w = 0; w < NW; ++w) b = s_min[w] < b ? s_min[w] : b;
    for (int w = 0; w < (int)blockIdx.x; ++w) b = wb[w] > b ? wb[w] : b;
    s_bound = b;
  }
  __syncthreads();
  const unsigned long long bound = s_bound;
  const long start = lo > k ? lo : k;
  int total = 0;
  const unsigned lt = (1u << lane) - 1u;
  for (long tb = start; tb < hi; tb += (long)U * RP_BLOCK) {
    unsigned long long kk[U];
    unsigned bal[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const long e = tb + (long)u * RP_BLOCK + t;
      kk[u] = e < hi ? sel_key(M[e], pos) : 0ULL;
      bal[u] = __ballot_sync(0xffffffffu, e < hi && kk[u] > bound);
      if (lane == 0) s_cnt[u * NW + warp] = __popc(bal[u]);
    }
    __syncthreads();
    if (warp == 0) {
      // exclusive scan of the U * NW counts in (u, warp) order: lane owns 4
      int v[4], sum = 0;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        v[q] = s_cnt[lane * 4 + q];
        sum += v[q];
      }
      int incl = sum;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      int run = incl - sum;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        s_cnt[lane * 4 + q] = run;
        run += v[q];
      }
      if (lane == 31) s_total = incl;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if ((bal[u] >> lane) & 1u) {
        const long e = tb + (long)u * RP_BLOCK + t;
        const int o = total + s_cnt[u * NW + warp] + __popc(bal[u] & lt);
        cand[lo + o] = HNode{kk[u], e};
      }
    }
    total += s_total;
    __syncthreads();
  }
  if (t == 0) wcnt[blockIdx.x] = total;
}

// libstdc++ __adjust_heap(first, hole, len, first[hole]) + __push_heap with
// comp(a, b) = a.key > b.key, one thread, on the split heap (node n at
// storage n + 1).
__device__ void rp_adjust(unsigned long long* hk, unsigned* hidx, int hole, int lim, int half) {
  const unsigned long long vk = hk[hole + 1];
  const unsigned vi = hidx[hole + 1];
  const int top = hole;
  int child = hole;
  while (child < lim) {
    child = 2 * (child + 1);
    if (hk[child + 1] > hk[child]) child--;
    hk[hole + 1] = hk[child + 1];
    hidx[hole + 1] = hidx[child + 1];
    hole = child;
  }
  if (child == half) {
    child = 2 * (child + 1);
    hk[hole + 1] = hk[child];
    hidx[hole + 1] = hidx[child];
    hole = child - 1;
  }
  int parent = (hole - 1) / 2;
  while (hole > top && hk[parent + 1] > vk) {
    hk[hole + 1] = hk[parent + 1];
    hidx[hole + 1] = hidx[parent + 1];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  hk[hole + 1] = vk;
  hidx[hole + 1] = vi;
}

// __pop_heap's replacement of the top by (vk, vi), one thread.  libstdc++
// moves the hole from the top to a leaf along the preferred children (the
// left one only when its key is strictly smaller) and then sifts vk up; along
// that path keys never decrease, so the net effect is: every path node whose
// key is <= vk moves up one level and vk takes the place of the last one
// moved.  The walk therefore stops at the first preferred child above vk.
// Two levels per step: the children and the four grandchildren of the hole
// are read together (the key array is padded to 2 * len + 8 entries so the
// look-ahead reads stay inside it).  Returns the new top key.
__device__ __forceinline__ unsigned long long rp_insert(unsigned long long* hk, unsigned* hidx, int lim, int half,
                                                        unsigned long long vk, unsigned vi) {
  int hole = 0;
  unsigned long long top = vk;
  bool stop = false;
  while (hole < lim) {
    const ulonglong2 c2 = *reinterpret_cast<const ulonglong2*>(hk + 2 * hole + 2);
    const ulonglong2 gl = *reinterpret_cast<const ulonglong2*>(hk + 4 * hole + 4);
    const ulonglong2 gr = *reinterpret_cast<const ulonglong2*>(hk + 4 * hole + 6);
    const bool left = c2.y > c2.x;
    const unsigned long long ck = left ? c2.x : c2.y;
    const int c = 2 * hole + 2 - (left ? 1 : 0);
    if (ck > vk) {
      stop = true;
      break;
    }
    if (hole == 0) top = ck;
    hk[hole + 1] = ck;
    hidx[hole + 1] = hidx[c + 1];
    hole = c;
    if (c >= lim) break;
    const bool l2 = left ? (gl.y > gl.x) : (gr.y > gr.x);
    const unsigned long long gk = left ? (l2 ? gl.x : gl.y) : (l2 ? gr.x : gr.y);
    const int gc = 2 * c + 2 - (l2 ? 1 : 0);
    if (gk > vk) {
      stop = true;
      break;
    }
    hk[c + 1] = gk;
    hidx[c + 1] = hidx[gc + 1];
    hole = gc;
  }
  if (!stop && hole == half) {
    const unsigned long long ck = hk[2 * hole + 2];
    if (!(ck > vk)) {
      if (hole == 0) top = ck;
      hk[hole + 1] = ck;
      hidx[hole + 1] = hidx[2 * hole + 2];
      hole = 2 * hole + 1;
    }
  }
  hk[hole + 1] = vk;
  hidx[hole + 1] = vi;
  return top;
}

// Replays the candidates buf[0..cnt) against the heap with one warp, several
// replacements in flight.  A replacement (rp_insert's walk, one level per
// step) reads the children of its hole and writes the hole; if every
// replacement in flight is at least two levels below the next one, the
// levels they touch never overlap, so each step advances all of them at once
// (lane = one replacement).  A candidate is taken only once the previous one
// has passed level 1, when the top it is compared with is final; the result
// is the sequential replay's.  On return nothing is in flight and top is the
// heap's top key.
__device__ __forceinline__ void rp_pipeline(const HNode* buf, int cnt, unsigned long long* hk, unsigned* hidx,
                                            int lim, int half, unsigned long long& top) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  bool act = false;
  int hole = 0;
  unsigned long long vk = 0;
  unsigned vi = 0;
  // replacements start on even steps only (the previous one is then two
  // levels down) and take lanes round robin: a replacement lasts at most one
  // step per heap level (< 32 for k < 2^31), so a lane is free again after
  // 32 starts
  int next_lane = 0;
  int drain = 0;  // steps left once the candidates are used up
  // a window of 32 candidates in registers, one per lane; wmask = not yet passed
  int q0 = 0;
  unsigned long long wk = lane < cnt ? buf[lane].key : 0ULL;
  unsigned wi = lane < cnt ? (unsigned)buf[lane].idx : 0u;
  unsigned wmask = __ballot_sync(FULL, lane < cnt);
  for (int step = 0;; ++step) {
    if ((step & 1) == 0 && drain == 0) {
      unsigned m = wmask & __ballot_sync(FULL, wk > top);
      while (!m) {
        q0 += 32;
        if (q0 >= cnt) break;
        const int i = q0 + lane;
        wk = i < cnt ? buf[i].key : 0ULL;
        wi = i < cnt ? (unsigned)buf[i].idx : 0u;
        wmask = __ballot_sync(FULL, i < cnt);
        m = wmask & __ballot_sync(FULL, wk > top);
      }
      if (m) {
        const int src = __ffs(m) - 1;
        wmask &= ~((2u << src) - 1u);
        const unsigned long long nk = __shfl_sync(FULL, wk, src);
        const unsigned ni = __shfl_sync(FULL, wi, src);
        if (lane == next_lane) {
          act = true;
          hole = 0;
          vk = nk;
          vi = ni;
        }
        next_lane = (next_lane + 1) & 31;
      } else {
        wmask = 0;
        drain = 33;
      }
    }
    if (drain && --drain == 0) break;
    // one level for every replacement in flight, without branches: the
    // children of any node below k lie inside the padded arrays
    {
      const int h = act ? hole : 0;
      const ulonglong2 c2 = *reinterpret_cast<const ulonglong2*>(hk + 2 * h + 2);
      const uint2 i2 = *reinterpret_cast<const uint2*>(hidx + 2 * h + 2);
      const bool two = h < lim, one = h == half;
      const bool left = one || (two && c2.y > c2.x);
      const unsigned long long ck = left ? c2.x : c2.y;
      const unsigned cidx = left ? i2.x : i2.y;
      const bool move = (two || one) && !(ck > vk);
      const int c = 2 * h + 2 - (left ? 1 : 0);
      const bool leaf = c >= lim && c != half;
      if (act) {
        hk[h + 1] = move ? ck : vk;
        hidx[h + 1] = move ? cidx : vi;
      }
      if (act && move && leaf) {
        hk[c + 1] = vk;
        hidx[c + 1] = vi;
      }
      act = act && move && !leaf;
      hole = c;
    }
    __syncwarp();
    top = hk[1];
  }
}

// HEAP_SMEM: the heap is in shared memory after the staging buffers (the
// compiler then addresses it as shared memory); else in gk / gi.  Positions
// are 32-bit (the host takes this path only for fewer than 2^32 entries).
template <typename T, bool HEAP_SMEM>
__global__ void __launch_bounds__(PX_THREADS)
    k_rp_replay(const T* __restrict__ M, long N, int pos, long k, long wmax, int nwin, TopkState* st,
                unsigned char* __restrict__ flags, const HNode* __restrict__ cand, const int* __restrict__ wcnt,
                unsigned long long* gk, unsigned* gi) {
  if (st->sel_case != 2) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ long s_off[RP_MAXWIN + 1];
  __shared__ long s_lo[RP_MAXWIN];
  HNode* stage = reinterpret_cast<HNode*>(smem_raw);  // 2 x RP_STAGE
  unsigned long long* hk;
  unsigned* hidx;
  if (HEAP_SMEM) {
    hk = reinterpret_cast<unsigned long long*>(smem_raw + 2 * RP_STAGE * sizeof(HNode));
    hidx = reinterpret_cast<unsigned*>(smem_raw + 2 * RP_STAGE * sizeof(HNode) +
                                       sizeof(unsigned long long) * rp_key_len(k));
  } else {
    hk = gk;
    hidx = gi;
  }
  const int t = threadIdx.x, warp = t >> 5;
  const int lim = (int)((k - 1) / 2);
  const int half = (k & 1) == 0 ? (int)((k - 2) / 2) : -1;
  for (int i = t; i < (int)k; i += blockDim.x) {
    hk[i + 1] = sel_key(M[i], pos);
    hidx[i + 1] = (unsigned)i;
  }
  if (t == 0) {
    long acc = 0;
    for (int w = 0; w < nwin; ++w) {
      long lo, hi;
      rp_window(w, N, k, wmax, &lo, &hi);
      s_off[w] = acc;
      s_lo[w] = lo;
      acc += wcnt[w];
    }
    s_off[nwin] = acc;
  }
  __syncthreads();
  // make_heap, deepest parents first, one level at a time
  if (k >= 2) {
    const int lastp = (int)((k - 2) / 2);
    for (int L = 31 - __clz(lastp + 1); L >= 0; --L) {
      const int a = (1 << L) - 1, b = min((2 << L) - 2, lastp);
      for (int n = a + t; n <= b; n += blockDim.x) rp_adjust(hk, hidx, n, lim, half);
      __syncthreads();
    }
  }
  const long total = s_off[nwin];
  const long nsteps = (total + RP_STAGE - 1) / RP_STAGE;
  auto stage_chunk = [&](long c, HNode* dst, int t0, int nthr) {
    const long q0 = c * RP_STAGE;
    const int cnt = (int)min((long)RP_STAGE, total - q0);
    for (int j = t0; j < cnt; j += nthr) {
      const long q = q0 + j;
      int a = 0, b = nwin - 1;
      while (a < b) {
        const int mid = (a + b + 1) >> 1;
        if (s_off[mid] <= q) a = mid;
        else b = mid - 1;
      }
      dst[j] = cand[s_lo[a] + (q - s_off[a])];
    }
  };
  if (nsteps > 0) stage_chunk(0, stage, t, blockDim.x);
  __syncthreads();
  unsigned long long top = hk[1];
  for (long c = 0; c < nsteps; ++c) {
    if (warp != 0) {
      if (c + 1 < nsteps) stage_chunk(c + 1, stage + ((c + 1) & 1) * RP_STAGE, t - 32, blockDim.x - 32);
    } else {
      rp_pipeline(stage + (c & 1) * RP_STAGE, (int)min((long)RP_STAGE, total - c * RP_STAGE), hk, hidx, lim, half,
                  top);
    }
    __syncthreads();
  }
  const unsigned long long tt = st->t;
  for (int i = t; i < (int)k; i += blockDim.x)
    if (hk[i + 1] == tt) flags[hidx[i + 1]] = 1;
}

// ------------------------------------------------------------------ sp apply
template <typename T>
__global__ void k_sp_apply(T* __restrict__ M, long N, int pos, const TopkState* st, unsigned char* __restrict__ flags,
                           int* d_status) {
  // the selection is complete: its status goes to the caller's word
  if (d_status && blockIdx.x == 0 && threadIdx.x == 0 && st->status) atomicCAS(d_status, 0, st->status);
  const unsigned long long t = st->t;
  const int cs = st->sel_case;
  const long long tau = st->tau;
  // four entries per thread in flight; pos_adj(m, pos) is m unless pos
  // turned it into +0 (a zero key on a non-zero magnitude); entries that
  // keep their bits are not rewritten
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i0 = blockIdx.x * (long)blockDim.x + threadIdx.x; i0 < N; i0 += 4 * stride) {
    T m[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) m[u] = i0 + u * stride < N ? M[i0 + u * stride] : T(0);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const long i = i0 + u * stride;
      if (i >= N) break;
      const unsigned long long key = sel_key(m[u], pos);
      bool keep = key > t;
      if (!keep && key == t) {
        if (cs == 0) keep = true;
        else if (cs == 1) keep = i <= tau;
        else if (cs == 2) keep = flags[i] != 0;
      }
      if (cs == 2) flags[i] = 0;
      const bool adjusted = key == 0 && mag_key(m[u]) != 0;
      const T out = keep && !adjusted ? m[u] : T(0);
      if (raw_bits(out) != raw_bits(m[u])) M[i] = out;
    }
  }
}

// The second half, run by the last of chunk c's SQ_SEG segment blocks to
// finish (all of them have written their partials and marks): every lane
// continues its chain from its first marked segment over the later marked
// ones, in order, then the lanes are added by the tree.  The other blocks'
// writes are read from L2.  Every thread of the block calls it.
template <typename T>
__device__ void sq_chunk_lanes(const T* __restrict__ M, long N, int c, const double* __restrict__ seg,
                               unsigned* __restrict__ mask, double* partials, T* lane) {
  const int t = threadIdx.x;
  unsigned m = __ldcg(&mask[c * CR_LANES + t]);
  T acc = T(0);
  if (m) {
    acc = __ldcg(reinterpret_cast<const T*>(seg) + ((long)c * SQ_SEG + (__ffs(m) - 1)) * CR_LANES + t);
    m &= m - 1;
    while (m) {
      const int s = __ffs(m) - 1;
      m &= m - 1;
      const long base = (long)c * CR_CHUNK + t + (long)s * SQ_PER * CR_LANES;
      for (int u = 0; u < SQ_PER; ++u) {
        const long i = base + (long)u * CR_LANES;
        if (i < N) {
          const T x = __ldcg(M + i);
          if (mag_key(x) != 0) acc = fmad(x, x, acc);
        }
      }
    }
    mask[c * CR_LANES + t] = 0;  // zero again for the next use
  }
  lane[t] = acc;
  const T part = lane_tree_256(lane);
  if (t == 0) reinterpret_cast<T*>(partials)[c] = part;
}

// After a segment block's partials and marks: the last block of the chunk
// finishes it (per-chunk arrival counter, reset by that block).
template <typename T>
__device__ __forceinline__ void sq_segment_done(const T* __restrict__ M, long N, int c, const double* seg,
                                                unsigned* mask, unsigned* done, double* partials) {
  __shared__ T lane[CR_LANES];
  __shared__ int last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    last = atomicAdd(&done[c], 1u) == (unsigned)(SQ_SEG - 1);
    if (last) done[c] = 0;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  sq_chunk_lanes<T>(M, N, c, seg, mask, partials, lane);
}

// k_sp_apply with the first half of the normalisation's sum of squares
// (k_sumsq_seg) on the entries it leaves: block (c, s) of SQ_SEG blocks per
// chunk, lane t owns the entries t + CR_LANES * (SQ_PER * s + u) of chunk c,
// decides and writes them as k_sp_apply does and chains the squares of the
// kept ones in order.
template <typename T>
__global__ void __launch_bounds__(CR_LANES)
    k_sp_apply_sq(T* __restrict__ M, long N, int pos, const TopkState* st, unsigned char* __restrict__ flags,
                  int* d_status, double* __restrict__ seg, unsigned* __restrict__ mask,
                  unsigned* __restrict__ done, double* partials) {
  if (d_status && blockIdx.x == 0 && threadIdx.x == 0 && st->status) atomicCAS(d_status, 0, st->status);
  const unsigned long long t = st->t;
  const int cs = st->sel_case;
  const long long tau = st->tau;
  const int c = blockIdx.x / SQ_SEG, s = blockIdx.x % SQ_SEG, ln = threadIdx.x;
  const long base = (long)c * CR_CHUNK + ln + (long)s * SQ_PER * CR_LANES;
  T m[SQ_PER];
#pragma unroll
  for (int u = 0; u < SQ_PER; ++u) {
    const long i = base + (long)u * CR_LANES;
    m[u] = i < N ? M[i] : T(0);
  }
  T acc = T(0);
  bool nz = false;
#pragma unroll
  for (int u = 0; u < SQ_PER; ++u) {
    const long i = base + (long)u * CR_LANES;
    if (i >= N) break;
    const unsigned long long key = sel_key(m[u], pos);
    bool keep = key > t;
    if (!keep && key == t) {
      if (cs == 0) keep = true;
      else if (cs == 1) keep = i <= tau;
      else if (cs == 2) keep = flags[i] != 0;
    }
    if (cs == 2) flags[i] = 0;
    const bool adjusted = key == 0 && mag_key(m[u]) != 0;
    const T out = keep && !adjusted ? m[u] : T(0);
    if (raw_bits(out) != raw_bits(m[u])) M[i] = out;
    if (mag_key(out) != 0) {
      acc = fmad(out, out, acc);
      nz = true;
    }
  }
  if (nz) {
    reinterpret_cast<T*>(seg)[((long)c * SQ_SEG + s) * CR_LANES + ln] = acc;
    atomicOr(&mask[c * CR_LANES + ln], 1u << s);
  }
  sq_segment_done<T>(M, N, c, seg, mask, done, partials);
}

template <typename T>
__global__ void k_pos_only(T* __restrict__ M, long N) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x)
    if (M[i] < T(0)) M[i] = T(0);
}

template <typename T>
__global__ void k_zero(T* __restrict__ M, long N) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) M[i] = T(0);
}

// ------------------------------------------------------------------ line top-k
// Heap selection of the k largest |v| of one line (a column or a row),
// marking flags |= bit at the kept positions.  One thread per line.
template <typename T>
__global__ void k_line_topk(const T* __restrict__ M, int rows, int cols, int by_col, int k, int pos,
                            unsigned char* __restrict__ flags, unsigned char bit) {
  const int nlines = by_col ? cols : rows;
  const int len = by_col ? rows : cols;
  const int line = blockIdx.x * blockDim.x + threadIdx.x;
  if (line >= nlines) return;
  auto at = [&](int e) -> long { return by_col ? (long)line * rows + e : (long)e * rows + line; };
  if (k >= len) {
    for (int e = 0; e < len; ++e) flags[at(e)] |= bit;
    return;
  }
  HNode hn[LINE_KMAX];
  HeapView h{hn};
  for (int e = 0; e < k; ++e) hn[e] = HNode{mag_key(pos_adj(M[at(e)], pos)), e};
  if (k >= 2) {
    int parent = (k - 2) / 2;
    while (true) {
      heap_adjust(h, parent, k, hn[parent]);
      if (parent == 0) break;
      parent--;
    }
  }
  for (int e = k; e < len; ++e) {
    const unsigned long long key = mag_key(pos_adj(M[at(e)], pos));
    if (key > hn[0].key) heap_adjust(h, 0, k, HNode{key, e});
  }
  for (int e = 0; e < k; ++e) flags[at((int)hn[e].idx)] |= bit;
}

template <typename T>
__global__ void k_flag_apply(T* __restrict__ M, long N, int pos, unsigned char* __restrict__ flags) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    const T v = pos_adj(M[i], pos);
    M[i] = flags[i] ? v : T(0);
    flags[i] = 0;
  }
}

// ------------------------------------------------------------------ norms
// normcol: one block per column; canonical norm of the column, scale by
// s / norm (a zero column stays zero).  normlin: the same per row.
template <typename T>
__global__ void __launch_bounds__(PX_THREADS)
    k_normline(T* __restrict__ M, int rows, int cols, int by_col, double s, int pos) {
  __shared__ T lane[PX_THREADS];
  const int line = blockIdx.x;
  const int len = by_col ? rows : cols;
  auto at = [&](long e) -> long { return by_col ? (long)line * rows + e : e * rows + line; };
  T total = T(0);
  for (long c0 = 0; c0 < len; c0 += CR_CHUNK) {
    const long c1 = min((long)len, c0 + CR_CHUNK);
    T acc = T(0);
    for (long e = c0 + threadIdx.x; e < c1; e += CR_LANES) {
      const T v = pos_adj(M[at(e)], pos);
      acc = fmad(v, v, acc);
    }
    lane[threadIdx.x] = acc;
    total = addr(total, lane_tree_256(lane));
  }
  __shared__ T s_scal;
  if (threadIdx.x == 0) {
    T scal = sqrtr(total);
    if (scal != T(0)) scal = divr((T)s, scal);
    s_scal = scal;
  }
  __syncthreads();
  const T scal = s_scal;
  for (long e = threadIdx.x; e < len; e += blockDim.x) M[at(e)] = mulr(pos_adj(M[at(e)], pos), scal);
}

template <typename T>
__global__ void k_supp(T* __restrict__ M, long N, const T* __restrict__ S, int pos) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x)
    M[i] = mulr(pos_adj(M[i], pos), S[i]);
}

// Canonical sum of squares: one block per chunk of 65536 entries.
template <typename T>
__global__ void __launch_bounds__(PX_THREADS) k_chunk_sumsq(const T* __restrict__ M, long N, double* partials) {
  __shared__ T lane[PX_THREADS];
  const long c0 = blockIdx.x * CR_CHUNK, c1 = min(N, c0 + CR_CHUNK);
  // A zero entry adds +0 to a non-negative partial, so a warp issues the
  // FMA of a batch position only when one of its lanes holds a non-zero
  // there (the sparse projections leave few non-zeros; an FP64 FMA issues at
  // the same cost for 1 or 32 lanes).  The positions to do come from ballots
  // and are walked by a loop, in order.
  // Thirty-two loads per thread are issued before any is used (the loop is
  // otherwise one memory round trip per batch).
  T acc = T(0);
  long i = c0 + threadIdx.x;
  for (; i + 31 * CR_LANES < c1; i += 32 * CR_LANES) {
    T v[32];
#pragma unroll
    for (int u = 0; u < 32; ++u) v[u] = M[i + u * CR_LANES];
    const unsigned am = __activemask();
    unsigned todo = 0;
#pragma unroll
    for (int u = 0; u < 32; ++u) todo |= (__ballot_sync(am, mag_key(v[u]) != 0) ? 1u : 0u) << u;
    while (todo) {
      const int u = __ffs(todo) - 1;
      todo &= todo - 1;
      T x = v[0];
#pragma unroll
      for (int q = 1; q < 32; ++q) x = u == q ? v[q] : x;
      acc = fmad(x, x, acc);
    }
  }
  for (; i < c1; i += CR_LANES) {
    const T v = M[i];
    if (mag_key(v) != 0) acc = fmad(v, v, acc);
  }
  lane[threadIdx.x] = acc;
  const T part = lane_tree_256(lane);
  if (threadIdx.x == 0) reinterpret_cast<T*>(partials)[blockIdx.x] = part;
}

// The same canonical sum of squares split over SQ_SEG blocks per chunk, for
// the sparse results of the projections: block (c, s) computes, for every
// lane t of chunk c, the sequential fma over the lane's values SQ_PER * s ..
// SQ_PER * s + SQ_PER - 1 from +0 (zeros add +0 to a non-negative partial
// and are skipped) and marks the segments that held a non-zero; the last
// block of the chunk to finish continues each lane's chain from its first
// marked segment over the later marked ones, in order, then adds the lanes by
// the tree (sq_segment_done).  Most lanes of a sparse block have no or one
// marked segment, so the chain rarely reloads anything; a dense block costs
// what k_chunk_sumsq costs.
template <typename T>
__global__ void __launch_bounds__(CR_LANES) k_sumsq_seg(const T* __restrict__ M, long N, double* __restrict__ seg,
                                                         unsigned* __restrict__ mask, unsigned* __restrict__ done,
                                                         double* partials) {
  const int c = blockIdx.x / SQ_SEG, s = blockIdx.x % SQ_SEG, t = threadIdx.x;
  const long base = (long)c * CR_CHUNK + t + (long)s * SQ_PER * CR_LANES;
  T v[SQ_PER];
#pragma unroll
  for (int u = 0; u < SQ_PER; ++u) {
    const long i = base + (long)u * CR_LANES;
    v[u] = i < N ? M[i] : T(0);
  }
  T acc = T(0);
  bool nz = false;
#pragma unroll
  for (int u = 0; u < SQ_PER; ++u)
    if (mag_key(v[u]) != 0) {
      acc = fmad(v[u], v[u], acc);
      nz = true;
    }
  if (nz) {
    reinterpret_cast<T*>(seg)[((long)c * SQ_SEG + s) * CR_LANES + t] = acc;
    atomicOr(&mask[c * CR_LANES + t], 1u << s);
  }
  sq_segment_done<T>(M, N, c, seg, mask, done, partials);
}

// rcnt, ccnt (optional): per-row and per-column counts of the non-zero
// results, added to (column-major M with `rows` rows), for the dense -> CSR
// conversion that follows.
template <typename T>
__device__ __forceinline__ void scale_store(T* M, long i, T x, T s, int rows, int* rcnt, int* ccnt) {
  const T y = mulr(x, s);
  M[i] = y;
  if (rcnt && mag_key(y) != 0) {
    atomicAdd(&rcnt[i % rows], 1);
    atomicAdd(&ccnt[i / rows], 1);
  }
}

// MatDense::normalize (faust_MatDense.hpp:1225-1250): scale = FPP(1.0/norm),
// domain_error (here FGB_ERR_ZERO_NORM) on a zero norm.  Every block of the
// scaling kernel adds the chunk partials in order itself (one thread: the
// FP64 square root and division are a few hundred cycles), which saves the
// launch of a one-thread kernel.
template <typename T>
__global__ void k_scale(T* __restrict__ M, long N, const double* __restrict__ partials, int nchunks, int* status,
                        int rows, int* __restrict__ rcnt, int* __restrict__ ccnt) {
  __shared__ T s_inv;
  if (threadIdx.x == 0) {
    T total = T(0);
    for (int c = 0; c < nchunks; ++c) total = addr(total, reinterpret_cast<const T*>(partials)[c]);
    const T n = sqrtr(total);
    T inv = T(0);
    if (n == T(0)) {
      if (status && blockIdx.x == 0) atomicCAS(status, 0, (int)FGB_ERR_ZERO_NORM);
    } else {
      inv = (T)__ddiv_rn(1.0, (double)n);
    }
    s_inv = inv;
  }
  __syncthreads();
  const T s = s_inv;
  // a zero times a finite non-negative scale keeps its bits: not rewritten,
  // and a warp of zeros issues no multiply
  const bool skip_zeros = raw_bits(s) < raw_bits(T(INFINITY));
  const long stride = (long)gridDim.x * blockDim.x;
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  for (; i + 3 * stride < N; i += 4 * stride) {
    T v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) v[u] = M[i + u * stride];
    const unsigned am = __activemask();
    unsigned todo = 0;
#pragma unroll
    for (int u = 0; u < 4; ++u) todo |= (__ballot_sync(am, !skip_zeros || mag_key(v[u]) != 0) ? 1u : 0u) << u;
    while (todo) {
      const int u = __ffs(todo) - 1;
      todo &= todo - 1;
      T x = v[0];
#pragma unroll
      for (int q = 1; q < 4; ++q) x = u == q ? v[q] : x;
      if (!skip_zeros || mag_key(x) != 0) scale_store(M, i + u * stride, x, s, rows, rcnt, ccnt);
    }
  }
  for (; i < N; i += stride) {
    const T v = M[i];
    if (!skip_zeros || mag_key(v) != 0) scale_store(M, i, v, s, rows, rcnt, ccnt);
  }
}


__global__ void k_topk_init(TopkState* st, long long k) {
  TopkState z;
  memset(&z, 0, sizeof(z));
  z.k_rem = k;
  *st = z;
}

// ------------------------------------------------------------------ host side
static int grid_for(fgb_ctx* ctx, long n) {
  long g = (n + PX_THREADS - 1) / PX_THREADS;
  return (int)std::max(1L, std::min(g, 4L * ctx->sm_count));
}

template <typename T>
static fgb_status queue_normalize(fgb_ctx* ctx, ProxWork& w, T* M, long N, int* d_status, bool seg_done = false,
                                  int rows = 0, int cols = 0) {
  const int nchunks = (int)((N + CR_CHUNK - 1) / CR_CHUNK);
  if (w.sq_seg && w.sq_mask && w.sq_done && nchunks <= w.sq_chunks) {
    if (!seg_done) {
      k_sumsq_seg<T><<<nchunks * SQ_SEG, CR_LANES, 0, ctx->stream>>>(M, N, w.sq_seg, w.sq_mask, w.sq_done,
                                                                     w.partials);
      FGB_LAUNCHED(ctx);
    }
  } else {
    k_chunk_sumsq<T><<<nchunks, PX_THREADS, 0, ctx->stream>>>(M, N, w.partials);
    FGB_LAUNCHED(ctx);
  }
  // the non-zeros per row and column for a dense -> CSR conversion of M that
  // may follow (when the workspace holds both count arrays)
  int *rcnt = nullptr, *ccnt = nullptr;
  if (rows > 0 && cols > 0 && (long)rows * cols == N && w.growable && w.cap_rows >= rows + cols + 2) {
    if (w.counted)  // counts of an earlier matrix no conversion consumed
      FGB_CUDA(ctx, cudaMemsetAsync(w.row_cnt, 0, sizeof(int) * (w.cap_rows + 2), ctx->stream));
    rcnt = w.row_cnt;
    ccnt = w.row_cnt + rows;
    w.counted = M;
  }
  k_scale<T><<<grid_for(ctx, N), PX_THREADS, 0, ctx->stream>>>(M, N, w.partials, nchunks, d_status, rows, rcnt, ccnt);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

// Largest dynamic shared memory the tie-replay kernels are launched with on a
// device of `optin` bytes per block (the on-chip heap variants are taken only
// when the heap fits under these caps).
static size_t rp_replay_cap(size_t optin) { return std::min<size_t>(optin > 24 * 1024 ? optin - 24 * 1024 : 0, 200 * 1024); }
static size_t heap_replay_cap(size_t optin) { return std::min<size_t>(optin > 8192 ? optin - 8192 : 0, 200 * 1024); }

// Opts the tie-replay kernels into their largest dynamic shared memory, once
// per device for the whole process.  The attribute belongs to the kernel on
// the device, not to a context: setting it per launch size from several
// contexts could lower it under a launch another context has already sized,
// so it is set once to the cap every launch stays under.
static fgb_status replay_opt_in(fgb_ctx* ctx) {
  static std::atomic<int> done[64];
  const int dev = ctx->device;
  if (dev >= 0 && dev < 64 && done[dev].load(std::memory_order_acquire)) return FGB_OK;
  const int rp = (int)rp_replay_cap(ctx->smem_optin), hr = (int)heap_replay_cap(ctx->smem_optin);
  const int stage = (int)(2 * (size_t)RP_STAGE * sizeof(HNode));
  FGB_CUDA(ctx, cudaFuncSetAttribute(k_rp_replay<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, rp));
  FGB_CUDA(ctx, cudaFuncSetAttribute(k_rp_replay<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, rp));
  FGB_CUDA(ctx, cudaFuncSetAttribute(k_rp_replay<float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, stage));
  FGB_CUDA(ctx, cudaFuncSetAttribute(k_rp_replay<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, stage));
  FGB_CUDA(ctx, cudaFuncSetAttribute(k_heap_replay<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, hr));
  FGB_CUDA(ctx, cudaFuncSetAttribute(k_heap_replay<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, hr));
  if (dev >= 0 && dev < 64) done[dev].store(1, std::memory_order_release);
  return FGB_OK;
}

// Pre-filtered tie replay (k_rp_bounds, k_rp_filter, k_rp_replay); every
// kernel returns at once unless the selection needs the heap order.
template <typename T>
static fgb_status queue_tie_replay(fgb_ctx* ctx, ProxWork& w, const T* M, long N, long k, int pos) {
  const long wmax = rp_wmax(N, k);
  const int nwin = rp_window_count(N, k, wmax);
  if (nwin > RP_MAXWIN) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "tie replay: %d windows", nwin);
  if (w.cand_cap < N) {
    dfree(w.cand);
    dfree(w.wbound);
    dfree(w.wcount);
    w.cand = nullptr;
    w.wbound = nullptr;
    w.wcount = nullptr;
    w.cand_cap = 0;
    FGB_TRY(dmalloc(ctx, &w.cand, sizeof(HNode) * (size_t)N));
    FGB_TRY(dmalloc(ctx, (void**)&w.wbound, sizeof(unsigned long long) * RP_MAXWIN));
    FGB_TRY(dmalloc(ctx, (void**)&w.wcount, sizeof(int) * RP_MAXWIN));
    w.cand_cap = N;
  }
  const long hkn = rp_key_len(k);  // key array (padded), then k + 2 positions
  const size_t stage_bytes = 2 * (size_t)RP_STAGE * sizeof(HNode);
  const size_t heap_bytes = (sizeof(unsigned long long) + sizeof(unsigned)) * (size_t)hkn;
  const size_t cap = rp_replay_cap(ctx->smem_optin);
  const bool in_smem = stage_bytes + heap_bytes <= cap;
  const size_t smem = stage_bytes + (in_smem ? heap_bytes : 0);
  unsigned long long* gk = nullptr;
  unsigned* gi = nullptr;
  if (!in_smem) {
    if (w.heap2_cap < k) {
      dfree(w.heap2);
      w.heap2 = nullptr;
      w.heap2_cap = 0;
      FGB_TRY(dmalloc(ctx, &w.heap2, heap_bytes));
      w.heap2_cap = k;
    }
    gk = reinterpret_cast<unsigned long long*>(w.heap2);
    gi = reinterpret_cast<unsigned*>(gk + hkn);
  }
  k_rp_bounds<T><<<nwin, RP_BLOCK, 0, ctx->stream>>>(M, N, pos, k, wmax, w.state, w.wbound);
  FGB_LAUNCHED(ctx);
  k_rp_filter<T><<<nwin, RP_BLOCK, 0, ctx->stream>>>(M, N, pos, k, wmax, w.state, w.wbound,
                                                     reinterpret_cast<HNode*>(w.cand), w.wcount);
  FGB_LAUNCHED(ctx);
  auto kern = in_smem ? k_rp_replay<T, true> : k_rp_replay<T, false>;
  FGB_TRY(replay_opt_in(ctx));
  {
    const cudaError_t pre = cudaGetLastError();
    if (pre != cudaSuccess) return cuda_check(ctx, pre, "error pending before the tie replay launch");
  }
  kern<<<1, PX_THREADS, smem, ctx->stream>>>(M, N, pos, k, wmax, nwin, w.state, w.flags,
                                             reinterpret_cast<const HNode*>(w.cand), w.wcount, gk, gi);
  {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
      return fail(ctx, FGB_ERR_CUDA, "k_rp_replay launch (FP%d, %s heap, %zu B dynamic shared memory): %s",
                  (int)sizeof(T) * 8, in_smem ? "on-chip" : "global", smem, cudaGetErrorString(e));
    ctx->launches.fetch_add(1, std::memory_order_relaxed);
  }
  return FGB_OK;
}

template <typename T>
static fgb_status queue_sp(fgb_ctx* ctx, ProxWork& w, T* M, long N, long k, int pos, int* d_status,
                           bool* seg_done = nullptr) {
  const int g = grid_for(ctx, N);
  if (!w.hist_passes) {
    k_topk_init<<<1, 1, 0, ctx->stream>>>(w.state, k);
    FGB_LAUNCHED(ctx);
  }
  if (w.hist_passes) {
    // every pass in one cooperative launch (blocks co-resident for the barrier)
    int& nb = ctx->rs_coop_blocks[sizeof(T) == 8];
    if (!nb) {
      int per_sm = 0;
      FGB_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_radix_select<T>, PX_THREADS, 0));
      nb = std::max(1, std::min(per_sm, 2)) * ctx->sm_count;
    }
    const int grid = (int)std::min<long>(nb, std::max(1L, (N + PX_THREADS - 1) / PX_THREADS));
    const int npass = sizeof(T) == 8 ? 6 : 3;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(PX_THREADS);
    cfg.stream = ctx->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const T* Mc = M;
    // keys held in registers when every thread's share fits
    int& nbr = ctx->rs_coop_blocks_reg[sizeof(T) == 8];
    if (!nbr) {
      int per_sm = 0;
      FGB_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_radix_select_reg<T>, PX_THREADS, 0));
      nbr = std::max(1, std::min(per_sm, 1)) * ctx->sm_count;
    }
    if (N <= (long)nbr * PX_THREADS * RS_KREG) {
      cfg.gridDim = dim3((unsigned)std::min<long>(nbr, std::max(1L, (N + PX_THREADS - 1) / PX_THREADS)));
      FGB_CUDA(ctx, cudaLaunchKernelEx(&cfg, k_radix_select_reg<T>, Mc, N, pos, npass, (long long)k, w.state,
                                       w.hist_passes, w.rs_list));
    } else {
      FGB_CUDA(ctx, cudaLaunchKernelEx(&cfg, k_radix_select<T>, Mc, N, pos, npass, (long long)k, w.state,
                                       w.hist_passes, w.rs_list));
    }
    FGB_LAUNCHED(ctx);
  } else if (sizeof(T) == 8) {
    const int shifts[6] = {52, 41, 30, 19, 8, 0};
    const int bits[6] = {11, 11, 11, 11, 11, 8};
    for (int p = 0; p < 6; ++p) {
      k_radix_pass<T><<<g, PX_THREADS, 0, ctx->stream>>>(M, N, pos, shifts[p], bits[p], w.state, w.hist);
      FGB_LAUNCHED(ctx);
    }
  } else {
    const int shifts[3] = {20, 9, 0};
    const int bits[3] = {11, 11, 9};
    for (int p = 0; p < 3; ++p) {
      k_radix_pass<T><<<g, PX_THREADS, 0, ctx->stream>>>(M, N, pos, shifts[p], bits[p], w.state, w.hist);
      FGB_LAUNCHED(ctx);
    }
  }
  const long chunk = std::max(8192L, (N + 2047) / 2048);
  const int nch = (int)((N + chunk - 1) / chunk);
  k_tie_case<T><<<nch, PX_THREADS, 0, ctx->stream>>>(M, N, pos, chunk, w.state, w.chunk_cnt);
  FGB_LAUNCHED(ctx);
  if (w.growable && N < (1L << 32) - 1) {
    FGB_TRY(queue_tie_replay<T>(ctx, w, M, N, k, pos));
  } else {
    // candidates of one chunk, then the heap itself when it fits on chip;
    // larger heaps live in the workspace
    const size_t cand_bytes = (size_t)HR_CHUNK * sizeof(HNode);
    const size_t heap_bytes = (size_t)k * sizeof(HNode);
    const size_t cap = heap_replay_cap(ctx->smem_optin);
    const bool use_smem = cand_bytes + heap_bytes <= cap;
    size_t smem = use_smem ? cand_bytes + heap_bytes : cand_bytes;
    HNode* gheap = nullptr;
    if (!use_smem) {
      if (w.heap_cap < k) {
        dfree(w.heap);
        w.heap = nullptr;
        w.heap_cap = 0;
        FGB_TRY(dmalloc(ctx, &w.heap, heap_bytes));
        w.heap_cap = k;
      }
      gheap = reinterpret_cast<HNode*>(w.heap);
    }
    auto kern = k_heap_replay<T>;
    FGB_TRY(replay_opt_in(ctx));
    kern<<<1, PX_THREADS, smem, ctx->stream>>>(M, N, pos, (int)k, w.state, w.flags, gheap, use_smem ? 1 : 0);
    FGB_LAUNCHED(ctx);
  }
  const int nchunks = (int)((N + CR_CHUNK - 1) / CR_CHUNK);
  if (seg_done && w.sq_seg && w.sq_mask && w.sq_done && nchunks <= w.sq_chunks) {
    // the normalisation follows: its segment sums come with the apply
    k_sp_apply_sq<T><<<nchunks * SQ_SEG, CR_LANES, 0, ctx->stream>>>(M, N, pos, w.state, w.flags, d_status, w.sq_seg,
                                                                   w.sq_mask, w.sq_done, w.partials);
    *seg_done = true;
  } else {
    k_sp_apply<T><<<g, PX_THREADS, 0, ctx->stream>>>(M, N, pos, w.state, w.flags, d_status);
  }
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

template <typename T>
fgb_status launch_prox(fgb_ctx* ctx, ProxWork& w, const fgb_constraint& c, T* M, int rows, int cols,
                       const T* supp_dev, int* d_status) {
  const long N = (long)rows * cols;
  FGB_TRY(prox_work_reserve(ctx, w, N, std::max(rows, cols)));
  const int g = grid_for(ctx, N);
  int pos = c.pos != 0;
  bool seg_done = false;  // the sum of squares' segment pass already ran
  switch (c.kind) {
    case FGB_SP_POS:
      pos = 1;
      /* fall through */
    case FGB_SP: {
      // prox_sp (faust_prox.hpp:71-96)
      if (c.k <= 0) {
        k_zero<T><<<g, PX_THREADS, 0, ctx->stream>>>(M, N);
        FGB_LAUNCHED(ctx);
      } else if (c.k < N) {
        FGB_TRY(queue_sp<T>(ctx, w, M, N, (long)c.k, pos, d_status, c.normalized ? &seg_done : nullptr));
      } else if (pos) {
        k_pos_only<T><<<g, PX_THREADS, 0, ctx->stream>>>(M, N);
        FGB_LAUNCHED(ctx);
      }
      break;
    }
    case FGB_SPCOL:
    case FGB_SPLIN:
    case FGB_SPLINCOL: {
      // prox_spcol / prox_splin / prox_splincol (faust_prox.hpp:112-202);
      // splincol ignores pos, as the reference applies it after copying.
      if (c.kind == FGB_SPLINCOL) pos = 0;
      if (c.k <= 0) {
        k_zero<T><<<g, PX_THREADS, 0, ctx->stream>>>(M, N);
        FGB_LAUNCHED(ctx);
        break;
      }
      if (c.k > LINE_KMAX && !((c.kind == FGB_SPCOL && c.k >= rows) || (c.kind == FGB_SPLIN && c.k >= cols) ||
                               (c.kind == FGB_SPLINCOL && c.k >= rows && c.k >= cols)))
        return fail(ctx, FGB_ERR_NOT_SUPPORTED, "per-line top-k supports k <= %d", LINE_KMAX);
      const int k = (int)std::min<long long>(c.k, LINE_KMAX + (long long)std::max(rows, cols));
      if (c.kind != FGB_SPLIN) {
        k_line_topk<T><<<(cols + 127) / 128, 128, 0, ctx->stream>>>(M, rows, cols, 1, std::min(k, rows), pos,
                                                                   w.flags, 1);
        FGB_LAUNCHED(ctx);
      }
      if (c.kind != FGB_SPCOL) {
        k_line_topk<T><<<(rows + 127) / 128, 128, 0, ctx->stream>>>(M, rows, cols, 0, std::min(k, cols), pos,
                                                                   w.flags, 2);
        FGB_LAUNCHED(ctx);
      }
      k_flag_apply<T><<<g, PX_THREADS, 0, ctx->stream>>>(M, N, pos, w.flags);
      FGB_LAUNCHED(ctx);
      break;
    }
    case FGB_NORMCOL:
    case FGB_NORMLIN: {
      if (c.s < 0) return fail(ctx, FGB_ERR_INVALID_ARG, "Faust::prox_normcol : s < 0 ");
      if (c.s == 0) {
        k_zero<T><<<g, PX_THREADS, 0, ctx->stream>>>(M, N);
        FGB_LAUNCHED(ctx);
      } else {
        const bool by_col = c.kind == FGB_NORMCOL;
        k_normline<T><<<by_col ? cols : rows, PX_THREADS, 0, ctx->stream>>>(M, rows, cols, by_col ? 1 : 0, c.s, pos);
        FGB_LAUNCHED(ctx);
      }
      break;
    }
    case FGB_SUPP: {
      if (!supp_dev) return fail(ctx, FGB_ERR_INVALID_ARG, "prox_supp: missing support");
      k_supp<T><<<g, PX_THREADS, 0, ctx->stream>>>(M, N, supp_dev, pos);
      FGB_LAUNCHED(ctx);
      break;
    }
    default:
      return fail(ctx, FGB_ERR_INVALID_ARG, "project : cannot project with this constraint name");
  }
  if (c.normalized) FGB_TRY(queue_normalize<T>(ctx, w, M, N, d_status, seg_done, rows, cols));
  return FGB_OK;
}

// dense -> CSR and CSR of the transpose.  One warp per row (lanes over
// columns) and one warp per column (lanes over rows) count the non-zero
// entries, a block scans both count arrays, then the same warps write the
// entries by ballot compaction, which keeps rows in column order and
// columns in row order.  Each warp loads eight 32-entry groups before it
// uses them (the loop is otherwise one L2 round trip per group), and the
// zero tests are on the bits.
template <typename T>
__global__ void __launch_bounds__(256)
    k_d2c_count_rc(const T* __restrict__ M, int rows, int cols, int* __restrict__ rcnt, int* __restrict__ ccnt,
                   int with_cols) {
  const long w = (blockIdx.x * (long)blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  const bool is_row = w < rows;
  if (!is_row && !(with_cols && w < (long)rows + cols)) return;
  // entry e of the line: M[base + e * step]
  const long base = is_row ? w : (w - rows) * (long)rows;
  const long step = is_row ? rows : 1;
  const int len = is_row ? cols : rows;
  int c = 0;
  int e = lane;
  for (; e + 7 * 32 < len; e += 8 * 32) {
    T v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = M[base + (long)(e + u * 32) * step];
#pragma unroll
    for (int u = 0; u < 8; ++u) c += mag_key(v[u]) != 0;
  }
  for (; e < len; e += 32) c += mag_key(M[base + (long)e * step]) != 0;
  for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if (lane == 0) (is_row ? rcnt[w] : ccnt[w - rows]) = c;
}

// Exclusive scan of cnt[0..n) into ptr[0..n] by one block (a multiple of 32
// threads, at most 1024): per-thread runs, then a two-level shuffle scan.
// part: at least 32 ints of shared memory.
__device__ void block_excl_scan(const int* __restrict__ cnt, int n, int* __restrict__ ptr, int* part) {
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int r0 = threadIdx.x * per, r1 = min(n, r0 + per);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int s = 0;
  for (int r = r0; r < r1; ++r) s += cnt[r];
  int incl = s;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) part[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int v = lane < nw ? part[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += y;
    }
    if (lane < nw) part[lane] = v;  // inclusive warp totals
  }
  __syncthreads();
  int run = incl - s + (warp ? part[warp - 1] : 0);
  if (threadIdx.x == 0) ptr[n] = part[nw - 1];
  for (int r = r0; r < r1; ++r) {
    ptr[r] = run;
    run += cnt[r];
  }
  __syncthreads();
}

// An entry count above the factor's capacity (which the constraint bounds)
// is reported through *status and the offsets are clamped so that later
// kernels stay inside the arrays.
__global__ void __launch_bounds__(1024) k_d2c_scan_rc(int* rcnt_w, int rows, int* ccnt_w, int cols,
                                                      int* __restrict__ rowptr, int* __restrict__ t_rowptr,
                                                      int with_cols, int cap, int* status, int* maxrc) {
  const int* rcnt = rcnt_w;
  const int* ccnt = ccnt_w;
  __shared__ int part[32];
  __shared__ int mx[2];
  block_excl_scan(rcnt, rows, rowptr, part);
  if (with_cols) block_excl_scan(ccnt, cols, t_rowptr, part);
  if (maxrc) {
    // longest row and column, for the long-row kernels of the products
    if (threadIdx.x < 2) mx[threadIdx.x] = 0;
    __syncthreads();
    int a = 0, b = 0;
    for (int r = threadIdx.x; r < rows; r += blockDim.x) a = max(a, rcnt[r]);
    if (with_cols)
      for (int c = threadIdx.x; c < cols; c += blockDim.x) b = max(b, ccnt[c]);
    for (int s = 16; s >= 1; s >>= 1) {
      a = max(a, __shfl_xor_sync(0xffffffffu, a, s));
      b = max(b, __shfl_xor_sync(0xffffffffu, b, s));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMax(&mx[0], a);
      atomicMax(&mx[1], b);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      maxrc[0] = mx[0];
      maxrc[1] = with_cols ? mx[1] : -1;
    }
  }
  // zero the counts for the next conversion (the normalisation of the
  // projections adds to them)
  __syncthreads();
  for (int r = threadIdx.x; r < rows; r += blockDim.x) rcnt_w[r] = 0;
  for (int c = threadIdx.x; c < cols; c += blockDim.x) ccnt_w[c] = 0;
  if (rowptr[rows] > cap) {
    for (int r = threadIdx.x; r <= rows; r += blockDim.x) rowptr[r] = min(rowptr[r], cap);
    if (with_cols)
      for (int c = threadIdx.x; c <= cols; c += blockDim.x) t_rowptr[c] = min(t_rowptr[c], cap);
    if (threadIdx.x == 0 && status) atomicCAS(status, 0, (int)FGB_ERR_INVALID_ARG);
  }
}

template <typename T>
__global__ void __launch_bounds__(256)
    k_d2c_write_rc(const T* __restrict__ M, int rows, int cols, const int* __restrict__ rowptr,
                   int* __restrict__ colind, T* __restrict__ val, const int* __restrict__ t_rowptr,
                   int* __restrict__ t_colind, T* __restrict__ t_val, int cap, int with_cols) {
  const long w = (blockIdx.x * (long)blockDim.x + threadIdx.x) / 32;
  const unsigned lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const bool is_row = w < rows;
  if (!is_row && !(with_cols && w < (long)rows + cols)) return;
  const long base = is_row ? w : (w - rows) * (long)rows;
  const long step = is_row ? rows : 1;
  const int len = is_row ? cols : rows;
  int* __restrict__ ind = is_row ? colind : t_colind;
  T* __restrict__ out = is_row ? val : t_val;
  int at = is_row ? rowptr[w] : t_rowptr[w - rows];
  for (int e0 = 0; e0 < len; e0 += 8 * 32) {
    T v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = e0 + u * 32 + (int)lane;
      v[u] = e < len ? M[base + (long)e * step] : T(0);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const bool nz = mag_key(v[u]) != 0;
      const unsigned m = __ballot_sync(0xffffffffu, nz);
      if (nz) {
        const int p = at + __popc(m & lt);
        if (p < cap) {
          ind[p] = e0 + u * 32 + (int)lane;
          out[p] = v[u];
        }
      }
      at += __popc(m);
    }
  }
}

template <typename T>
fgb_status launch_dense_to_csr(fgb_ctx* ctx, ProxWork& w, const T* M, DevFactor& f, int* status) {
  FGB_TRY(prox_work_reserve(ctx, w, (long)f.rows * f.cols, f.rows + f.cols + 2));
  const int with_cols = f.t_rowptr ? 1 : 0;
  const long warps = (long)f.rows + (with_cols ? f.cols : 0);
  const int blocks = (int)((warps * 32 + 255) / 256);
  int* rcnt = w.row_cnt;
  int* ccnt = w.row_cnt + f.rows;
  if (w.counted != (const void*)M) {
    k_d2c_count_rc<T><<<blocks, 256, 0, ctx->stream>>>(M, f.rows, f.cols, rcnt, ccnt, with_cols);
    FGB_LAUNCHED(ctx);
  }  // else the normalisation of the projection counted them
  w.counted = nullptr;
  k_d2c_scan_rc<<<1, 1024, 0, ctx->stream>>>(rcnt, f.rows, ccnt, f.cols, f.rowptr, f.t_rowptr, with_cols, f.cap,
                                             status, f.d_maxrc);
  FGB_LAUNCHED(ctx);
  k_d2c_write_rc<T><<<blocks, 256, 0, ctx->stream>>>(M, f.rows, f.cols, f.rowptr, f.colind, (T*)f.val, f.t_rowptr,
                                                     f.t_colind, (T*)f.t_val, f.cap, with_cols);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

template fgb_status launch_prox<float>(fgb_ctx*, ProxWork&, const fgb_constraint&, float*, int, int, const float*,
                                       int*);
template fgb_status launch_prox<double>(fgb_ctx*, ProxWork&, const fgb_constraint&, double*, int, int,
                                        const double*, int*);
template fgb_status launch_dense_to_csr<float>(fgb_ctx*, ProxWork&, const float*, DevFactor&, int*);
template fgb_status launch_dense_to_csr<double>(fgb_ctx*, ProxWork&, const double*, DevFactor&, int*);

}  // namespace fgb
