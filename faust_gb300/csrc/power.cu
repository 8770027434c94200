// power.cu — power iteration for spectral norms of CSR chains, one block per
// chain, vectors in shared memory, the whole loop on the device (no host
// round trip per iteration), with palm4msa2's step-size epilogue.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "rowdot.cuh"
#include "power.cuh"

namespace fgb {

void pi_chain_build(const DevFactor* F, int lo, int hi, PIChain& ch) {
  std::memset(&ch, 0, sizeof(ch));
  if (hi <= lo) {
    ch.empty = 1;
    return;
  }
  for (int i = lo; i < hi; ++i) {
    ch.maxdim = std::max(ch.maxdim, std::max(F[i].rows, F[i].cols));
  }
  const int rows = F[lo].rows, cols = F[hi - 1].cols;
  auto fwd = [&](int i) { return PIOp{F[i].rowptr, F[i].colind, F[i].val, F[i].rows, 0}; };
  auto adj = [&](int i) { return PIOp{F[i].t_rowptr, F[i].t_colind, F[i].t_val, F[i].cols, 0}; };
  if (cols < rows) {
    // F^H F: x -> F^H (F x); F x applies F[hi-1] first.
    ch.n = cols;
    for (int i = hi - 1; i >= lo; --i) ch.ops[ch.nops++] = fwd(i);
    for (int i = lo; i < hi; ++i) ch.ops[ch.nops++] = adj(i);
  } else {
    // F F^H: x -> F (F^H x); F^H x applies F[lo]^H first.
    ch.n = rows;
    for (int i = lo; i < hi; ++i) ch.ops[ch.nops++] = adj(i);
    for (int i = hi - 1; i >= lo; --i) ch.ops[ch.nops++] = fwd(i);
  }
}

// static shared memory of k_power_iteration (op table, scalars, counters)
// plus slack, kept out of the dynamic allocation
constexpr size_t PI_STATIC_SMEM = 4096;

template <typename T>
__device__ __forceinline__ T absd(T x) {
  return x < T(0) ? -x : x;
}

// Faust::power_iteration on the chain operator: start vector from
// srand(418)/rand() mapped to [-1,1] (Eigen Random), loop while
// |l_old - l| > thr or |l| <= thr (at most max_iter), normalise by 1/||x||,
// x = A x, stop with 0 on a zero vector, l = <x_norm, x>.  Result:
// |sqrt(l)| (Transform::spectralNorm).
//
// The CSR arrays of the chain's products are copied into shared memory once
// (as many as fit after the vectors), so each of the ~2*len products of an
// iteration is a shared-memory pass; the rest are read from L2.
struct PIStaged {
  const int* rp;
  const int* ci;
  const void* v;
  int rows;
  int pad;
};

// The stored entries of one row of one product, held in registers ahead of
// its use (the first PI_PF of them; longer rows read the rest in place).
constexpr int PI_PF = 4;
template <typename TF>
struct PIRow {
  int b, e;
  int c[PI_PF];
  TF v[PI_PF];
};

template <typename TF>
__device__ __forceinline__ void pi_rowptr(const PIStaged& op, int r, int& b, int& e) {
  if (r < op.rows) {
    b = op.rp[r];
    e = op.rp[r + 1];
  } else {
    b = e = 0;
  }
}

template <typename TF>
__device__ __forceinline__ void pi_entries(const PIStaged& op, PIRow<TF>& R) {
  const TF* v = reinterpret_cast<const TF*>(op.v);
#pragma unroll
  for (int u = 0; u < PI_PF; ++u)
    if (R.b + u < R.e) {
      R.c[u] = op.ci[R.b + u];
      R.v[u] = v[R.b + u];
    }
}

template <typename TF, typename TC>
__global__ void __launch_bounds__(PI_THREADS, 1)
    k_power_iteration(const __grid_constant__ PIChain ca, const __grid_constant__ PIChain cb,
                      const PIChain* __restrict__ dchains, int max_iter, TC thr, const TC* __restrict__ x0, PIOut* out,
                      const __grid_constant__ PIPalm palm, int maxn, int smem_bytes) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ PIStaged ops[PI_MAX_OPS];
  __shared__ TC s_inv, s_nrm;
  // rows of more than PI_CHUNK entries of the current product, done one
  // warp each after the thread-per-row pass (list in the dynamic area, room
  // for every row; two counters, used alternately)
  __shared__ int s_nlong[2];
  __shared__ int s_nnz[PI_MAX_OPS];  // stored entries of every product
  __shared__ int s_zero;
  TC* buf0 = reinterpret_cast<TC*>(smem_raw);
  TC* buf1 = buf0 + maxn;
  TC* buf2 = buf1 + maxn;
  TC* lane = buf2 + maxn;
  int* s_long = reinterpret_cast<int*>(lane + CR_LANES);
  unsigned char* pool = reinterpret_cast<unsigned char*>(s_long) + ((long)maxn * 4 + 15) / 16 * 16;
  const long pool_bytes = smem_bytes - (long)(pool - smem_raw);
  const PIChain& ch = dchains ? dchains[blockIdx.x] : ((blockIdx.x == 0) ? ca : cb);
  double result = 1.0;
  int flag = 0;
  int st = 0;
  // a factor without entries makes the product zero (nnz read on the device:
  // factors produced by the PALM loop only know it there); one thread per
  // product reads its count
  if (threadIdx.x == 0) s_zero = 0;
  __syncthreads();
  if (!ch.empty && (int)threadIdx.x < ch.nops) {
    const int nz = ch.ops[threadIdx.x].rowptr[ch.ops[threadIdx.x].rows];
    s_nnz[threadIdx.x] = nz;
    if (nz == 0) s_zero = 1;
  }
  __syncthreads();
  const bool zero = s_zero != 0;
  if (ch.empty) {
    result = 1.0;
  } else if (zero) {
    result = 0.0;
  } else {
    const int n = ch.n;
    // stage the products' CSR arrays (16-byte aligned pieces) while they fit
    if (threadIdx.x == 0) {
      long off = 0;
      for (int o = 0; o < ch.nops; ++o) {
        const PIOp op = ch.ops[o];
        const int nnz = s_nnz[o];
        const long need = ((long)(op.rows + 1) * 4 + 15) / 16 * 16 + ((long)nnz * 4 + 15) / 16 * 16 +
                          ((long)nnz * sizeof(TF) + 15) / 16 * 16;
        if (off + need <= pool_bytes) {
          int* rp = reinterpret_cast<int*>(pool + off);
          off += ((long)(op.rows + 1) * 4 + 15) / 16 * 16;
          int* ci = reinterpret_cast<int*>(pool + off);
          off += ((long)nnz * 4 + 15) / 16 * 16;
          TF* v = reinterpret_cast<TF*>(pool + off);
          off += ((long)nnz * sizeof(TF) + 15) / 16 * 16;
          ops[o] = PIStaged{rp, ci, v, op.rows, 1};
        } else {
          ops[o] = PIStaged{op.rowptr, op.colind, op.val, op.rows, 0};
        }
      }
    }
    __syncthreads();
    // copies of the staged products: the loads of all products are
    // independent, so every thread walks them without waiting in between
    for (int o = 0; o < ch.nops; ++o) {
      if (!ops[o].pad) continue;
      const PIOp op = ch.ops[o];
      const int nnz = s_nnz[o];
      int* rp = const_cast<int*>(ops[o].rp);
      int* ci = const_cast<int*>(ops[o].ci);
      TF* v = reinterpret_cast<TF*>(const_cast<void*>(ops[o].v));
      const TF* gv = reinterpret_cast<const TF*>(op.val);
      for (int i = threadIdx.x; i <= op.rows; i += blockDim.x) rp[i] = __ldg(op.rowptr + i);
      for (int i = threadIdx.x; i < nnz; i += blockDim.x) {
        ci[i] = __ldg(op.colind + i);
        v[i] = __ldg(gv + i);
      }
    }
    __syncthreads();
    // the three vectors are consecutive: vector i at buf0 + i * maxn
    int xi = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) buf0[i] = x0[i];
    __syncthreads();
    // Software pipeline over the products (the same sequence every
    // iteration): while product o is computed, a thread reads the row
    // pointers of its first row of product o + 3 and the entries of that row
    // of product o + 1, so the L2 latency of the products not staged on chip
    // overlaps the work of the products before them.
    const int nops = ch.nops;
    const int r0 = threadIdx.x;
    PIRow<TF> P0, P1;
    int b2, e2, b3, e3;
    pi_rowptr<TF>(ops[0], r0, P0.b, P0.e);
    pi_entries<TF>(ops[0], P0);
    pi_rowptr<TF>(ops[1 % nops], r0, P1.b, P1.e);
    pi_rowptr<TF>(ops[2 % nops], r0, b2, e2);
    TC lam_old = TC(1), lam = TC(0);
    int it = 0;
    bool zero_vec = false;
    if (threadIdx.x == 0) s_nlong[0] = s_nlong[1] = 0;
    int gop = 0;  // products done (selects the long-row counter)
    const int wlane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const TC athr = absd(thr);
    while ((absd(subr(lam_old, lam)) > athr || absd(lam) <= athr) && it < max_iter) {
      ++it;
      lam_old = lam;
      TC* x = buf0 + (long)xi * maxn;
      // scalar FP64 work (sqrt, division) by one thread: GB300's FP64 pipe
      // is narrow, 1024 redundant copies would saturate it
      const TC ss = block_cdot<TC>(x, x, n, lane);
      if (threadIdx.x == 0) {
        s_nrm = sqrtr(ss);
        s_inv = s_nrm == TC(0) ? TC(0) : divr(TC(1), s_nrm);
      }
      __syncthreads();
      const TC nrm = s_nrm;
      if (nrm == TC(0)) {
        st = FGB_ERR_ZERO_NORM;
        break;
      }
      const TC inv = s_inv;
      for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = mulr(x[i], inv);
      __syncthreads();
      // products ping-pong between the two buffers other than x, which keeps
      // the normalised vector for the dot product
      int si = xi, di = (xi + 1) % 3;
      for (int o = 0; o < nops; ++o) {
        const PIStaged op = ops[o];
        const TF* __restrict__ val = reinterpret_cast<const TF*>(op.v);
        const TC* src = buf0 + (long)si * maxn;
        TC* dst = buf0 + (long)di * maxn;
        // issue the loads for later products
        pi_rowptr<TF>(ops[(o + 3) % nops], r0, b3, e3);
        pi_entries<TF>(ops[(o + 1) % nops], P1);
        int* const nlong = &s_nlong[gop & 1];
        if (r0 < op.rows) {
          if (P0.e - P0.b > PI_CHUNK) {
            s_long[atomicAdd(nlong, 1)] = r0;
          } else {
            TC acc = TC(0);
#pragma unroll
            for (int u = 0; u < PI_PF; ++u)
              if (P0.b + u < P0.e) acc = fmad((TC)P0.v[u], src[P0.c[u]], acc);
            for (int p = P0.b + PI_PF; p < P0.e; ++p) acc = fmad((TC)val[p], src[op.ci[p]], acc);
            dst[r0] = acc;
          }
        }
        for (int r = r0 + blockDim.x; r < op.rows; r += blockDim.x) {
          const int p0 = op.rp[r], p1 = op.rp[r + 1];
          if (p1 - p0 > PI_CHUNK) {
            s_long[atomicAdd(nlong, 1)] = r;
            continue;
          }
          TC acc = TC(0);
          for (int p = p0; p < p1; ++p) acc = fmad((TC)val[p], src[op.ci[p]], acc);
          dst[r] = acc;
        }
        __syncthreads();
        {
          const int nl = *nlong;
          if (threadIdx.x == 0) s_nlong[(gop + 1) & 1] = 0;
          for (int q = warp; q < nl; q += nwarps) {
            const int r = s_long[q];
            const TC v = pi_row_warp<TC, TF>(op.ci, val, op.rp[r], op.rp[r + 1], src, wlane);
            if (wlane == 0) dst[r] = v;
          }
          if (nl) __syncthreads();
          ++gop;
        }
        P0 = P1;
        P1.b = b2;
        P1.e = e2;
        b2 = b3;
        e2 = e3;
        si = di;
        di = 3 - xi - si;
      }
      const TC* res = buf0 + (long)si * maxn;
      int nz = 0;
      for (int i = threadIdx.x; i < n; i += blockDim.x) nz |= (res[i] != TC(0));
      if (!__syncthreads_or(nz)) {
        zero_vec = true;
        break;
      }
      lam = block_cdot<TC>(x, res, n, lane);
      xi = si;
    }
    if (st == 0) {
      if (zero_vec) {
        result = 0.0;
        flag = 0;
      } else {
        flag = (it < max_iter) ? it : -1;
        if (threadIdx.x == 0) result = (double)absd(sqrtr(lam));
      }
    }
  }
  if (threadIdx.x == 0) {
    out->norm[blockIdx.x] = result;
    out->flag[blockIdx.x] = flag;
    if (st) atomicCAS(&out->status, 0, st);
    __threadfence();
    const unsigned prev = atomicAdd(&out->done, 1u);
    if (prev == gridDim.x - 1) {
      __threadfence();
      out->done = 0;
      if (palm.enabled) {
        TF* c = reinterpret_cast<TF*>(palm.c);
        TF* alpha = reinterpret_cast<TF*>(palm.alpha);
        const TF lamv = *reinterpret_cast<const TF*>(palm.lambda);
        TF cv;
        if (palm.constant_step) {
          cv = divr(TF(1), (TF)palm.step_size);
        } else {
          const double own = out->norm[0];
          const double nR = palm.ext_norm ? (palm.ext_is_r ? *palm.ext_norm : own) : out->norm[0];
          const double nL = palm.ext_norm ? (palm.ext_is_r ? own : *palm.ext_norm) : out->norm[1];
          if (isnan(nR) || isnan(nL)) atomicCAS(&out->status, 0, (int)FGB_ERR_NAN);
          if ((nR == 0.0 && (palm.it > 0 || !palm.r2l)) || (nL == 0.0 && (palm.it > 0 || palm.r2l)))
            atomicCAS(&out->status, 0, (int)FGB_ERR_ZERO_NORM);
          const double tnR = (double)(TF)nR, tnL = (double)(TF)nL, l = (double)lamv;
          double cc = __dmul_rn(1.001, l);
          cc = __dmul_rn(cc, l);
          cc = __dmul_rn(cc, tnR);
          cc = __dmul_rn(cc, tnR);
          cc = __dmul_rn(cc, tnL);
          cc = __dmul_rn(cc, tnL);
          cv = (TF)cc;
        }
        *c = cv;
        *alpha = divr(lamv, cv);
      }
    }
  }
}

// -1 + (2*r)/RAND_MAX in each precision, the mapping of Eigen's Random().
__global__ void k_start_vectors(int n, const int* __restrict__ rnd, double* __restrict__ xd, float* __restrict__ xf) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    xd[i] = __dadd_rn(-1.0, __ddiv_rn(__dmul_rn(2.0, (double)rnd[i]), (double)RAND_MAX));
    xf[i] = __fadd_rn(-1.f, __fdiv_rn(__fmul_rn(2.f, (float)rnd[i]), (float)RAND_MAX));
  }
}

fgb_status pi_rand_device(fgb_ctx* ctx, int n, const int** d_rand) {
  if (ctx->rand_n < n) {
    // glibc rand() after srand(418) = random()'s TYPE_3 generator with a
    // 128-byte state, reproduced with initstate_r/random_r so the caller's
    // global generator is left alone.
    std::vector<int> h(n);
    static thread_local char state[128];
    struct random_data rd;
    std::memset(&rd, 0, sizeof(rd));
    std::memset(state, 0, sizeof(state));
    initstate_r(418u, state, sizeof(state), &rd);
    for (int i = 0; i < n; ++i) {
      int32_t r;
      random_r(&rd, &r);
      h[i] = r;
    }
    if (ctx->rand_dev) cudaFree(ctx->rand_dev);
    ctx->rand_dev = nullptr;
    ctx->rand_n = 0;
    if (ctx->x0_d) cudaFree(ctx->x0_d);
    if (ctx->x0_f) cudaFree(ctx->x0_f);
    ctx->x0_d = nullptr;
    ctx->x0_f = nullptr;
    FGB_TRY(dmalloc(ctx, (void**)&ctx->rand_dev, sizeof(int) * n));
    FGB_TRY(dmalloc(ctx, (void**)&ctx->x0_d, sizeof(double) * n));
    FGB_TRY(dmalloc(ctx, (void**)&ctx->x0_f, sizeof(float) * n));
    FGB_CUDA(ctx, cudaMemcpy(ctx->rand_dev, h.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    k_start_vectors<<<std::max(1, std::min((n + 255) / 256, 64)), 256, 0, ctx->stream>>>(n, ctx->rand_dev, ctx->x0_d,
                                                                                        ctx->x0_f);
    FGB_LAUNCHED(ctx);
    FGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->rand_n = n;
  }
  *d_rand = ctx->rand_dev;
  return FGB_OK;
}

template <typename TF, typename TC>
static fgb_status launch_pi_t(fgb_ctx* ctx, const PIChain& a, const PIChain& b, int max_iter, double thr,
                              const int* d_rand, PIOut* d_out, const PIPalm& palm, cudaStream_t stream) {
  const int maxn = std::max(1, std::max(a.maxdim, b.maxdim));
  const size_t vec = (3 * (size_t)maxn + CR_LANES) * sizeof(TC) + ((size_t)maxn * 4 + 15) / 16 * 16;
  const size_t cap = std::min<size_t>(ctx->smem_optin > PI_STATIC_SMEM ? ctx->smem_optin - PI_STATIC_SMEM : 0,
                                      216 * 1024);
  if (vec > cap)
    return fail(ctx, FGB_ERR_NOT_SUPPORTED, "power iteration: vector of %d entries does not fit on chip", maxn);
  // the rest of shared memory stages the chain's CSR arrays
  const size_t smem = cap;
  auto kern = k_power_iteration<TF, TC>;
  FGB_TRY(smem_opt_in(ctx, (const void*)kern, smem));
  const TC* x0 = sizeof(TC) == 8 ? (const TC*)(const void*)ctx->x0_d : (const TC*)(const void*)ctx->x0_f;
  (void)d_rand;
  kern<<<palm.ext_norm ? 1 : 2, PI_THREADS, smem, stream>>>(a, b, nullptr, max_iter, (TC)thr, x0, d_out, palm, maxn,
                                                            (int)smem);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

fgb_status launch_power_iteration(fgb_ctx* ctx, fgb_dtype tf, bool fp64, const PIChain& a, const PIChain& b,
                                  int max_iter, double thr, const int* d_rand, PIOut* d_out, const PIPalm& palm,
                                  cudaStream_t stream) {
  if (a.nops > PI_MAX_OPS || b.nops > PI_MAX_OPS) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "power iteration: chain too long");
  if (!stream) stream = ctx->stream;
  if (tf == FGB_F64) return launch_pi_t<double, double>(ctx, a, b, max_iter, thr, d_rand, d_out, palm, stream);
  if (tf == FGB_F32) {
    if (fp64) return launch_pi_t<float, double>(ctx, a, b, max_iter, thr, d_rand, d_out, palm, stream);
    return launch_pi_t<float, float>(ctx, a, b, max_iter, thr, d_rand, d_out, palm, stream);
  }
  return fail(ctx, FGB_ERR_NOT_SUPPORTED, "power iteration: F32 or F64 factors");
}

template <typename TF, typename TC>
static fgb_status launch_pi_many_t(fgb_ctx* ctx, const PIChain* d_chains, int nchains, int maxn, int max_iter,
                                   double thr, PIOut* d_out, cudaStream_t stream) {
  maxn = std::max(1, maxn);
  const size_t vec = (3 * (size_t)maxn + CR_LANES) * sizeof(TC) + ((size_t)maxn * 4 + 15) / 16 * 16;
  const size_t cap = std::min<size_t>(ctx->smem_optin > PI_STATIC_SMEM ? ctx->smem_optin - PI_STATIC_SMEM : 0,
                                      216 * 1024);
  if (vec > cap)
    return fail(ctx, FGB_ERR_NOT_SUPPORTED, "power iteration: vector of %d entries does not fit on chip", maxn);
  const size_t smem = cap;
  auto kern = k_power_iteration<TF, TC>;
  FGB_TRY(smem_opt_in(ctx, (const void*)kern, smem));
  const TC* x0 = sizeof(TC) == 8 ? (const TC*)(const void*)ctx->x0_d : (const TC*)(const void*)ctx->x0_f;
  PIChain none;
  std::memset(&none, 0, sizeof(none));
  none.empty = 1;
  PIPalm palm;
  std::memset(&palm, 0, sizeof(palm));
  kern<<<nchains, PI_THREADS, smem, stream>>>(none, none, d_chains, max_iter, (TC)thr, x0, d_out, palm, maxn,
                                              (int)smem);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

fgb_status launch_power_iteration_many(fgb_ctx* ctx, fgb_dtype tf, bool fp64, const PIChain* d_chains, int nchains,
                                       int maxn, int max_iter, double thr, PIOut* d_out, cudaStream_t stream) {
  if (nchains <= 0 || nchains > PI_MAX_CHAINS)
    return fail(ctx, FGB_ERR_NOT_SUPPORTED, "power iteration: %d chains", nchains);
  if (!stream) stream = ctx->stream;
  if (tf == FGB_F64) return launch_pi_many_t<double, double>(ctx, d_chains, nchains, maxn, max_iter, thr, d_out, stream);
  if (tf == FGB_F32) {
    if (fp64) return launch_pi_many_t<float, double>(ctx, d_chains, nchains, maxn, max_iter, thr, d_out, stream);
    return launch_pi_many_t<float, float>(ctx, d_chains, nchains, maxn, max_iter, thr, d_out, stream);
  }
  return fail(ctx, FGB_ERR_NOT_SUPPORTED, "power iteration: F32 or F64 factors");
}

fgb_status chain_spectral_norm_sync(fgb_ctx* ctx, fgb_dtype dt, const DevFactor* F, int lo, int hi, int max_iter,
                                    double thr, double* norm, int* flag) {
  PIChain a, b;
  pi_chain_build(F, lo, hi, a);
  std::memset(&b, 0, sizeof(b));
  b.empty = 1;
  const int* rnd = nullptr;
  FGB_TRY(pi_rand_device(ctx, std::max(1, a.n), &rnd));
  PIOut* d_out = nullptr;
  FGB_TRY(dmalloc(ctx, (void**)&d_out, sizeof(PIOut)));
  FGB_CUDA(ctx, cudaMemsetAsync(d_out, 0, sizeof(PIOut), ctx->stream));
  PIPalm palm;
  std::memset(&palm, 0, sizeof(palm));
  fgb_status s = launch_power_iteration(ctx, dt, true, a, b, max_iter, thr, rnd, d_out, palm);
  PIOut h;
  std::memset(&h, 0, sizeof(h));
  if (s == FGB_OK) {
    cudaError_t e = cudaMemcpyAsync(&h, d_out, sizeof(PIOut), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) s = cuda_check(ctx, e, "spectral norm");
  }
  dfree(d_out);
  if (s != FGB_OK) return s;
  if (h.status) return fail(ctx, (fgb_status)h.status, "Can't normalize a zero-norm vector.");
  *norm = h.norm[0];
  *flag = h.flag[0];
  return FGB_OK;
}

}  // namespace fgb
