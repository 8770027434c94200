// palm.cu — palm4msa2 (src/algorithm/factorization/faust_palm4msa2020.hpp)
// on the GPU.
//
// Every quantity of the loop stays on the device: factors (CSR + the CSR of
// their transpose, fixed capacities), the packed products pR (L2R) / pL (R2L)
// of init_ite, lambda, the step constant c and alpha = lambda / c.  One outer
// iteration is a fixed sequence of kernels (no host decision inside), so it
// is captured once into a CUDA graph and replayed; the host only checks the
// status word and the cancel flag every few iterations.
//
// Products follow the sparse-chain order of the oracle: each factor is
// applied to a dense block in turn, every entry a sequential fma over the
// factor's stored entries; the residual E = lambda*P - A and the step
// D = S_f - alpha*G are fused into the epilogue of the last product.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "csr.cuh"
#include "power.cuh"
#include "prox.cuh"

namespace fgb {

void free_factor(DevFactor& f);

// ------------------------------------------------------------------ small kernels
template <typename T>
__global__ void k_lambda_minus(const T* __restrict__ P, const T* __restrict__ A, long N, const T* lam,
                               T* __restrict__ out) {
  const T l = *lam;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x)
    out[i] = subr(mulr(l, P[i]), A[i]);
}

template <typename T>
__global__ void k_d_minus(T* __restrict__ D, const T* __restrict__ G, long N, const T* alpha) {
  const T a = *alpha;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x)
    D[i] = subr(D[i], mulr(a, G[i]));
}

// Canonical <A,S> and ||S||^2 (lanes of 256 per chunk of 65536 entries, each
// lane a sequential fma over its entries), every 32 lanes of a chunk on a
// block of one warp: a lane's chain is sequential, and on GB300 an FP64 FMA
// warp instruction takes a scheduler 64 cycles whatever the number of active
// lanes, so the 4096 lanes of a 1024^2 block run on 128 SMs instead of 16.
// The lane values go to `lanes` (chunk c: <A,S> lanes at 512 c, ||S||^2
// lanes at 512 c + 256); k_lambda_lanes adds them by the lane tree.
template <typename T>
__global__ void __launch_bounds__(32) k_lane_dot2(const T* __restrict__ A, const T* __restrict__ S, long N,
                                                 double* __restrict__ lanes) {
  const int c = blockIdx.x / (CR_LANES / 32), t = (blockIdx.x % (CR_LANES / 32)) * 32 + threadIdx.x;
  const long c0 = (long)c * CR_CHUNK, c1 = min(N, c0 + CR_CHUNK);
  T a = T(0), s = T(0);
#pragma unroll 8
  for (long i = c0 + t; i < c1; i += CR_LANES) {
    const T x = A[i], y = S[i];
    a = fmad(x, y, a);
    s = fmad(y, y, s);
  }
  reinterpret_cast<T*>(lanes)[(long)c * 2 * CR_LANES + t] = a;
  reinterpret_cast<T*>(lanes)[(long)c * 2 * CR_LANES + CR_LANES + t] = s;
}

// update_lambda (faust_palm4msa2020.hpp:441-493), lambda = tr / (nS*nS),
// from the lane values of k_lane_dot2: per chunk the pairwise lane tree of
// lane_tree_256, the chunk partials added in order.  One block of 1024
// threads: warp w builds tree w (chunk w / 2, <A,S> or ||S||^2), 32 trees at a
// time, so the trees of a 1024^2 block run side by side.
constexpr int LT_WARPS = 32;
template <typename T>
__global__ void __launch_bounds__(LT_WARPS * 32) k_lambda_lanes(const double* lanes, int nchunks, T* lam,
                                                               int* status, int no_lambda_error) {
  __shared__ T part[LT_WARPS];
  const int t = threadIdx.x & 31, w = threadIdx.x >> 5;
  T tr = T(0), ss = T(0);
  for (int g = 0; g < 2 * nchunks; g += LT_WARPS) {
    if (g + w < 2 * nchunks) {
      const T* l = reinterpret_cast<const T*>(lanes) + (long)(g + w) * CR_LANES;
      const T a0 = addr(l[t], l[t + 128]);
      const T a1 = addr(l[t + 32], l[t + 160]);
      const T a2 = addr(l[t + 64], l[t + 192]);
      const T a3 = addr(l[t + 96], l[t + 224]);
      T c = addr(addr(a0, a2), addr(a1, a3));
#pragma unroll
      for (int s = 16; s >= 1; s >>= 1) c = addr(c, __shfl_down_sync(0xffffffffu, c, s));
      if (t == 0) part[w] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0)
      for (int q = 0; q < LT_WARPS && g + q < 2 * nchunks; q += 2) {
        tr = addr(tr, part[q]);
        ss = addr(ss, part[q + 1]);
      }
    __syncthreads();
  }
  if (threadIdx.x) return;
  const T nS = sqrtr(ss);
  if (nS == T(0)) {
    if (!no_lambda_error) atomicCAS(status, 0, (int)FGB_ERR_ZERO_NORM);
    return;
  }
  if (isnan(tr) || isnan(nS)) {
    if (!no_lambda_error) atomicCAS(status, 0, (int)FGB_ERR_NAN);
    return;
  }
  *lam = divr(tr, mulr(nS, nS));
}

// ||lambda*S - A|| / ||A|| pieces: per chunk sum of e^2 and a^2.
template <typename T>
__global__ void __launch_bounds__(256) k_chunk_relerr(const T* __restrict__ A, const T* __restrict__ S, long N,
                                                     const T* lam, double* part) {
  __shared__ T lane[256];
  const T l = *lam;
  const long c0 = blockIdx.x * CR_CHUNK, c1 = min(N, c0 + CR_CHUNK);
  T e = T(0), a = T(0);
  for (long i = c0 + threadIdx.x; i < c1; i += CR_LANES) {
    const T d = subr(mulr(l, S[i]), A[i]);
    e = fmad(d, d, e);
    a = fmad(A[i], A[i], a);
  }
  lane[threadIdx.x] = e;
  const T pe = lane_tree_256(lane);
  lane[threadIdx.x] = a;
  const T pa = lane_tree_256(lane);
  if (threadIdx.x == 0) {
    reinterpret_cast<T*>(part)[2 * blockIdx.x] = pe;
    reinterpret_cast<T*>(part)[2 * blockIdx.x + 1] = pa;
  }
}

template <typename T>
__global__ void k_relerr_final(const double* part, int nchunks, double* out) {
  T e = T(0), a = T(0);
  for (int c = 0; c < nchunks; ++c) {
    e = addr(e, reinterpret_cast<const T*>(part)[2 * c]);
    a = addr(a, reinterpret_cast<const T*>(part)[2 * c + 1]);
  }
  *out = (double)divr(sqrtr(e), sqrtr(a));
}

template <typename T>
__global__ void k_set_scalar(T* p, double v) {
  *p = (T)v;
}

// ------------------------------------------------------------------ driver
long palm_factor_capacity(const fgb_constraint& c) {
  const long N = (long)c.rows * c.cols;
  long cap = N;
  switch (c.kind) {
    case FGB_SP:
    case FGB_SP_POS: cap = std::min<long>(N, std::max<long long>(c.k, 0)); break;
    case FGB_SPCOL: cap = std::min<long>(N, std::max<long long>(c.k, 0) * c.cols); break;
    case FGB_SPLIN: cap = std::min<long>(N, std::max<long long>(c.k, 0) * c.rows); break;
    case FGB_SPLINCOL: cap = std::min<long>(N, std::max<long long>(c.k, 0) * ((long)c.rows + c.cols)); break;
    default: cap = N;
  }
  return std::max<long>(cap, std::min(c.rows, c.cols));
}

template <typename T>
struct Palm {
  fgb_ctx* ctx = nullptr;
  int J = 0;
  std::vector<fgb_constraint> cons;
  std::vector<DevFactor> S;
  std::vector<T*> packed;
  std::vector<T*> supp;
  const T* A = nullptr;
  int arows = 0, acols = 0;
  T* buf[2] = {nullptr, nullptr};
  T* D = nullptr;
  T* lam = nullptr;
  T* c = nullptr;
  T* alpha = nullptr;
  int* status = nullptr;
  PIOut* pi = nullptr;
  double* part = nullptr;
  double* lanes2 = nullptr;  // lane values of the update_lambda reduction
  const int* rnd = nullptr;
  ProxWork pw;
  fgb_palm_params p;
  bool r2l = false;
  long long graph_nodes = 0;
  // the step-size power iteration (two blocks) runs on a side stream beside
  // the gradient products (whole grid) and joins before alpha is read
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // The chains not yet touched by the current sweep (R_f = S[f+1..J) left to
  // right, L_f = S[0..f) right to left) only hold factors of the previous
  // iteration: their J norms are computed in one launch at the start of the
  // iteration, on a second side stream; each update then iterates only its
  // other chain.
  bool hoist = false;
  cudaStream_t side2 = nullptr;
  cudaEvent_t ev_it = nullptr, ev_old = nullptr;
  PIChain* d_old_chains = nullptr;
  PIOut* pi_old = nullptr;
  int old_maxn = 0;

  ~Palm() {
    if (side) cudaStreamDestroy(side);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (side2) cudaStreamDestroy(side2);
    if (ev_it) cudaEventDestroy(ev_it);
    if (ev_old) cudaEventDestroy(ev_old);
    dfree(d_old_chains);
    dfree(pi_old);
    for (auto& f : S) free_factor(f);
    for (auto* q : packed) dfree(q);
    for (auto* q : supp) dfree(q);
    dfree(buf[0]);
    dfree(buf[1]);
    dfree(D);
    dfree(lam);
    dfree(c);
    dfree(alpha);
    dfree(status);
    dfree(pi);
    dfree(part);
    dfree(lanes2);
    prox_work_free(pw);
  }

  int grid(long n) const { return (int)std::max(1L, std::min((n + 255) / 256, 4L * ctx->sm_count)); }

  // The factors' longest row (d_maxrc[0]) and column (d_maxrc[1]) are on the
  // device; the long-row kernels read them and end at once without long rows.
  static const int* dmax(const DevFactor& f, int which) { return f.d_maxrc ? f.d_maxrc + which : nullptr; }
  // Y = S X
  fgb_status mul_S(const DevFactor& f, const T* X, int ncols, T* Y, const Epi<T>& e) {
    return launch_csr_spmm<T>(ctx, f.rowptr, f.colind, (const T*)f.val, f.rows, f.cols, X, f.cols, ncols, Y, f.rows, e,
                              -1, dmax(f, 0));
  }
  // Y = S^H X (transpose CSR)
  fgb_status mul_SH(const DevFactor& f, const T* X, int ncols, T* Y, const Epi<T>& e) {
    return launch_csr_spmm<T>(ctx, f.t_rowptr, f.t_colind, (const T*)f.t_val, f.cols, f.rows, X, f.rows, ncols, Y,
                              f.cols, e, -1, dmax(f, 1));
  }
  // Y = X S (X: xrows x f.rows)
  fgb_status mul_XS(const T* X, int xrows, const DevFactor& f, T* Y, const Epi<T>& e) {
    return launch_dense_csrT<T>(ctx, X, xrows, xrows, f.t_rowptr, f.t_colind, (const T*)f.t_val, f.cols, f.rows, Y,
                                xrows, e, -1, dmax(f, 1));
  }
  // Y = X S^H (X: xrows x f.cols)
  fgb_status mul_XSH(const T* X, int xrows, const DevFactor& f, T* Y, const Epi<T>& e) {
    return launch_dense_csrT<T>(ctx, X, xrows, xrows, f.rowptr, f.colind, (const T*)f.val, f.rows, f.cols, Y, xrows,
                                e, -1, dmax(f, 0));
  }
  fgb_status dense_of(const DevFactor& f, T* out) { return launch_csr_to_dense<T>(ctx, f, out); }

  // ---------------------------------------------------------------- setup
  fgb_status setup(const T* A_dev, int rows, int cols, const fgb_constraint* cs, int nf, const fgb_palm_params& pp,
                   const void* const* init_facts, double init_lambda, const DevFactor* init_dev = nullptr) {
    J = nf;
    p = pp;
    r2l = p.is_update_way_R2L != 0;
    A = A_dev;
    arows = rows;
    acols = cols;
    cons.assign(cs, cs + nf);
    if (p.no_normalization)
      for (auto& c0 : cons) c0.normalized = 0;
    int maxdim = std::max(rows, cols);
    for (int i = 0; i < J; ++i) maxdim = std::max(maxdim, std::max(cons[i].rows, cons[i].cols));
    const size_t es = sizeof(T);
    FGB_TRY(dmalloc(ctx, (void**)&buf[0], es * (size_t)maxdim * maxdim));
    FGB_TRY(dmalloc(ctx, (void**)&buf[1], es * (size_t)maxdim * maxdim));
    FGB_TRY(dmalloc(ctx, (void**)&D, es * (size_t)maxdim * maxdim));
    FGB_TRY(dmalloc(ctx, (void**)&lam, sizeof(double)));
    FGB_TRY(dmalloc(ctx, (void**)&c, sizeof(double)));
    FGB_TRY(dmalloc(ctx, (void**)&alpha, sizeof(double)));
    FGB_TRY(dmalloc(ctx, (void**)&status, sizeof(int)));
    FGB_TRY(dmalloc(ctx, (void**)&pi, sizeof(PIOut)));
    FGB_TRY(dmalloc(ctx, (void**)&part, sizeof(double) * 2 * ((size_t)maxdim * maxdim / CR_CHUNK + 2)));
    FGB_TRY(dmalloc(ctx, (void**)&lanes2, sizeof(double) * 2 * CR_LANES * ((size_t)maxdim * maxdim / CR_CHUNK + 2)));
    FGB_CUDA(ctx, cudaMemsetAsync(status, 0, sizeof(int), ctx->stream));
    FGB_CUDA(ctx, cudaMemsetAsync(pi, 0, sizeof(PIOut), ctx->stream));
    k_set_scalar<T><<<1, 1, 0, ctx->stream>>>(lam, init_lambda);
    FGB_LAUNCHED(ctx);
    FGB_TRY(pi_rand_device(ctx, maxdim, &rnd));
    FGB_TRY(prox_work_reserve(ctx, pw, (long)maxdim * maxdim, 2 * maxdim + 2));
    packed.assign(J, nullptr);
    supp.assign(J, nullptr);
    S.resize(J);
    for (int i = 0; i < J; ++i) {
      FGB_TRY(dmalloc(ctx, (void**)&packed[i], es * (size_t)maxdim * maxdim));
      DevFactor& f = S[i];
      f.format = FGB_CSR;
      f.rows = cons[i].rows;
      f.cols = cons[i].cols;
      f.cap = (int)palm_factor_capacity(cons[i]);
      FGB_TRY(dmalloc(ctx, (void**)&f.rowptr, sizeof(int) * (f.rows + 1)));
      FGB_TRY(dmalloc(ctx, (void**)&f.colind, sizeof(int) * f.cap));
      FGB_TRY(dmalloc(ctx, &f.val, es * f.cap));
      FGB_TRY(dmalloc(ctx, (void**)&f.t_rowptr, sizeof(int) * (f.cols + 1)));
      FGB_TRY(dmalloc(ctx, (void**)&f.t_colind, sizeof(int) * f.cap));
      FGB_TRY(dmalloc(ctx, &f.t_val, es * f.cap));
      FGB_TRY(dmalloc(ctx, (void**)&f.d_maxrc, 2 * sizeof(int)));
      if (cons[i].kind == FGB_SUPP) {
        FGB_TRY(dmalloc(ctx, (void**)&supp[i], es * (size_t)f.rows * f.cols));
        FGB_CUDA(ctx, cudaMemcpyAsync(supp[i], cons[i].supp, es * (size_t)f.rows * f.cols, cudaMemcpyHostToDevice,
                                      ctx->stream));
      }
    }
    // Initial factors (faust_palm4msa2020.hpp:115-149): the first factor to
    // update is zero, the others identity; or the caller's init_facts.
    std::vector<T> h;
    for (int i = 0; i < J && init_dev; ++i) {
      // device-resident initial factors (CSR): densified, then the usual
      // dense -> CSR of the factor (its transpose included)
      DevFactor& f = S[i];
      const DevFactor& g = init_dev[i];
      if (g.rows != f.rows || g.cols != f.cols)
        return fail(ctx, FGB_ERR_INVALID_ARG, "initial factor %d is %d x %d, the constraint %d x %d", i, g.rows, g.cols,
                    f.rows, f.cols);
      if (g.nnz > f.cap) {
        dfree(f.colind);
        dfree(f.val);
        dfree(f.t_colind);
        dfree(f.t_val);
        f.cap = g.nnz;
        FGB_TRY(dmalloc(ctx, (void**)&f.colind, sizeof(int) * f.cap));
        FGB_TRY(dmalloc(ctx, &f.val, es * f.cap));
        FGB_TRY(dmalloc(ctx, (void**)&f.t_colind, sizeof(int) * f.cap));
        FGB_TRY(dmalloc(ctx, &f.t_val, es * f.cap));
      }
      FGB_TRY(launch_csr_to_dense<T>(ctx, g, D));
      FGB_TRY(launch_dense_to_csr<T>(ctx, pw, D, f, status));
    }
    if (init_dev) {
      FGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      return FGB_OK;
    }
    for (int i = 0; i < J; ++i) {
      DevFactor& f = S[i];
      h.assign((size_t)f.rows * f.cols, T(0));
      if (init_facts) {
        std::memcpy(h.data(), init_facts[i], es * h.size());
      } else {
        const bool zero = r2l ? (i == J - 1) : (i == 0);
        if (!zero)
          for (int d = 0; d < std::min(f.rows, f.cols); ++d) h[(size_t)d * f.rows + d] = T(1);
      }
      long nnz = 0;
      for (auto v : h) nnz += v != T(0);
      if (nnz > f.cap) {
        // grow the capacity for an initial factor denser than the constraint allows
        dfree(f.colind);
        dfree(f.val);
        dfree(f.t_colind);
        dfree(f.t_val);
        f.cap = (int)nnz;
        FGB_TRY(dmalloc(ctx, (void**)&f.colind, sizeof(int) * f.cap));
        FGB_TRY(dmalloc(ctx, &f.val, es * f.cap));
        FGB_TRY(dmalloc(ctx, (void**)&f.t_colind, sizeof(int) * f.cap));
        FGB_TRY(dmalloc(ctx, &f.t_val, es * f.cap));
      }
      FGB_CUDA(ctx, cudaMemcpyAsync(D, h.data(), es * h.size(), cudaMemcpyHostToDevice, ctx->stream));
      FGB_TRY(launch_dense_to_csr<T>(ctx, pw, D, f, status));
      FGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return FGB_OK;
  }

  // ---------------------------------------------------------------- one iteration
  fgb_status step_size(int f, int it) {
    PIChain a, b;
    PIPalm pp;
    std::memset(&pp, 0, sizeof(pp));
    if (p.constant_step_size) {
      std::memset(&a, 0, sizeof(a));
      std::memset(&b, 0, sizeof(b));
      a.empty = b.empty = 1;
    } else if (hoist) {
      // only the chain the sweep has already updated; the other norm comes
      // from the launch at the start of the iteration
      std::memset(&b, 0, sizeof(b));
      b.empty = 1;
      if (!r2l)
        pi_chain_build(S.data(), 0, f, a);  // L
      else
        pi_chain_build(S.data(), f + 1, J, a);  // R
      pp.ext_norm = &pi_old->norm[f];
      pp.ext_is_r = r2l ? 0 : 1;
      FGB_CUDA(ctx, cudaStreamWaitEvent(side, ev_old, 0));
    } else {
      pi_chain_build(S.data(), f + 1, J, a);  // R
      pi_chain_build(S.data(), 0, f, b);      // L
    }
    pp.enabled = 1;
    pp.it = it;
    pp.r2l = r2l ? 1 : 0;
    pp.constant_step = p.constant_step_size;
    pp.step_size = p.step_size;
    pp.lambda = lam;
    pp.c = c;
    pp.alpha = alpha;
    const bool fp64 = sizeof(T) == 8 || p.norm2_fp64;
    return launch_power_iteration(ctx, sizeof(T) == 8 ? FGB_F64 : FGB_F32, fp64, a, b, p.norm2_max_iter,
                                  p.norm2_threshold, rnd, pi, pp, side);
  }

  fgb_status init_ite() {
    if (J < 2) return FGB_OK;
    const Epi<T> st;
    if (!r2l) {
      // pR[J-2] = S[J-1]; pR[i] = S[i+1] pR[i+1]  (dims n_{i+1} x m_{J-1})
      FGB_TRY(dense_of(S[J - 1], packed[J - 2]));
      for (int i = J - 3; i >= 0; --i) FGB_TRY(mul_S(S[i + 1], packed[i + 1], acols, packed[i], st));
    } else {
      // pL[1] = S[0]; pL[i] = pL[i-1] S[i-1]  (dims n_0 x m_{i-1})
      FGB_TRY(dense_of(S[0], packed[1]));
      for (int i = 2; i < J; ++i) FGB_TRY(mul_XS(packed[i - 1], arows, S[i - 1], packed[i], st));
    }
    return FGB_OK;
  }

  fgb_status update_fact(int f, int it) {
    FGB_CUDA(ctx, cudaEventRecord(ev_fork, ctx->stream));
    FGB_CUDA(ctx, cudaStreamWaitEvent(side, ev_fork, 0));
    FGB_TRY(step_size(f, it));
    FGB_CUDA(ctx, cudaEventRecord(ev_join, side));
    const bool hasL = f > 0, hasR = f + 1 < J;
    const DevFactor& Sf = S[f];
    Epi<T> st;
    Epi<T> eE;
    eE.mode = EPI_LAMBDA_MINUS;
    eE.aux = A;
    eE.ld_aux = arows;
    eE.scal = lam;
    Epi<T> eD;
    eD.mode = EPI_D_MINUS;
    eD.aux = D;
    eD.ld_aux = Sf.rows;
    eD.scal = alpha;
    // dense image of the current factor (the D of update_fact)
    FGB_TRY(dense_of(Sf, D));
    int cur = 0;
    T* E = nullptr;
    // ---- E = lambda * L D R - A
    if (!r2l) {
      const int nL = f;  // products S_{f-1} .. S_0 after the first
      if (hasR) {
        FGB_TRY(mul_S(Sf, packed[f], acols, buf[cur], nL == 0 ? eE : st));
      } else if (nL == 0) {
        k_lambda_minus<T><<<grid((long)arows * acols), 256, 0, ctx->stream>>>(D, A, (long)arows * acols, lam, buf[cur]);
        FGB_LAUNCHED(ctx);
      } else {
        FGB_TRY(dense_of(Sf, buf[cur]));
      }
      const T* src = (hasR || nL == 0) ? buf[cur] : buf[cur];
      for (int l = f - 1; l >= 0; --l) {
        FGB_TRY(mul_S(S[l], src, acols, buf[cur ^ 1], l == 0 ? eE : st));
        cur ^= 1;
        src = buf[cur];
      }
      E = buf[cur];
    } else {
      const int nR = J - 1 - f;
      if (hasL) {
        FGB_TRY(mul_XS(packed[f], arows, Sf, buf[cur], nR == 0 ? eE : st));
      } else if (nR == 0) {
        k_lambda_minus<T><<<grid((long)arows * acols), 256, 0, ctx->stream>>>(D, A, (long)arows * acols, lam, buf[cur]);
        FGB_LAUNCHED(ctx);
      } else {
        FGB_TRY(dense_of(Sf, buf[cur]));
      }
      for (int l = f + 1; l < J; ++l) {
        FGB_TRY(mul_XS(buf[cur], arows, S[l], buf[cur ^ 1], l == J - 1 ? eE : st));
        cur ^= 1;
      }
      E = buf[cur];
    }
    // ---- G = L^H E R^H, D = S_f - alpha G (fused into the last product)
    // shape of the running block: rows x cols
    int rows = arows, cols = acols;
    std::vector<std::pair<int, int>> ops;  // (kind 0 = S^H left, 1 = X S^H right, factor)
    if (!r2l) {
      for (int l = 0; l < f; ++l) ops.push_back({0, l});
      for (int l = J - 1; l > f; --l) ops.push_back({1, l});
    } else {
      for (int l = J - 1; l > f; --l) ops.push_back({1, l});
      for (int l = 0; l < f; ++l) ops.push_back({0, l});
    }
    if (ops.empty()) {
      FGB_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ev_join, 0));
      k_d_minus<T><<<grid((long)Sf.rows * Sf.cols), 256, 0, ctx->stream>>>(D, E, (long)Sf.rows * Sf.cols, alpha);
      FGB_LAUNCHED(ctx);
    } else {
      const T* src = E;
      for (size_t q = 0; q < ops.size(); ++q) {
        const bool last = q + 1 == ops.size();
        const DevFactor& F = S[ops[q].second];
        T* dst = last ? D : buf[cur ^ 1];
        if (last) FGB_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ev_join, 0));
        if (ops[q].first == 0) {
          FGB_TRY(mul_SH(F, src, cols, dst, last ? eD : st));
          rows = F.cols;
        } else {
          FGB_TRY(mul_XSH(src, rows, F, dst, last ? eD : st));
          cols = F.rows;
        }
        if (!last) {
          cur ^= 1;
          src = buf[cur];
        }
      }
    }
    // ---- projection and replacement
    FGB_TRY(launch_prox<T>(ctx, pw, cons[f], D, Sf.rows, Sf.cols, supp[f], status));
    FGB_TRY(launch_dense_to_csr<T>(ctx, pw, D, S[f], status));
    return FGB_OK;
  }

  fgb_status update_lambda() {
    // S_mat following the reuse rule of :449-468.
    T* Smat = nullptr;
    const Epi<T> st;
    const bool reuse = p.packing_RL || J <= 2;
    if (J == 1) {
      FGB_TRY(dense_of(S[0], buf[0]));
      Smat = buf[0];
    } else {
      bool use_pR0 = false;
      if (reuse) {
        const long lhs = (long)S[0].cols * cons[1].rows;
        const long rhs = (long)cons[J - 2].cols * S[J - 1].rows;
        use_pR0 = lhs < rhs;
      }
      if (reuse && !r2l && use_pR0) {
        FGB_TRY(mul_S(S[0], packed[0], acols, buf[0], st));  // pR[0] from init_ite
        Smat = buf[0];
      } else if (reuse && r2l && !use_pR0) {
        FGB_TRY(mul_XS(packed[J - 1], arows, S[J - 1], buf[0], st));  // pL[n-1] from init_ite
        Smat = buf[0];
      } else {
        int cur = 0;
        FGB_TRY(dense_of(S[J - 1], buf[cur]));
        for (int l = J - 2; l >= 0; --l) {
          FGB_TRY(mul_S(S[l], buf[cur], acols, buf[cur ^ 1], st));
          cur ^= 1;
        }
        Smat = buf[cur];
      }
    }
    const long N = (long)arows * acols;
    const int nch = (int)((N + CR_CHUNK - 1) / CR_CHUNK);
    k_lane_dot2<T><<<nch * (CR_LANES / 32), 32, 0, ctx->stream>>>(A, Smat, N, lanes2);
    FGB_LAUNCHED(ctx);
    k_lambda_lanes<T><<<1, LT_WARPS * 32, 0, ctx->stream>>>(lanes2, nch, lam, status, p.no_lambda_error);
    FGB_LAUNCHED(ctx);
    return FGB_OK;
  }

  fgb_status iteration(int it) {
    if (hoist) {
      FGB_CUDA(ctx, cudaEventRecord(ev_it, ctx->stream));
      FGB_CUDA(ctx, cudaStreamWaitEvent(side2, ev_it, 0));
      const bool fp64 = sizeof(T) == 8 || p.norm2_fp64;
      FGB_TRY(launch_power_iteration_many(ctx, sizeof(T) == 8 ? FGB_F64 : FGB_F32, fp64, d_old_chains, J, old_maxn,
                                          p.norm2_max_iter, p.norm2_threshold, pi_old, side2));
      FGB_CUDA(ctx, cudaEventRecord(ev_old, side2));
    }
    FGB_TRY(init_ite());
    for (int s = 0; s < J; ++s) FGB_TRY(update_fact(r2l ? J - 1 - s : s, it));
    if (!p.no_lambda) FGB_TRY(update_lambda());
    return FGB_OK;
  }

  // the run's status word, then the power iterations' (zero or NaN norms)
  fgb_status read_status(int* st) {
    int h[3] = {0, 0, 0};
    FGB_CUDA(ctx, cudaMemcpyAsync(&h[0], status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    FGB_CUDA(ctx, cudaMemcpyAsync(&h[1], &pi->status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    if (pi_old)
      FGB_CUDA(ctx, cudaMemcpyAsync(&h[2], &pi_old->status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    FGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *st = h[0] ? h[0] : (h[1] ? h[1] : h[2]);
    return FGB_OK;
  }

  fgb_status run() {
    if (p.nb_it <= 0) return FGB_OK;
    if (!side) {
      FGB_CUDA(ctx, cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
      FGB_CUDA(ctx, cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
      FGB_CUDA(ctx, cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    }
    hoist = !p.constant_step_size && J >= 2 && J <= PI_MAX_CHAINS && !getenv("FGB_NO_PI_HOIST");
    if (hoist && !d_old_chains) {
      // chain f: the factors the sweep reaches after f (their buffers do not
      // move during the run, so the descriptors are built once)
      std::vector<PIChain> h(J);
      old_maxn = 1;
      for (int f = 0; f < J; ++f) {
        if (!r2l)
          pi_chain_build(S.data(), f + 1, J, h[f]);
        else
          pi_chain_build(S.data(), 0, f, h[f]);
        if (h[f].nops > PI_MAX_OPS) hoist = false;
        old_maxn = std::max(old_maxn, h[f].maxdim);
      }
      if (hoist) {
        FGB_TRY(dmalloc(ctx, (void**)&d_old_chains, sizeof(PIChain) * J));
        FGB_TRY(dmalloc(ctx, (void**)&pi_old, sizeof(PIOut)));
        FGB_CUDA(ctx, cudaMemcpy(d_old_chains, h.data(), sizeof(PIChain) * J, cudaMemcpyHostToDevice));
        FGB_CUDA(ctx, cudaMemset(pi_old, 0, sizeof(PIOut)));
        FGB_CUDA(ctx, cudaStreamCreateWithFlags(&side2, cudaStreamNonBlocking));
        FGB_CUDA(ctx, cudaEventCreateWithFlags(&ev_it, cudaEventDisableTiming));
        FGB_CUDA(ctx, cudaEventCreateWithFlags(&ev_old, cudaEventDisableTiming));
      }
    }
    // iteration 0 eagerly (its zero-norm rule differs), the rest as a graph
    FGB_TRY(iteration(0));
    int st = 0;
    FGB_TRY(read_status(&st));
    if (st) return fail(ctx, (fgb_status)st, "palm4msa2: %s at iteration 0", status_text(st));
    if (p.nb_it == 1) return FGB_OK;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool use_graph = ctx->stream != nullptr && !getenv("FGB_NO_GRAPH");
    if (use_graph) {
      // capture iterations >= 1 once; on any capture failure run eagerly
      const long long l0 = ctx->launches.load();
      bool ok = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
      fgb_status s = ok ? iteration(1) : FGB_ERR_CUDA;
      cudaError_t e = ok ? cudaStreamEndCapture(ctx->stream, &graph) : cudaErrorUnknown;
      ok = ok && s == FGB_OK && e == cudaSuccess && graph;
      if (ok) ok = cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
      if (ok) {
        size_t nodes = 0;
        cudaGraphGetNodes(graph, nullptr, &nodes);
        graph_nodes = (long long)nodes;
      } else {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        cudaGetLastError();
        use_graph = false;
      }
      ctx->launches.store(l0);
      ctx->err.clear();
    }
    fgb_status result = FGB_OK;
    for (int it = 1; it < p.nb_it; ++it) {
      if (ctx->cancel_host && *ctx->cancel_host) {
        *ctx->cancel_host = 0;
        result = fail(ctx, FGB_ERR_CANCELLED, "palm4msa2 cancelled at iteration %d", it);
        break;
      }
      if (use_graph) {
        cudaError_t e = cudaGraphLaunch(exec, ctx->stream);
        if (e != cudaSuccess) {
          result = cuda_check(ctx, e, "cudaGraphLaunch");
          break;
        }
        ctx->launches.fetch_add(graph_nodes);
      } else {
        result = iteration(it);
        if (result != FGB_OK) break;
      }
      if ((it & 7) == 0 || it + 1 == p.nb_it) {
        result = read_status(&st);
        if (result != FGB_OK) break;
        if (st) {
          result = fail(ctx, (fgb_status)st, "palm4msa2: %s near iteration %d", status_text(st), it);
          break;
        }
      }
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    return result;
  }

  static const char* status_text(int st) {
    switch (st) {
      case FGB_ERR_ZERO_NORM: return "zero norm (2-norm of L or R, a factor, or S in update_lambda)";
      case FGB_ERR_NAN: return "NaN in a 2-norm or in lambda";
      case FGB_ERR_INVALID_ARG: return "inconsistent selection state";
      default: return "error";
    }
  }
};

// Transfers the factors of a finished run into a Faust handle.
template <typename T>
static fgb_status palm_to_faust(Palm<T>& P, fgb_dtype dt, fgb_faust** out) {
  fgb_faust* F = new fgb_faust();
  F->ctx = P.ctx;
  F->dtype = dt;
  F->f = P.S;
  P.S.clear();
  for (auto& f : F->f) {
    int nnz = 0;
    cudaMemcpy(&nnz, f.rowptr + f.rows, sizeof(int), cudaMemcpyDeviceToHost);
    f.nnz = nnz;
    f.has_t = true;
  }
  *out = F;
  return FGB_OK;
}

template <typename T>
static fgb_status palm_entry(fgb_ctx* ctx, fgb_dtype dt, const void* A_dev, int rows, int cols, int nfacts,
                             const fgb_constraint* cons, const fgb_palm_params* params, const void* const* init_facts,
                             double* lambda, fgb_faust** out) {
  if (nfacts <= 0 || !cons) return fail(ctx, FGB_ERR_INVALID_ARG, "No constraint passed to palm4msa.");
  if (cons[0].rows != rows || cons[nfacts - 1].cols != cols)
    return fail(ctx, FGB_ERR_INVALID_ARG, "constraint shapes do not match A (%d x %d)", rows, cols);
  for (int i = 0; i < nfacts; ++i) {
    if (cons[i].rows <= 0 || cons[i].cols <= 0) return fail(ctx, FGB_ERR_INVALID_ARG, "constraint %d: bad shape", i);
    if (i > 0 && cons[i - 1].cols != cons[i].rows)
      return fail(ctx, FGB_ERR_INVALID_ARG, "constraint %d rows != constraint %d cols", i, i - 1);
    if (cons[i].kind == FGB_SUPP && !cons[i].supp) return fail(ctx, FGB_ERR_INVALID_ARG, "SUPP without support");
    if ((cons[i].kind == FGB_NORMCOL || cons[i].kind == FGB_NORMLIN) && cons[i].s < 0)
      return fail(ctx, FGB_ERR_INVALID_ARG, "Faust::prox_normcol : s < 0 ");
  }
  if (params->norm2_max_iter <= 0 && !params->constant_step_size)
    return fail(ctx, FGB_ERR_INVALID_ARG, "power_iteration :  nbr_iter_max <= 0");
  FGB_CUDA(ctx, cudaSetDevice(ctx->device));
  // The run uses a private stream (capturable into a graph even when the
  // caller works on the legacy default stream), ordered after the caller's.
  cudaStream_t user = ctx->stream, ps = nullptr;
  FGB_CUDA(ctx, cudaStreamSynchronize(user));
  FGB_CUDA(ctx, cudaStreamCreateWithFlags(&ps, cudaStreamNonBlocking));
  ctx->stream = ps;
  fgb_status s;
  {
    Palm<T> P;
    P.ctx = ctx;
    s = P.setup((const T*)A_dev, rows, cols, cons, nfacts, *params, init_facts, lambda ? *lambda : 1.0);
    if (s == FGB_OK) s = P.run();
    if (s == FGB_OK) {
      T lt;
      s = cuda_check(ctx, cudaMemcpy(&lt, P.lam, sizeof(T), cudaMemcpyDeviceToHost), "read lambda");
      if (s == FGB_OK && lambda) *lambda = (double)lt;
    }
    if (s == FGB_OK && out) s = palm_to_faust(P, dt, out);
    cudaStreamSynchronize(ps);
  }
  ctx->stream = user;
  cudaStreamDestroy(ps);
  return s;
}

// Reads the entry counts of factors left on the device by a finished run.
static fgb_status read_nnz(fgb_ctx* ctx, std::vector<DevFactor>& S) {
  for (auto& f : S) {
    int nnz = 0;
    FGB_CUDA(ctx, cudaMemcpy(&nnz, f.rowptr + f.rows, sizeof(int), cudaMemcpyDeviceToHost));
    f.nnz = nnz;
    f.has_t = true;
  }
  return FGB_OK;
}

// Faust::hierarchical (src/algorithm/factorization/faust_hierarchical.hpp:1-121),
// 2020 version: step i splits the current residual (the last factor, or the
// first when is_fact_side_left) in two by palm4msa2 with the constraints
// (fac_i, res_i) from the default zero / identity start and lambda 1, the
// global lambda is multiplied by that run's lambda, the two factors replace
// the residual, and palm4msa2 then refines every factor against A starting
// from them and from the global lambda.
template <typename T>
static fgb_status hier_impl(fgb_ctx* ctx, fgb_dtype dt, const void* A_host, int rows, int cols, int nsteps,
                            const fgb_constraint* fac, const fgb_constraint* res, const fgb_palm_params* p2,
                            const fgb_palm_params* pg, int left, double* lambda, fgb_faust** out) {
  if (nsteps <= 0 || !fac || !res) return fail(ctx, FGB_ERR_INVALID_ARG, "hierarchical: no constraint");
  const size_t es = sizeof(T);
  T* A = nullptr;
  T* dense = nullptr;
  FGB_TRY(dmalloc(ctx, (void**)&A, es * (size_t)rows * cols));
  fgb_status s = cuda_check(ctx, cudaMemcpy(A, A_host, es * (size_t)rows * cols, cudaMemcpyHostToDevice), "copy A");
  cudaStream_t user = ctx->stream, ps = nullptr;
  if (s == FGB_OK) s = cuda_check(ctx, cudaStreamCreateWithFlags(&ps, cudaStreamNonBlocking), "stream");
  if (s == FGB_OK) ctx->stream = ps;
  std::vector<DevFactor> S;
  double glo_lambda = 1.0;
  for (int i = 0; i < nsteps && s == FGB_OK; ++i) {
    // the matrix split at this step
    const T* Si = A;
    int sr = rows, sc = cols;
    if (i > 0) {
      const DevFactor& r = left ? S.front() : S.back();
      sr = r.rows;
      sc = r.cols;
      dfree(dense);
      dense = nullptr;
      s = dmalloc(ctx, (void**)&dense, es * (size_t)sr * sc);
      if (s == FGB_OK) s = launch_csr_to_dense<T>(ctx, r, dense);
      Si = dense;
    }
    if (s != FGB_OK) break;
    const fgb_constraint lc[2] = {left ? res[i] : fac[i], left ? fac[i] : res[i]};
    if (lc[0].rows != sr || lc[1].cols != sc || lc[0].cols != lc[1].rows) {
      s = fail(ctx, FGB_ERR_INVALID_ARG, "hierarchical step %d: constraints %dx%d, %dx%d do not split %d x %d", i,
               lc[0].rows, lc[0].cols, lc[1].rows, lc[1].cols, sr, sc);
      break;
    }
    std::vector<DevFactor> two;
    double lam_local = 1.0;
    {
      Palm<T> L;
      L.ctx = ctx;
      s = L.setup(Si, sr, sc, lc, 2, *p2, nullptr, 1.0);
      if (s == FGB_OK) s = L.run();
      T lt = T(1);
      if (s == FGB_OK) s = cuda_check(ctx, cudaMemcpy(&lt, L.lam, sizeof(T), cudaMemcpyDeviceToHost), "lambda");
      lam_local = (double)lt;
      if (s == FGB_OK) {
        two = L.S;
        L.S.clear();
        s = read_nnz(ctx, two);
      }
    }
    if (s != FGB_OK) {
      for (auto& f : two) free_factor(f);
      break;
    }
    glo_lambda *= lam_local;
    if (i > 0) {
      if (left) {
        free_factor(S.front());
        S.erase(S.begin());
      } else {
        free_factor(S.back());
        S.pop_back();
      }
    }
    if (left)
      S.insert(S.begin(), two.begin(), two.end());
    else
      S.insert(S.end(), two.begin(), two.end());
    // constraints of the global run, in the order of the factors
    std::vector<fgb_constraint> gc;
    if (left) {
      gc.push_back(res[i]);
      for (int j = i; j >= 0; --j) gc.push_back(fac[j]);
    } else {
      for (int j = 0; j <= i; ++j) gc.push_back(fac[j]);
      gc.push_back(res[i]);
    }
    {
      Palm<T> G;
      G.ctx = ctx;
      s = G.setup(A, rows, cols, gc.data(), (int)gc.size(), *pg, nullptr, glo_lambda, S.data());
      if (s == FGB_OK) s = G.run();
      T lt = T(1);
      if (s == FGB_OK) s = cuda_check(ctx, cudaMemcpy(&lt, G.lam, sizeof(T), cudaMemcpyDeviceToHost), "lambda");
      if (s == FGB_OK) {
        glo_lambda = (double)lt;
        for (auto& f : S) free_factor(f);
        S = G.S;
        G.S.clear();
        s = read_nnz(ctx, S);
      }
    }
  }
  if (ps) cudaStreamSynchronize(ps);
  ctx->stream = user;
  if (ps) cudaStreamDestroy(ps);
  dfree(dense);
  dfree(A);
  if (s != FGB_OK) {
    for (auto& f : S) free_factor(f);
    return s;
  }
  if (lambda) *lambda = glo_lambda;
  if (out) {
    fgb_faust* F = new fgb_faust();
    F->ctx = ctx;
    F->dtype = dt;
    F->f = S;
    *out = F;
  } else {
    for (auto& f : S) free_factor(f);
  }
  return FGB_OK;
}

}  // namespace fgb

using namespace fgb;

extern "C" {

fgb_status fgb_palm_params_default(fgb_palm_params* p) {
  if (!p) return FGB_ERR_INVALID_ARG;
  p->nb_it = 200;
  p->is_update_way_R2L = 0;
  p->packing_RL = 1;
  p->no_normalization = 0;
  p->no_lambda = 0;
  p->norm2_threshold = 1e-6;
  p->norm2_max_iter = 100;
  p->constant_step_size = 0;
  p->step_size = 1e-16;
  p->no_lambda_error = 0;
  p->norm2_fp64 = 0;
  return FGB_OK;
}

fgb_status fgb_prox(fgb_ctx* ctx, fgb_dtype dtype, const fgb_constraint* cons, void* M) {
  if (!ctx || !cons || !M) return FGB_ERR_INVALID_ARG;
  if (dtype != FGB_F32 && dtype != FGB_F64) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "prox: F32 or F64");
  FGB_CUDA(ctx, cudaSetDevice(ctx->device));
  ProxWork w;
  void* supp = nullptr;
  int* status = nullptr;
  const size_t es = dtype_size(dtype);
  fgb_status s = dmalloc(ctx, (void**)&status, sizeof(int));
  if (s == FGB_OK) s = cuda_check(ctx, cudaMemsetAsync(status, 0, sizeof(int), ctx->stream), "memset");
  if (s == FGB_OK && cons->kind == FGB_SUPP) {
    if (!cons->supp) s = fail(ctx, FGB_ERR_INVALID_ARG, "prox_supp: missing support");
    if (s == FGB_OK) s = dmalloc(ctx, &supp, es * (size_t)cons->rows * cons->cols);
    if (s == FGB_OK)
      s = cuda_check(ctx, cudaMemcpy(supp, cons->supp, es * (size_t)cons->rows * cons->cols, cudaMemcpyHostToDevice),
                     "copy support");
  }
  if (s == FGB_OK) {
    if (dtype == FGB_F64)
      s = launch_prox<double>(ctx, w, *cons, (double*)M, cons->rows, cons->cols, (const double*)supp, status);
    else
      s = launch_prox<float>(ctx, w, *cons, (float*)M, cons->rows, cons->cols, (const float*)supp, status);
  }
  int st = 0;
  if (s == FGB_OK) {
    cudaError_t e = cudaMemcpyAsync(&st, status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    s = cuda_check(ctx, e, "prox");
  }
  prox_work_free(w);
  dfree(supp);
  dfree(status);
  if (s != FGB_OK) return s;
  if (st == FGB_ERR_ZERO_NORM) return fail(ctx, FGB_ERR_ZERO_NORM, "the norm is zero, can't normalize.");
  if (st) return fail(ctx, (fgb_status)st, "prox: device status %d", st);
  return FGB_OK;
}

fgb_status fgb_palm4msa2_device(fgb_ctx* ctx, fgb_dtype dtype, const void* A_dev, int rows, int cols, int nfacts,
                                const fgb_constraint* cons, const fgb_palm_params* params,
                                const void* const* init_facts, double* lambda, fgb_faust** out) {
  if (!ctx || !A_dev || !params) return FGB_ERR_INVALID_ARG;
  if (dtype == FGB_F64)
    return palm_entry<double>(ctx, dtype, A_dev, rows, cols, nfacts, cons, params, init_facts, lambda, out);
  if (dtype == FGB_F32)
    return palm_entry<float>(ctx, dtype, A_dev, rows, cols, nfacts, cons, params, init_facts, lambda, out);
  return fail(ctx, FGB_ERR_NOT_SUPPORTED, "palm4msa2: F32 or F64");
}

fgb_status fgb_palm4msa2(fgb_ctx* ctx, fgb_dtype dtype, const void* A, int rows, int cols, int nfacts,
                         const fgb_constraint* cons, const fgb_palm_params* params, const void* const* init_facts,
                         double* lambda, fgb_faust** out) {
  if (!ctx || !A || !params) return FGB_ERR_INVALID_ARG;
  if (rows <= 0 || cols <= 0) return fail(ctx, FGB_ERR_INVALID_ARG, "palm4msa2: empty A");
  FGB_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t bytes = dtype_size(dtype) * (size_t)rows * cols;
  void* dA = nullptr;
  FGB_TRY(dmalloc(ctx, &dA, bytes));
  fgb_status s = cuda_check(ctx, cudaMemcpyAsync(dA, A, bytes, cudaMemcpyHostToDevice, ctx->stream), "copy A");
  if (s == FGB_OK) s = fgb_palm4msa2_device(ctx, dtype, dA, rows, cols, nfacts, cons, params, init_facts, lambda, out);
  cudaStreamSynchronize(ctx->stream);
  dfree(dA);
  return s;
}

fgb_status fgb_rel_err(fgb_faust* F, const void* A_dev, double lambda, double* out) {
  if (!F || !A_dev || !out) return FGB_ERR_INVALID_ARG;
  fgb_ctx* ctx = F->ctx;
  if (F->dtype != FGB_F64 && F->dtype != FGB_F32) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "rel_err: F32/F64");
  FGB_CUDA(ctx, cudaSetDevice(ctx->device));
  const int rows = F->f.front().rows, cols = F->f.back().cols;
  const int J = (int)F->f.size();
  const size_t es = dtype_size(F->dtype);
  int maxdim = 0;
  for (auto& f : F->f) maxdim = std::max(maxdim, std::max(f.rows, f.cols));
  void *b0 = nullptr, *b1 = nullptr, *lam = nullptr, *res = nullptr, *part = nullptr;
  const long N = (long)rows * cols;
  const int nch = (int)((N + CR_CHUNK - 1) / CR_CHUNK);
  fgb_status s = dmalloc(ctx, &b0, es * (size_t)maxdim * cols);
  if (s == FGB_OK) s = dmalloc(ctx, &b1, es * (size_t)maxdim * cols);
  if (s == FGB_OK) s = dmalloc(ctx, &lam, 8);
  if (s == FGB_OK) s = dmalloc(ctx, &res, 8);
  if (s == FGB_OK) s = dmalloc(ctx, &part, 16 * (size_t)(nch + 1));
  if (s == FGB_OK) {
    // full product, right to left, then the canonical norms
    if (F->dtype == FGB_F64) {
      s = launch_csr_to_dense<double>(ctx, F->f[J - 1], (double*)b0);
      void* cur = b0;
      void* nxt = b1;
      for (int l = J - 2; s == FGB_OK && l >= 0; --l) {
        const DevFactor& f = F->f[l];
        s = launch_csr_spmm<double>(ctx, f.rowptr, f.colind, (const double*)f.val, f.rows, f.cols,
                                    (const double*)cur, f.cols, cols, (double*)nxt, f.rows, Epi<double>());
        std::swap(cur, nxt);
      }
      if (s == FGB_OK) {
        k_set_scalar<double><<<1, 1, 0, ctx->stream>>>((double*)lam, lambda);
        k_chunk_relerr<double><<<nch, 256, 0, ctx->stream>>>((const double*)A_dev, (const double*)cur, N,
                                                             (const double*)lam, (double*)part);
        k_relerr_final<double><<<1, 1, 0, ctx->stream>>>((const double*)part, nch, (double*)res);
        ctx->launches.fetch_add(3);
      }
    } else {
      s = launch_csr_to_dense<float>(ctx, F->f[J - 1], (float*)b0);
      void* cur = b0;
      void* nxt = b1;
      for (int l = J - 2; s == FGB_OK && l >= 0; --l) {
        const DevFactor& f = F->f[l];
        s = launch_csr_spmm<float>(ctx, f.rowptr, f.colind, (const float*)f.val, f.rows, f.cols, (const float*)cur,
                                   f.cols, cols, (float*)nxt, f.rows, Epi<float>());
        std::swap(cur, nxt);
      }
      if (s == FGB_OK) {
        k_set_scalar<float><<<1, 1, 0, ctx->stream>>>((float*)lam, lambda);
        k_chunk_relerr<float><<<nch, 256, 0, ctx->stream>>>((const float*)A_dev, (const float*)cur, N,
                                                            (const float*)lam, (double*)part);
        k_relerr_final<float><<<1, 1, 0, ctx->stream>>>((const double*)part, nch, (double*)res);
        ctx->launches.fetch_add(3);
      }
    }
  }
  if (s == FGB_OK) {
    cudaError_t e = cudaMemcpyAsync(out, res, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    s = cuda_check(ctx, e, "rel_err");
  }
  dfree(b0);
  dfree(b1);
  dfree(lam);
  dfree(res);
  dfree(part);
  return s;
}

}  // extern "C"

extern "C" fgb_status fgb_hierarchical(fgb_ctx* ctx, fgb_dtype dtype, const void* A, int rows, int cols, int nsteps,
                                       const fgb_constraint* fac_cons, const fgb_constraint* res_cons,
                                       const fgb_palm_params* params_2facts, const fgb_palm_params* params_global,
                                       int is_fact_side_left, double* lambda, fgb_faust** out) {
  if (!ctx || !A || !params_2facts || !params_global) return FGB_ERR_INVALID_ARG;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, FGB_ERR_CUDA, "cudaSetDevice");
  if (dtype == FGB_F64)
    return hier_impl<double>(ctx, dtype, A, rows, cols, nsteps, fac_cons, res_cons, params_2facts, params_global,
                             is_fact_side_left, lambda, out);
  if (dtype == FGB_F32)
    return hier_impl<float>(ctx, dtype, A, rows, cols, nsteps, fac_cons, res_cons, params_2facts, params_global,
                            is_fact_side_left, lambda, out);
  return fail(ctx, FGB_ERR_NOT_SUPPORTED, "hierarchical: F32 or F64");
}
