// gemm_tc.cu — BF16 GEMM on tcgen05 for the warm-start MLP:
//     C[M x N] = A[M x K] * B[N x K]^T   (+ bias[n], ReLU)
// A and B row-major (K contiguous, i.e. both K-major), FP32 accumulation in
// TMEM, output BF16 or FP32 row-major.  128 x 128 tiles, K in steps of 64
// through a 6-stage TMA ring (128-byte swizzle); warp 0 loads, one lane of
// warp 1 issues the MMAs, warps 2-5 drain TMEM.  With split_k > 1 each CTA
// takes a K range of a tile and adds its FP32 partial into C with atomics
// (C must start at zero; the bias/activation pass runs afterwards).  Waits
// are bounded like the BSR kernel's.
#include <algorithm>

#include "tc_common.cuh"

namespace fgb {
namespace tc {

constexpr int GM = 128, GN = 128, GK = 64;
constexpr int G_STAGES = 6;
constexpr int G_A = GM * GK * 2, G_B = GN * GK * 2, G_STAGE = G_A + G_B;
constexpr int G_ACC = 2;
constexpr int G_TMEM = G_ACC * GN;  // 256 columns
constexpr int G_THREADS = 192;

struct GShared {
  uint64_t full[G_STAGES];
  uint64_t empty[G_STAGES];
  uint64_t acc_full[G_ACC];
  uint64_t acc_empty[G_ACC];
  uint32_t tmem_base;
  int abort_flag;
};

enum { ACT_NONE = 0, ACT_RELU = 1 };

__device__ __forceinline__ uint32_t f2bf2(float lo, float hi) {
  const __nv_bfloat162 x = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&x);
}

__global__ void __launch_bounds__(G_THREADS, 1)
    k_gemm_tn(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int M, int N, int K,
              int split_k, void* __restrict__ C, long ldc, int c_f32, const float* __restrict__ bias, int act,
              int atomic_out, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  GShared* sh = reinterpret_cast<GShared*>(base + G_STAGES * G_STAGE);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int mt = M / GM, nt = N / GN, ksteps = K / GK;
  const long items = (long)mt * nt * split_k;
  const int kper = (ksteps + split_k - 1) / split_k;

  if (threadIdx.x == 0) {
    for (int s = 0; s < G_STAGES; ++s) {
      mbar_init(&sh->full[s], 1);
      mbar_init(&sh->empty[s], 1);
    }
    for (int a = 0; a < G_ACC; ++a) {
      mbar_init(&sh->acc_full[a], 1);
      mbar_init(&sh->acc_empty[a], 4);
    }
    sh->abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&sh->tmem_base)),
                 "r"((uint32_t)G_TMEM));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = sh->tmem_base;
  volatile int* abort_flag = &sh->abort_flag;
  // item -> (tile n, tile m, k range): consecutive items share the B tile
  auto decode = [&](long it, int& tm, int& tn, int& k0, int& k1) {
    const int ks = (int)(it % split_k);
    const long t = it / split_k;
    tm = (int)(t % mt);
    tn = (int)(t / mt);
    k0 = ks * kper;
    k1 = min(ksteps, k0 + kper);
  };

  if (warp == 0) {
    if (lane == 0) {
      int s = 0;
      uint32_t ph = 0;
      bool ok = true;
      int pend[G_STAGES];
      for (int u = 0; u < G_STAGES; ++u) pend[u] = -1;
      for (long it = blockIdx.x; it < items && ok; it += gridDim.x) {
        int tm, tn, k0, k1;
        decode(it, tm, tn, k0, k1);
        for (int kk = k0; kk < k1; ++kk) {
          if (!mbar_wait(&sh->empty[s], ph ^ 1u, abort_flag)) {
            ok = false;
            break;
          }
          unsigned char* st = base + s * G_STAGE;
          mbar_expect_tx(&sh->full[s], G_STAGE);
          tma_load_2d(st, &tmA, kk * GK, tm * GM, &sh->full[s]);
          tma_load_2d(st + G_A, &tmB, kk * GK, tn * GN, &sh->full[s]);
          pend[s] = (int)ph;
          if (++s == G_STAGES) {
            s = 0;
            ph ^= 1u;
          }
        }
      }
      if (!ok) {
        atomicExch(err, 1);
        *abort_flag = 1;
      }
      if (*abort_flag)
        for (int u = 0; u < G_STAGES; ++u)
          if (pend[u] >= 0)
            for (unsigned i = 0; i < WAIT_LIMIT && !mbar_try_wait(&sh->full[u], (uint32_t)pend[u]); ++i) {
            }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int s = 0, a = 0;
      uint32_t ph = 0, aph = 0;
      bool ok = true;
      const uint32_t idesc = idesc_bf16(GM, GN);
      for (long it = blockIdx.x; it < items && ok; it += gridDim.x) {
        int tm, tn, k0, k1;
        decode(it, tm, tn, k0, k1);
        if (k1 <= k0) continue;
        if (!mbar_wait(&sh->acc_empty[a], aph ^ 1u, abort_flag)) {
          ok = false;
          break;
        }
        fence_after();
        const uint32_t d = tmem + (uint32_t)(a * GN);
        for (int kk = k0; kk < k1; ++kk) {
          if (!mbar_wait(&sh->full[s], ph, abort_flag)) {
            ok = false;
            break;
          }
          fence_after();
          const uint32_t sa = su32(base + s * G_STAGE), sb = sa + G_A;
          const uint64_t ad = sdesc_k128(sa), bd = sdesc_k128(sb);
#pragma unroll
          for (int k = 0; k < GK / 16; ++k)
            mma_bf16(d, ad + (uint64_t)((k * 32) >> 4), bd + (uint64_t)((k * 32) >> 4), idesc,
                     (kk > k0 || k > 0) ? 1u : 0u);
          mma_commit(&sh->empty[s]);
          if (++s == G_STAGES) {
            s = 0;
            ph ^= 1u;
          }
        }
        if (!ok) break;
        mma_commit(&sh->acc_full[a]);
        if (++a == G_ACC) {
          a = 0;
          aph ^= 1u;
        }
      }
      if (!ok) {
        atomicExch(err, 1);
        *abort_flag = 1;
      }
    }
  } else {
    const int q = warp & 3;
    int a = 0;
    uint32_t aph = 0;
    bool ok = true;
    for (long it = blockIdx.x; it < items && ok; it += gridDim.x) {
      int tm, tn, k0, k1;
      decode(it, tm, tn, k0, k1);
      if (k1 <= k0) continue;
      bool got = true;
      if (lane == 0) got = mbar_wait(&sh->acc_full[a], aph, abort_flag);
      got = __shfl_sync(0xffffffffu, got ? 1 : 0, 0) != 0;
      if (!got) {
        ok = false;
        break;
      }
      fence_after();
      const long row = (long)tm * GM + q * 32 + lane;
      const int n0 = tn * GN;
      const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(a * GN);
#pragma unroll 1
      for (int c = 0; c < GN / 32; ++c) {
        uint32_t r[32];
        tmem_ld32(taddr + c * 32, r);
        tmem_ld_wait();
        float v[32];
#pragma unroll
        for (int u = 0; u < 32; ++u) v[u] = __uint_as_float(r[u]);
        const int nb = n0 + c * 32;
        if (atomic_out) {
          float* dst = reinterpret_cast<float*>(C) + row * ldc + nb;
#pragma unroll
          for (int u = 0; u < 32; ++u) atomicAdd(dst + u, v[u]);
        } else {
          if (bias) {
#pragma unroll
            for (int u = 0; u < 32; ++u) v[u] += bias[nb + u];
          }
          if (act == ACT_RELU) {
#pragma unroll
            for (int u = 0; u < 32; ++u) v[u] = fmaxf(v[u], 0.f);
          }
          if (c_f32) {
            float4* dst = reinterpret_cast<float4*>(reinterpret_cast<float*>(C) + row * ldc + nb);
#pragma unroll
            for (int u = 0; u < 8; ++u) dst[u] = make_float4(v[4 * u], v[4 * u + 1], v[4 * u + 2], v[4 * u + 3]);
          } else {
            uint4* dst = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(C) + row * ldc + nb);
#pragma unroll
            for (int u = 0; u < 4; ++u)
              dst[u] = make_uint4(f2bf2(v[8 * u], v[8 * u + 1]), f2bf2(v[8 * u + 2], v[8 * u + 3]),
                                  f2bf2(v[8 * u + 4], v[8 * u + 5]), f2bf2(v[8 * u + 6], v[8 * u + 7]));
          }
        }
      }
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&sh->acc_empty[a]);
      if (++a == G_ACC) {
        a = 0;
        aph ^= 1u;
      }
    }
    if (!ok && lane == 0) {
      atomicExch(err, 1);
      *abort_flag = 1;
    }
  }
  fence_before();
  __syncthreads();
  fence_after();
  __syncwarp();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)G_TMEM));
}

// bias + activation + conversion pass over an FP32 split-K result.
__global__ void k_bias_act(const float* __restrict__ in, long ldi, int M, int N, const float* __restrict__ bias,
                           int act, void* __restrict__ out, long ldo, int out_f32) {
  const long n = (long)M * N;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const long r = e / N, c = e % N;
    float v = in[r * ldi + c];
    if (bias) v += bias[c];
    if (act == ACT_RELU) v = fmaxf(v, 0.f);
    if (out_f32) reinterpret_cast<float*>(out)[r * ldo + c] = v;
    else reinterpret_cast<__nv_bfloat16*>(out)[r * ldo + c] = __float2bfloat16(v);
  }
}

}  // namespace tc

fgb_status launch_gemm_bf16(fgb_ctx* ctx, int M, int N, int K, const void* A, long lda, const void* B, long ldb,
                            void* C, long ldc, int c_f32, const float* bias, int act, int split_k, float* work) {
  using namespace tc;
  if (M <= 0 || N <= 0 || K <= 0 || M % GM || N % GN || K % GK)
    return fail(ctx, FGB_ERR_NOT_SUPPORTED, "gemm: M, N multiples of 128 and K a multiple of 64 (got %d %d %d)", M,
                N, K);
  if (lda % 8 || ldb % 8 || ((uintptr_t)A & 15) || ((uintptr_t)B & 15) || ((uintptr_t)C & 15) ||
      (c_f32 ? ldc % 4 : ldc % 8))
    return fail(ctx, FGB_ERR_NOT_SUPPORTED, "gemm: 16-byte aligned rows and bases required");
  CUtensorMap ma, mb;
  if (!make_map_bf16(&ma, A, (uint64_t)K, (uint64_t)M, (uint64_t)lda * 2, GK, GM) ||
      !make_map_bf16(&mb, B, (uint64_t)K, (uint64_t)N, (uint64_t)ldb * 2, GK, GN))
    return fail(ctx, FGB_ERR_CUDA, "gemm: tensor map creation failed");
  int* err = nullptr;
  FGB_TRY(kernel_err_word(ctx, &err));
  const size_t smem = G_STAGES * G_STAGE + sizeof(GShared) + 1024;
  FGB_TRY(smem_opt_in(ctx, (const void*)k_gemm_tn, smem));
  const int ksteps = K / GK;
  split_k = std::max(1, std::min(split_k, ksteps));
  const long tiles = (long)(M / GM) * (N / GN);
  const long items = tiles * split_k;
  const int grid = (int)std::min<long>(items, ctx->sm_count);
  if (split_k == 1) {
    k_gemm_tn<<<grid, G_THREADS, smem, ctx->stream>>>(ma, mb, M, N, K, 1, C, ldc, c_f32, bias, act, 0, err);
    FGB_LAUNCHED(ctx);
    return FGB_OK;
  }
  // split K: FP32 partial sums added into a zeroed buffer, then bias/act
  float* acc = (c_f32 && !bias && act == ACT_NONE) ? (float*)C : work;
  const long lda_acc = (acc == (float*)C) ? ldc : N;
  if (!acc) return fail(ctx, FGB_ERR_INVALID_ARG, "gemm: split_k > 1 needs an FP32 workspace of M*N");
  if (acc == (float*)C) {
    for (int r = 0; r < 1; ++r) FGB_CUDA(ctx, cudaMemset2DAsync(C, ldc * 4, 0, (size_t)N * 4, M, ctx->stream));
  } else {
    FGB_CUDA(ctx, cudaMemsetAsync(acc, 0, (size_t)M * N * 4, ctx->stream));
  }
  k_gemm_tn<<<grid, G_THREADS, smem, ctx->stream>>>(ma, mb, M, N, K, split_k, acc, lda_acc, 1, nullptr, ACT_NONE, 1,
                                                     err);
  FGB_LAUNCHED(ctx);
  if (acc != (float*)C) {
    k_bias_act<<<4 * ctx->sm_count, 256, 0, ctx->stream>>>(acc, N, M, N, bias, act, C, ldc, c_f32);
    FGB_LAUNCHED(ctx);
  }
  return FGB_OK;
}

}  // namespace fgb
