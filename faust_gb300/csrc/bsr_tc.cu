// bsr_tc.cu — BSR x dense on the 5th-generation tensor cores (tcgen05, TMEM
// accumulators, TMA-fed shared memory), BF16 operands, FP32 accumulation.
//
// BSRMat::mul (faust_MatBSR.hpp:827-836): Y(block row r) = sum over the
// stored blocks (r, c) of B_rc X(block row c).  The kernel computes Y^T tiles:
// for a tile of 128 columns j of X and one block row r,
//    D[j, y] = sum_blocks sum_c X[64*bc + c, j] * B[y, c]      (M=128, N=64)
// so the MMA's A operand is a 128 x 64 slab of X (its columns are contiguous
// in the column-major X: K-major, loaded by TMA with 128-byte swizzle) and the
// B operand is one 64 x 64 block stored row by row on the device (K-major,
// also TMA-loaded).  Each block contributes four K=16 MMAs; the 128 x 64 FP32
// accumulator lives in TMEM (four buffers rotate so the epilogue of one item
// overlaps the MMAs of the next).
//
// Warp roles (192 threads): warp 0 issues TMA loads, warp 1 issues MMAs (one
// lane), warps 2-5 drain TMEM (tcgen05.ld), convert to BF16 and store Y.
// Persistent grid (one CTA per SM); work items (column tile, block row) are
// ordered column tile major so the CTAs in flight share the same X columns
// in L2.  Every mbarrier wait is bounded: on expiry the CTA records an error,
// stops issuing, waits (bounded) for its own copies, frees TMEM and returns.
#include <cuda.h>

#include <algorithm>
#include <cstring>

#include "tc_common.cuh"

namespace fgb {

namespace tc {

constexpr int BLK = 64;         // BSR block size
constexpr int TM = 128;         // columns of X per MMA (M)
constexpr int A_BYTES = TM * BLK * 2;   // 16 KB
constexpr int B_BYTES = BLK * BLK * 2;  // 8 KB
constexpr int TMEM_COLS = 256;
constexpr int THREADS = 192;

// NS slabs of 128 columns of X per item share each block's load (NS = 2:
// 40 KB per stage instead of 2 x 24 KB for the same work, the L2-to-SM stream
// that bounds the kernel); the accumulators of an item take NS x 64 TMEM
// columns.
template <int NS>
struct Cfg {
  static constexpr int STAGES = NS == 2 ? 5 : 8;
  static constexpr int STAGE_BYTES = NS * A_BYTES + B_BYTES;
  static constexpr int ACC_BUFS = TMEM_COLS / (NS * BLK);
  static constexpr int ITEM_COLS = NS * TM;
};

struct Shared {
  uint64_t full[8];
  uint64_t empty[8];
  uint64_t acc_full[4];
  uint64_t acc_empty[4];
  uint32_t tmem_base;
  int abort_flag;
};

template <int NS>
__global__ void __launch_bounds__(THREADS, 1)
    k_bsr_tc(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmB,
             const int* __restrict__ browptr, const int* __restrict__ bcolind, int nbr, int nnzb, int stage_idx,
             int mtiles, __nv_bfloat16* __restrict__ Y, long ldy, int* __restrict__ err) {
  constexpr int STAGES = Cfg<NS>::STAGES, STAGE_BYTES = Cfg<NS>::STAGE_BYTES, ACC_BUFS = Cfg<NS>::ACC_BUFS;
  constexpr int ITEM_COLS = Cfg<NS>::ITEM_COLS;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // stage buffers start at a 1024-byte boundary (128-byte swizzle atoms)
  unsigned char* base = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  Shared* sh = reinterpret_cast<Shared*>(base + STAGES * STAGE_BYTES);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const long items = (long)mtiles * nbr;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&sh->full[s], 1);
      mbar_init(&sh->empty[s], 1);
    }
    for (int a = 0; a < ACC_BUFS; ++a) {
      mbar_init(&sh->acc_full[a], 1);
      mbar_init(&sh->acc_empty[a], 4);
    }
    sh->abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&sh->tmem_base)),
                 "r"((uint32_t)TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  // The block structure (row pointers, block columns) is read by every role
  // for every item: kept in shared memory when it fits, so no role waits on
  // a global load between items.
  const int* rp = browptr;
  const int* cix = bcolind;
  if (stage_idx) {
    int* s_rp = reinterpret_cast<int*>(base + STAGES * STAGE_BYTES + ((sizeof(Shared) + 15) & ~(size_t)15));
    int* s_ci = s_rp + ((nbr + 1 + 3) & ~3);
    for (int i = threadIdx.x; i <= nbr; i += THREADS) s_rp[i] = browptr[i];
    for (int i = threadIdx.x; i < nnzb; i += THREADS) s_ci[i] = bcolind[i];
    rp = s_rp;
    cix = s_ci;
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = sh->tmem_base;
  volatile int* abort_flag = &sh->abort_flag;

  if (warp == 0) {
    // ---------------------------------------------------------------- producer
    // The whole warp walks the items; the block indices of an item are read
    // with one coalesced load (32 per round) and lane 0 issues the TMA loads.
    int s = 0;
    uint32_t ph = 0;
    bool waited_ok = true;
    int pend[STAGES];  // parity of the last load issued into each stage, or -1
    for (int u = 0; u < STAGES; ++u) pend[u] = -1;
    for (long it = blockIdx.x; it < items && waited_ok; it += gridDim.x) {
      const int mt = (int)(it / nbr), br = (int)(it % nbr);
      const int p0 = rp[br], p1 = rp[br + 1];
      for (int pb = p0; pb < p1 && waited_ok; pb += 32) {
        const int mine = (pb + lane < p1) ? cix[pb + lane] : 0;
        const int nb = min(32, p1 - pb);
        for (int q = 0; q < nb; ++q) {
          const int bc = __shfl_sync(0xffffffffu, mine, q);
          bool ok = true;
          if (lane == 0) ok = mbar_wait(&sh->empty[s], ph ^ 1u, abort_flag);
          ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
          if (!ok) {
            waited_ok = false;
            break;
          }
          if (lane == 0) {
            unsigned char* st = base + s * STAGE_BYTES;
            mbar_expect_tx(&sh->full[s], STAGE_BYTES);
#pragma unroll
            for (int h = 0; h < NS; ++h) tma_load_2d(st + h * A_BYTES, &tmX, bc * BLK, mt * ITEM_COLS + h * TM, &sh->full[s]);
            tma_load_2d(st + NS * A_BYTES, &tmB, 0, (pb + q) * BLK, &sh->full[s]);
          }
          pend[s] = (int)ph;
          if (++s == STAGES) {
            s = 0;
            ph ^= 1u;
          }
        }
      }
    }
    if (lane == 0) {
      if (!waited_ok) {
        atomicExch(err, 1);
        *abort_flag = 1;
      }
      // on an abort, the copies this warp issued must land before the shared
      // memory is released (bounded waits)
      if (*abort_flag)
        for (int u = 0; u < STAGES; ++u)
          if (pend[u] >= 0)
            for (unsigned i = 0; i < WAIT_LIMIT && !mbar_try_wait(&sh->full[u], (uint32_t)pend[u]); ++i) {
            }
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---------------------------------------------------------------- MMA issuer
    if (lane == 0) {
      int s = 0, a = 0;
      uint32_t ph = 0, aph = 0;
      bool ok = true;
      for (long it = blockIdx.x; it < items && ok; it += gridDim.x) {
        const int br = (int)(it % nbr);
        const int p0 = rp[br], p1 = rp[br + 1];
        if (p1 == p0) continue;  // empty block row: the epilogue writes zeros
        if (!mbar_wait(&sh->acc_empty[a], aph ^ 1u, abort_flag)) {
          ok = false;
          break;
        }
        fence_after();
        const uint32_t d = tmem + (uint32_t)(a * NS * BLK);
        for (int p = p0; p < p1; ++p) {
          if (!mbar_wait(&sh->full[s], ph, abort_flag)) {
            ok = false;
            break;
          }
          fence_after();
          const uint32_t sa = su32(base + s * STAGE_BYTES), sb = sa + NS * A_BYTES;
          const uint64_t bd = sdesc_k128(sb);
#pragma unroll
          for (int h = 0; h < NS; ++h) {
            const uint64_t ad = sdesc_k128(sa + h * A_BYTES);
#pragma unroll
            for (int k = 0; k < BLK / 16; ++k)
              mma_bf16(d + (uint32_t)(h * BLK), ad + (uint64_t)((k * 32) >> 4), bd + (uint64_t)((k * 32) >> 4),
                       idesc_bf16(TM, BLK), (p > p0 || k > 0) ? 1u : 0u);
          }
          mma_commit(&sh->empty[s]);
          if (++s == STAGES) {
            s = 0;
            ph ^= 1u;
          }
        }
        if (!ok) break;
        mma_commit(&sh->acc_full[a]);
        if (++a == ACC_BUFS) {
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
    // ---------------------------------------------------------------- epilogue
    const int q = warp & 3;  // TMEM lane quadrant this warp may access
    int a = 0;
    uint32_t aph = 0;
    bool ok = true;
    for (long it = blockIdx.x; it < items && ok; it += gridDim.x) {
      const int mt = (int)(it / nbr), br = (int)(it % nbr);
      const int p0 = rp[br], p1 = rp[br + 1];
      if (p1 == p0) {
        const uint4 z = make_uint4(0, 0, 0, 0);
#pragma unroll
        for (int h = 0; h < NS; ++h) {
          const long j = (long)mt * ITEM_COLS + h * TM + q * 32 + lane;
          uint4* dst = reinterpret_cast<uint4*>(Y + j * ldy + (long)br * BLK);
#pragma unroll
          for (int u = 0; u < 8; ++u) dst[u] = z;
        }
        continue;
      }
      bool got = true;
      if (lane == 0) got = mbar_wait(&sh->acc_full[a], aph, abort_flag);
      got = __shfl_sync(0xffffffffu, got ? 1 : 0, 0) != 0;
      if (!got) {
        ok = false;
        break;
      }
      fence_after();
      uint32_t r[32];
      uint32_t packed[NS][32];
#pragma unroll
      for (int h = 0; h < NS; ++h) {
        const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(a * NS * BLK + h * BLK);
        tmem_ld32(taddr, r);
        tmem_ld_wait();
#pragma unroll
        for (int u = 0; u < 16; ++u) packed[h][u] = pack_bf16(r[2 * u], r[2 * u + 1]);
        tmem_ld32(taddr + 32, r);
        tmem_ld_wait();
#pragma unroll
        for (int u = 0; u < 16; ++u) packed[h][16 + u] = pack_bf16(r[2 * u], r[2 * u + 1]);
      }
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&sh->acc_empty[a]);
#pragma unroll
      for (int h = 0; h < NS; ++h) {
        const long j = (long)mt * ITEM_COLS + h * TM + q * 32 + lane;
        uint4* dst = reinterpret_cast<uint4*>(Y + j * ldy + (long)br * BLK);
#pragma unroll
        for (int u = 0; u < 8; ++u)
          dst[u] = make_uint4(packed[h][4 * u], packed[h][4 * u + 1], packed[h][4 * u + 2], packed[h][4 * u + 3]);
      }
      if (++a == ACC_BUFS) {
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
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)TMEM_COLS));
}

// Re-lays a column-major block (the ABI's storage) out row by row, the
// K-major operand layout of the kernel.
__global__ void k_blocks_rowmajor(const __nv_bfloat16* __restrict__ in, __nv_bfloat16* __restrict__ out, long nblk) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nblk * BLK * BLK; e += (long)gridDim.x * blockDim.x) {
    const long p = e / (BLK * BLK);
    const int w = (int)(e % (BLK * BLK));
    const int r = w / BLK, c = w % BLK;
    out[e] = in[p * BLK * BLK + (long)c * BLK + r];
  }
}

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
    cudaGetLastError();
  }
  return fn;
}

bool make_map_bf16(CUtensorMap* m, const void* base, uint64_t inner, uint64_t outer, uint64_t row_bytes,
                   uint32_t box_inner, uint32_t box_outer) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {inner, outer};
  cuuint64_t strides[1] = {row_bytes};
  cuuint32_t box[2] = {box_inner, box_outer};
  cuuint32_t es[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace tc

// Row-major copy of a factor's blocks (the kernel's K-major operand), built
// when the factor is uploaded.
fgb_status bsr_tc_prepare(fgb_ctx* ctx, DevFactor& f) {
  if (f.format != FGB_BSR || f.bm != tc::BLK || f.bn != tc::BLK || f.nnz == 0) return FGB_OK;
  FGB_TRY(dmalloc(ctx, &f.aux, (size_t)f.nnz * tc::BLK * tc::BLK * 2));
  tc::k_blocks_rowmajor<<<2 * ctx->sm_count, 256, 0, ctx->stream>>>((const __nv_bfloat16*)f.val,
                                                                   (__nv_bfloat16*)f.aux, (long)f.nnz);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

fgb_status launch_bsr_tc(fgb_ctx* ctx, const DevFactor& f, const __nv_bfloat16* X, int ldx, int ncols,
                         __nv_bfloat16* Y, int ldy, bool* taken) {
  *taken = false;
  if (getenv("FGB_BSR_SIMT")) return FGB_OK;
  // shapes the kernel takes: 64 x 64 blocks, whole 128-column tiles,
  // 16-byte aligned rows and bases
  if (f.bm != 64 || f.bn != 64 || f.nnz == 0) return FGB_OK;
  if (ncols % tc::TM || ldx % 8 || ldy % 8) return FGB_OK;
  if (((uintptr_t)X & 15) || ((uintptr_t)Y & 15)) return FGB_OK;
  // two 128-column slabs per item when the columns come in pairs of tiles
  const bool two = ncols % (2 * tc::TM) == 0;
  const int nbr = f.rows / tc::BLK, mtiles = ncols / (two ? 2 * tc::TM : tc::TM);
  const size_t stage_bytes = two ? (size_t)tc::Cfg<2>::STAGES * tc::Cfg<2>::STAGE_BYTES
                                 : (size_t)tc::Cfg<1>::STAGES * tc::Cfg<1>::STAGE_BYTES;
  const size_t base_smem = stage_bytes + ((sizeof(tc::Shared) + 15) & ~(size_t)15) + 1024;
  if (base_smem > ctx->smem_optin) return FGB_OK;
  const size_t idx_bytes = sizeof(int) * ((size_t)((nbr + 1 + 3) & ~3) + (size_t)f.nnz);
  const bool stage_idx = base_smem + idx_bytes <= ctx->smem_optin;
  const size_t smem = base_smem + (stage_idx ? idx_bytes : 0);
  const __nv_bfloat16* blocks = (const __nv_bfloat16*)f.aux;
  if (!blocks) return FGB_OK;
  CUtensorMap mx, mb;
  if (!tc::make_map_bf16(&mx, X, (uint64_t)f.cols, (uint64_t)ncols, (uint64_t)ldx * 2, tc::BLK, tc::TM)) return FGB_OK;
  if (!tc::make_map_bf16(&mb, blocks, (uint64_t)tc::BLK, (uint64_t)f.nnz * tc::BLK, tc::BLK * 2, tc::BLK, tc::BLK))
    return FGB_OK;
  int* err = nullptr;
  FGB_TRY(kernel_err_word(ctx, &err));
  auto kern = two ? tc::k_bsr_tc<2> : tc::k_bsr_tc<1>;
  FGB_TRY(smem_opt_in(ctx, (const void*)kern, smem));
  const long items = (long)nbr * mtiles;
  const int grid = (int)std::min<long>(items, ctx->sm_count);
  kern<<<grid, tc::THREADS, smem, ctx->stream>>>(mx, mb, f.rowptr, f.colind, nbr, f.nnz, stage_idx ? 1 : 0, mtiles,
                                                 Y, (long)ldy, err);
  FGB_LAUNCHED(ctx);
  *taken = true;
  return FGB_OK;
}

}  // namespace fgb
