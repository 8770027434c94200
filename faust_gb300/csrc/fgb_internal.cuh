// fgb_internal.cuh — shared internals of libfaust_gb300 (context, device
// factors, error plumbing, canonical reduction order).
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include <atomic>
#include <memory>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/fgb.h"

// Number of SMs on GB300; grids of the streaming kernels are sized in
// multiples of it (the runtime value is read once per context).
#define FGB_SM_COUNT_HINT 152

// ---------------------------------------------------------------- context
struct fgb_ctx {
  int device = 0;
  int sm_count = FGB_SM_COUNT_HINT;
  size_t smem_optin = 0;  // cudaDevAttrMaxSharedMemoryPerBlockOptin
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  std::atomic<long long> launches{0};
  // Host-mapped cancel flag polled by the PALM driver between iterations.
  volatile int* cancel_host = nullptr;
  int* cancel_dev = nullptr;
  // glibc rand() sequence after srand(418) (power-iteration start vector),
  // cached on the device.
  int* rand_dev = nullptr;
  int rand_n = 0;
  // the power-iteration start vector -1 + 2*rand()/RAND_MAX in FP64 and FP32
  double* x0_d = nullptr;
  float* x0_f = nullptr;
  // Side stream of the long-row product kernels, forked from and joined back
  // to `stream` by the two events around each product (null: run in line).
  cudaStream_t s_long = nullptr;
  cudaEvent_t ev_long_fork = nullptr, ev_long_join = nullptr;
  // Cooperative grid of the projection's radix select on this context's
  // device (FP32, FP64), computed on first use.
  int rs_coop_blocks[2] = {0, 0};
  int rs_coop_blocks_reg[2] = {0, 0};  // the same for the register-resident variant
  // Device word set by kernels whose bounded waits ran out (the tcgen05 BSR
  // and GEMM kernels, the radix butterfly kernel); read and cleared by
  // fgb_ctx_synchronize.
  int* kerr = nullptr;
};

namespace fgb {

// Records a message on the context and returns the status.
fgb_status fail(fgb_ctx* ctx, fgb_status st, const char* fmt, ...);
// Converts a CUDA error into FGB_ERR_CUDA with a message (or OK).
fgb_status cuda_check(fgb_ctx* ctx, cudaError_t e, const char* what);

#define FGB_CUDA(ctx, call)                                      \
  do {                                                           \
    cudaError_t e__ = (call);                                    \
    if (e__ != cudaSuccess) return fgb::cuda_check(ctx, e__, #call); \
  } while (0)

#define FGB_TRY(call)                  \
  do {                                 \
    fgb_status s__ = (call);           \
    if (s__ != FGB_OK) return s__;     \
  } while (0)

// Counts a kernel launch and checks the launch error.
#define FGB_STR2(x) #x
#define FGB_STR(x) FGB_STR2(x)
#define FGB_LAUNCHED(ctx)                                                                  \
  do {                                                                                     \
    (ctx)->launches.fetch_add(1, std::memory_order_relaxed);                               \
    cudaError_t e__ = cudaGetLastError();                                                  \
    if (e__ != cudaSuccess) return fgb::cuda_check(ctx, e__, "kernel launch at " __FILE__ ":" FGB_STR(__LINE__)); \
  } while (0)

size_t dtype_size(fgb_dtype t);

// Device allocation helpers (report OOM as FGB_ERR_OOM).
fgb_status dmalloc(fgb_ctx* ctx, void** p, size_t bytes);
void dfree(void* p);
// The context's kernel error word (allocated and zeroed on first use).
fgb_status kernel_err_word(fgb_ctx* ctx, int** out);
// After a synchronisation of the context's stream: FGB_ERR_TIMEOUT (and the
// word cleared) when a kernel recorded an expired bounded wait.
fgb_status check_kernel_err(fgb_ctx* ctx);
// Raises the kernel's dynamic shared-memory limit on the context's device to
// at least `bytes` (a per device and kernel attribute, only ever raised).
fgb_status smem_opt_in(fgb_ctx* ctx, const void* func, size_t bytes);

// ---------------------------------------------------------------- device factors
// A sparse factor resident on the device.  CSR keeps, beside its own arrays,
// the CSR of its transpose (built on the device) for S^H X and X S products.
struct DevFactor {
  int format = FGB_CSR;
  int rows = 0, cols = 0;
  int nnz = 0;    // CSR nonzeros / BSR blocks
  int cap = 0;    // capacity of colind/val (entries)
  int bm = 0, bn = 0;
  int* rowptr = nullptr;
  int* colind = nullptr;
  void* val = nullptr;
  // Transpose (CSR only): rows = cols of the factor.
  int* t_rowptr = nullptr;
  int* t_colind = nullptr;
  void* t_val = nullptr;
  bool has_t = false;
  // BSR: row-major copy of the blocks for the tensor-core kernel.
  void* aux = nullptr;
  // Butterfly support (stride of the entries r & ~h, r | h in every row),
  // 0 when the factor is not one, -1 until checked on the device.
  int bfly = -1;
  // Longest row / column (entries), -1 when not known on the host.
  int max_row = -1, max_col = -1;
  // The same two figures on the device (written by the dense -> CSR
  // conversion) for factors the host cannot see, e.g. PALM's, or null.
  int* d_maxrc = nullptr;
};

}  // namespace fgb

struct fgb_faust {
  fgb_ctx* ctx = nullptr;
  fgb_dtype dtype = FGB_F64;
  std::vector<fgb::DevFactor> f;
  // Ping-pong buffers for one-launch-per-factor products, grown on demand.
  void* buf[2] = {nullptr, nullptr};
  size_t buf_bytes = 0;
  // Pinned staging buffers for the host-memory entry point.
  void* hx = nullptr;
  void* hy = nullptr;
  size_t hx_bytes = 0, hy_bytes = 0;
  void* dx = nullptr;
  void* dy = nullptr;
  size_t dxy_bytes = 0;
  // Device descriptor arrays for the fused chain kernel (F, and F^T as the
  // chain of transposed factors in reverse order).
  void* chain_desc = nullptr;
  void* chain_desc_t = nullptr;
  // Factor values of the radix butterfly kernel in the order it reads them
  // (for F and for F^T), built on first use.
  void* brv[2] = {nullptr, nullptr};
  // Workspace of the dense product (intermediates and dense images).
  void* pws = nullptr;
  size_t pws_bytes = 0;
  // Copy streams and events of the pipelined host-buffer product.
  cudaStream_t s_in = nullptr, s_out = nullptr;
  cudaEvent_t ev_in[4] = {}, ev_done[4] = {}, ev_start = nullptr;
  // When set, the factor arrays are views into this shared device block
  // (results of one batched call) and are released with its last owner.
  std::shared_ptr<void> pool;
  ~fgb_faust();
};

namespace fgb {

// ---------------------------------------------------------------- canonical order
// Reductions over N values in column-major linear order: 256 lanes per chunk
// of 65536 values, lane t accumulating chunk offsets = t (mod 256) in order,
// a pairwise tree over the lanes, chunk partials added in order.  The oracle
// (oracle/faust_oracle.cpp) restates the same order, so results agree bit for
// bit.
constexpr int CR_LANES = 256;
constexpr long CR_CHUNK = 65536;

__device__ __forceinline__ float fmad(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmad(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float addr(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double addr(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float subr(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double subr(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float mulr(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mulr(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float divr(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double divr(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float sqrtr(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ double sqrtr(double a) { return __dsqrt_rn(a); }

// Pairwise tree over 256 lane partials held in shared memory `lane` (every
// thread of the block calls; blocks of at least 32 threads): level s adds
// lane t + s into lane t for t < s, s = 128, 64, ..., 1.  One warp evaluates
// it -- the three upper levels in registers (lane t of the warp holds the
// partials t, t + 32, t + 64, t + 96 of level 128), the five lower ones by
// shuffles -- with the same additions in the same association as the
// level-by-level form.  lane[0] carries the result to the block.
template <typename T>
__device__ __forceinline__ T lane_tree_256(T* lane) {
  __syncthreads();
  if (threadIdx.x < 32) {
    const int t = threadIdx.x;
    const T a0 = addr(lane[t], lane[t + 128]);
    const T a1 = addr(lane[t + 32], lane[t + 160]);
    const T a2 = addr(lane[t + 64], lane[t + 192]);
    const T a3 = addr(lane[t + 96], lane[t + 224]);
    T c = addr(addr(a0, a2), addr(a1, a3));
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) c = addr(c, __shfl_down_sync(0xffffffffu, c, s));
    if (t == 0) lane[0] = c;
  }
  __syncthreads();
  T r = lane[0];
  __syncthreads();
  return r;
}

// Canonical dot product of a[0..n) and b[0..n) by one block of at least 256
// threads (threads 0..255 hold the lanes); every thread receives the result.
template <typename T>
__device__ T block_cdot(const T* a, const T* b, long n, T* lane) {
  T total = T(0);
  for (long c0 = 0; c0 < n; c0 += CR_CHUNK) {
    long c1 = c0 + CR_CHUNK < n ? c0 + CR_CHUNK : n;
    if (threadIdx.x < CR_LANES) {
      T acc = T(0);
      for (long i = c0 + threadIdx.x; i < c1; i += CR_LANES) acc = fmad(a[i], b[i], acc);
      lane[threadIdx.x] = acc;
    }
    T part = lane_tree_256(lane);
    total = addr(total, part);
  }
  return total;
}

// Kernel helpers defined in the .cu files.
fgb_status csr_build_transpose(fgb_ctx* ctx, fgb_dtype dt, DevFactor& f);
// G_0 ... G_{nfac-1} X for the first nfac factors of op(F)'s product order
// (G_q = S_q, or S_{J-1-q}^T for op T, whose transposes must exist); faust.cu.
fgb_status faust_apply_prefix(fgb_faust* F, char op, int nfac, const void* X, int ldx, int ncols, void* Y, int ldy);
// The same product with the butterfly chain kernel when every factor has a
// butterfly support (bfly.cu); *ran = false when it does not apply.
fgb_status bfly_chain(fgb_faust* F, char op, int nfac, const void* X, int ldx, int ncols, void* Y, int ldy,
                      bool force, bool* ran);

}  // namespace fgb
