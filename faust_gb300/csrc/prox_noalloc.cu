// prox_noalloc.cu — fgb_prox_noalloc: the projection entry point for callers
// that cannot allocate device memory.
//
// Some programs call into this library from places where cudaMalloc is not
// allowed: host applications that reserve all of a GPU's memory up front and
// hand out nothing else (a serving process with a fixed memory budget, an
// embedder whose own pool owns the device), and latency-critical loops that
// must never reach the driver's allocator, whose cudaMalloc / cudaFree can
// synchronise the whole device.  For them the scratch memory of the
// projection (selection state, per-entry flags, reduction partials, row
// counts, the tie-replay heap) comes from one file-scope device array of
// fixed size instead of cudaMalloc.  Every GPU that loads this library holds
// that array until the process exits.
#include <atomic>
#include <cstring>

#include "prox.cuh"

namespace fgb {

// Limits of the no-allocation entry point.
constexpr long NOALLOC_MAX_ENTRIES = 4L << 20;  // rows * cols
constexpr int NOALLOC_MAX_LINES = 65536;        // rows + cols
constexpr long NOALLOC_MAX_HEAP = 65536;        // k of prox_sp's tie replay
constexpr size_t NOALLOC_BYTES = 6u << 20;      // 6 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

namespace {
constexpr int MAX_DEVICES = 64;
// Device address of g_noalloc_scratch on each device, looked up by the first
// call on that device.  Two threads may look it up at once; both store the
// same address.
std::atomic<unsigned char*> g_scratch_ptr[MAX_DEVICES];

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Makes `dev` current for the lifetime of the guard and gives the caller's
// current device back on every return path.
struct DeviceGuard {
  int prev = -1;
  bool ok = false;
  cudaError_t err = cudaSuccess;
  explicit DeviceGuard(int dev) {
    err = cudaGetDevice(&prev);
    if (err == cudaSuccess && prev != dev) err = cudaSetDevice(dev);
    ok = err == cudaSuccess;
  }
  ~DeviceGuard() {
    int cur = -1;
    if (ok && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

fgb_status prox_noalloc_on_device(fgb_ctx* ctx, fgb_dtype dtype, const fgb_constraint* cons, void* M,
                                  const void* supp_dev) {
  const long N = (long)cons->rows * cons->cols;
  // One-time set-up per device, with that device current: the host-side
  // name of the array is not a device address; ask the runtime for it.
  unsigned char* base = g_scratch_ptr[ctx->device].load(std::memory_order_acquire);
  if (!base) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return cuda_check(ctx, e == cudaSuccess ? cudaErrorInvalidSymbol : e,
                                                  "cudaGetSymbolAddress(scratch)");
    base = static_cast<unsigned char*>(p);
    g_scratch_ptr[ctx->device].store(base, std::memory_order_release);
  }
  // carve the scratch
  ProxWork w;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    unsigned char* q = base + off;
    off += align256(bytes);
    return q;
  };
  w.state = reinterpret_cast<TopkState*>(take(sizeof(TopkState)));
  w.hist = reinterpret_cast<unsigned*>(take(sizeof(unsigned) * 2048));
  w.flags = take((size_t)N);
  const long nchunks = (N + 8191) / 8192 + 2;
  w.chunk_cnt = reinterpret_cast<long long*>(take(sizeof(long long) * 2 * nchunks));
  w.partials = reinterpret_cast<double*>(take(sizeof(double) * (N / CR_CHUNK + 2)));
  w.scal = reinterpret_cast<double*>(take(sizeof(double) * 4));
  const int lines = cons->rows + cons->cols + 2;
  w.row_cnt = reinterpret_cast<int*>(take(sizeof(int) * lines));
  int* status = reinterpret_cast<int*>(take(sizeof(int)));
  const size_t heap_bytes = sizeof(long long) * 2 * (size_t)NOALLOC_MAX_HEAP;
  w.heap = take(heap_bytes);
  w.heap_cap = NOALLOC_MAX_HEAP;
  if (off > NOALLOC_BYTES) return fail(ctx, FGB_ERR_INVALID_ARG, "prox_noalloc: scratch layout exceeds the array");
  w.cap_elems = N;
  w.cap_rows = lines;
  // the kernels expect zeroed flags, histogram and status (the array keeps
  // whatever the previous call left)
  FGB_CUDA(ctx, cudaMemsetAsync(w.flags, 0, (size_t)N, ctx->stream));
  FGB_CUDA(ctx, cudaMemsetAsync(w.hist, 0, sizeof(unsigned) * 2048, ctx->stream));
  FGB_CUDA(ctx, cudaMemsetAsync(status, 0, sizeof(int), ctx->stream));
  fgb_status s;
  if (dtype == FGB_F64)
    s = launch_prox<double>(ctx, w, *cons, (double*)M, cons->rows, cons->cols, (const double*)supp_dev, status);
  else
    s = launch_prox<float>(ctx, w, *cons, (float*)M, cons->rows, cons->cols, (const float*)supp_dev, status);
  if (s != FGB_OK) return s;
  // The device status word is read back and the stream synchronised, so
  // the call returns only once the projection has finished.
  int st = 0;
  FGB_CUDA(ctx, cudaMemcpyAsync(&st, status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  FGB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (st == FGB_ERR_ZERO_NORM) return fail(ctx, FGB_ERR_ZERO_NORM, "the norm is zero, can't normalize.");
  if (st) return fail(ctx, (fgb_status)st, "prox_noalloc: device status %d", st);
  return FGB_OK;
}
}  // namespace

}  // namespace fgb

using namespace fgb;

extern "C" fgb_status fgb_prox_noalloc(fgb_ctx* ctx, fgb_dtype dtype, const fgb_constraint* cons, void* M,
                                       const void* supp_dev) {
  if (!ctx || !cons || !M) return FGB_ERR_INVALID_ARG;
  if (dtype != FGB_F32 && dtype != FGB_F64) return fail(ctx, FGB_ERR_NOT_SUPPORTED, "prox_noalloc: F32 or F64");
  const long N = (long)cons->rows * cons->cols;
  if (cons->rows <= 0 || cons->cols <= 0) return fail(ctx, FGB_ERR_INVALID_ARG, "prox_noalloc: empty matrix");
  if (N > NOALLOC_MAX_ENTRIES || (long)cons->rows + cons->cols > NOALLOC_MAX_LINES)
    return fail(ctx, FGB_ERR_INVALID_ARG,
                "prox_noalloc: %d x %d exceeds the fixed scratch (at most %ld entries and %d rows + columns)",
                cons->rows, cons->cols, NOALLOC_MAX_ENTRIES, NOALLOC_MAX_LINES);
  if ((cons->kind == FGB_SP || cons->kind == FGB_SP_POS) && cons->k > NOALLOC_MAX_HEAP && cons->k < N)
    return fail(ctx, FGB_ERR_INVALID_ARG, "prox_noalloc: sp with k = %lld exceeds the fixed scratch (k <= %ld)",
                cons->k, NOALLOC_MAX_HEAP);
  if (cons->kind == FGB_SUPP && !supp_dev)
    return fail(ctx, FGB_ERR_INVALID_ARG, "prox_noalloc: SUPP needs the support in device memory");
  if (ctx->device < 0 || ctx->device >= MAX_DEVICES) return fail(ctx, FGB_ERR_INVALID_ARG, "prox_noalloc: device id");
  DeviceGuard guard(ctx->device);
  if (!guard.ok) return cuda_check(ctx, guard.err, "cudaSetDevice");
  return prox_noalloc_on_device(ctx, dtype, cons, M, supp_dev);
}
