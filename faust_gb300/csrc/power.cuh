// power.cuh — device power iteration on chains of CSR factors
// (Faust::power_iteration, faust_linear_algebra.hpp:806-899, driven by
// Transform::spectralNorm, CPU/faust_Transform.hpp:683-708).
#pragma once

#include "fgb_internal.cuh"

namespace fgb {

constexpr int PI_MAX_OPS = 64;
constexpr int PI_THREADS = 512;
constexpr int PI_MAX_CHAINS = 64;

// One sparse product y = S x (or S^H x through the transpose's CSR).
struct PIOp {
  const int* rowptr;
  const int* colind;
  const void* val;
  int rows;  // length of y
  int pad;
};

// The operator F F^H (or F^H F) of one chain, as a list of products applied
// in order to the vector.  empty: no factor (norm 1); a factor without
// entries gives norm 0 (checked on the device), as Transform::spectralNorm.
struct PIChain {
  int nops;
  int n;
  int maxdim;  // longest intermediate vector
  int empty;
  int pad;
  PIOp ops[PI_MAX_OPS];
};

// Step-size epilogue of palm4msa2's update_fact (faust_palm4msa2020.hpp:563-617),
// computed by the last block to finish: c = 1.001*l*l*nR*nR*nL*nL (double
// arithmetic, rounded to FPP), alpha = l / c, and the NaN / zero-norm errors.
struct PIPalm {
  int enabled;
  int it;
  int r2l;
  int constant_step;
  double step_size;
  const void* lambda;  // FPP device scalar
  void* c;             // FPP device scalar
  void* alpha;         // FPP device scalar
  // When set, one of the two norms was computed earlier (a chain of factors
  // that the current sweep has not touched yet): ext_norm points to it and
  // the launch has one block, whose chain gives the other norm.  ext_is_r:
  // the external norm is ||R|| (left-to-right sweep) or ||L|| (right to left).
  const double* ext_norm;
  int ext_is_r;
  int pad;
};

struct PIOut {
  double norm[PI_MAX_CHAINS];
  int flag[PI_MAX_CHAINS];
  int status;        // fgb_status of the first failure (0 = ok)
  unsigned done;     // blocks finished (reset by the last one)
};

// Builds the op list of F[lo..hi) (square or wide: F F^H; tall: F^H F).
// Factors must have their transpose CSR.
void pi_chain_build(const DevFactor* F, int lo, int hi, PIChain& ch);

// Queues the two-chain power iteration kernel (chains with n == 0 are
// skipped) on `stream` (nullptr: the context's stream).  TF: factor value
// type; norms computed in TC.
fgb_status launch_power_iteration(fgb_ctx* ctx, fgb_dtype tf, bool fp64, const PIChain& a, const PIChain& b,
                                  int max_iter, double thr, const int* d_rand, PIOut* d_out, const PIPalm& palm,
                                  cudaStream_t stream = nullptr);

// Norms of nchains chains described in DEVICE memory (one block each, no
// step-size epilogue) into d_out->norm[0..nchains); maxn: the longest vector
// of any chain.
fgb_status launch_power_iteration_many(fgb_ctx* ctx, fgb_dtype tf, bool fp64, const PIChain* d_chains, int nchains,
                                       int maxn, int max_iter, double thr, PIOut* d_out, cudaStream_t stream);

// Raw glibc rand() values after srand(418), length n, in device memory,
// cached per context size.
fgb_status pi_rand_device(fgb_ctx* ctx, int n, const int** d_rand);

// Synchronous 2-norm of F[lo..hi) (for fgb_faust_spectral_norm).
fgb_status chain_spectral_norm_sync(fgb_ctx* ctx, fgb_dtype dt, const DevFactor* F, int lo, int hi, int max_iter,
                                    double thr, double* norm, int* flag);

}  // namespace fgb
