/* fgb.h — C ABI of faust_gb300: FAuST's Faust x dense product and palm4msa2
 * factor update on one GB300 (sm_103a).
 *
 * This ABI plays the role that libgm.so (the gpu_mod backend) plays for the
 * reference: FAuST's GPU2 layer dlopen()s a C library and calls plain
 * functions on opaque handles (src/faust_linear_operator/GPU2/
 * faust_gpu_mod_utils.h:24-97, faust_gpu_mod_utils.cpp:26-92).  Each entry
 * point below names the reference interface it replaces.
 *
 * Conventions
 *  - Dense matrices are column-major with a leading dimension (Eigen default,
 *    src/faust_linear_operator/CPU/faust_MatDense.h:142).
 *  - CSR factors: int32 rowptr (rows+1), int32 colind sorted inside each row,
 *    values (src/faust_linear_operator/CPU/faust_MatSparse.h:456-462).
 *  - BSR factors: int32 browptr (rows/bm+1), int32 bcolind, blocks of bm x bn
 *    stored column-major one after another (faust_MatBSR.h:122-145).
 *  - Every call returns an fgb_status; no C++ exception crosses the ABI.  The
 *    message of the last failure of a context is fgb_last_error(ctx).  The
 *    reference raises std::logic_error / std::runtime_error /
 *    std::domain_error for the same conditions (faust_exception.h:64-67).
 *  - Calls on one context are not thread-safe; use one context per host thread
 *    (as GPUModHandler, faust_gpu_mod_utils.cpp:26-92).
 *  - Work is queued on the context's stream; *_host entry points and the
 *    PALM drivers synchronise before returning.
 */
#ifndef FGB_H
#define FGB_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Exported even when the library is compiled with -fvisibility=hidden. */
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

typedef enum fgb_status {
  FGB_OK = 0,
  FGB_ERR_INVALID_ARG = 1,
  FGB_ERR_OOM = 2,
  FGB_ERR_CUDA = 3,
  FGB_ERR_NAN = 4,       /* NaN in a norm or in lambda (faust_palm4msa2020.hpp:593-597,482-490) */
  FGB_ERR_ZERO_NORM = 5, /* zero norm (faust_palm4msa2020.hpp:598-610, faust_MatDense.hpp:1246-1249) */
  FGB_ERR_CANCELLED = 6, /* fgb_cancel() was called (the reference's SIGINT flag, faust_palm4msa2020.cpp:9-28) */
  FGB_ERR_TIMEOUT = 7,   /* a bounded device-side wait ran out */
  FGB_ERR_NOT_SUPPORTED = 8
} fgb_status;

typedef enum fgb_dtype { FGB_F32 = 0, FGB_F64 = 1, FGB_BF16 = 2 } fgb_dtype;

typedef enum fgb_format { FGB_CSR = 0, FGB_BSR = 1 } fgb_format;

typedef struct fgb_ctx fgb_ctx;
typedef struct fgb_faust fgb_faust;

/* ------------------------------------------------------------------ context
 * Replaces gp_funcs->set_dev / set_stream (faust_gpu_mod_utils.h:100-102).
 * All work of the context is ordered on cuda_stream (a cudaStream_t; NULL is
 * the legacy default stream): kernels the context runs beside it (the
 * long-row part of a sparse product, the PALM power iterations) go to the
 * context's own streams, forked from cuda_stream by an event and joined back
 * before the next work queued on it, so the caller sees one stream (and a
 * capture of cuda_stream captures them too). */
fgb_status fgb_ctx_create(int device, void* cuda_stream, fgb_ctx** out);
fgb_status fgb_ctx_destroy(fgb_ctx* ctx);
const char* fgb_last_error(const fgb_ctx* ctx);
/* Waits for the context's stream.  Returns FGB_ERR_TIMEOUT (and clears the
 * record) when a kernel of the context gave up a bounded device-side wait
 * since the last call (the tensor-core BSR and GEMM kernels, the radix
 * butterfly kernel); the outputs of that launch are then undefined. */
fgb_status fgb_ctx_synchronize(fgb_ctx* ctx);
/* Asks a running palm4msa2 call of this context to stop at the next outer
 * iteration (the reference's palm4msa2 SIGINT flag,
 * faust_palm4msa2020.hpp:239-242).  Safe to call from another thread. */
fgb_status fgb_cancel(fgb_ctx* ctx);
/* Number of kernels this context launched since creation (diagnostics). */
long long fgb_ctx_kernel_launches(const fgb_ctx* ctx);

/* ------------------------------------------------------------------ Faust */
typedef struct fgb_factor_desc {
  int format;         /* fgb_format */
  int rows, cols;
  int nnz;            /* CSR: nonzeros; BSR: nonzero blocks */
  int bm, bn;         /* BSR block size (ignored for CSR) */
  const int* rowptr;  /* CSR rowptr[rows+1] / BSR browptr[rows/bm+1] */
  const int* colind;  /* CSR colind[nnz] / BSR bcolind[nnz] */
  const void* values; /* CSR values[nnz] / BSR blocks[nnz*bm*bn] */
} fgb_factor_desc;

/* Builds a device-resident Faust from factors held in HOST memory (copied).
 * Replaces TransformHelper<FPP,GPU2>(const TransformHelper<FPP,Cpu>&) /
 * MatSparse<FPP,GPU2>(const MatSparse<FPP,Cpu>&) -> spm_funcs->togpu
 * (src/faust_linear_operator/GPU2/faust_MatSparse_gpu.cpp.in). */
fgb_status fgb_faust_create(fgb_ctx* ctx, fgb_dtype dtype, int nfactors, const fgb_factor_desc* factors,
                            fgb_faust** out);
fgb_status fgb_faust_destroy(fgb_faust* F);
fgb_status fgb_faust_shape(const fgb_faust* F, int* rows, int* cols, int* nfactors);

/* Y = F X with X, Y in DEVICE memory (column-major), queued on the context
 * stream.  Factors are applied right to left as Transform<FPP,GPU2>::multiply
 * (faust_Transform_gpu.hpp:505-522) / Transform<FPP,Cpu>::multiply
 * (CPU/faust_Transform.hpp:1814-1855); replaces spm_funcs->mul_gpu_dsm_ext
 * (faust_MatSparse_gpu.cpp.in:462-471) and bsr_funcs->mul_gpu_dsm_ext
 * (faust_MatBSR_gpu.cpp.in:108-140).  X and Y must not overlap.  BF16 Fausts
 * take BF16 X and produce BF16 Y with FP32 accumulation.
 * mode: 0 = automatic, 1 = one launch per factor, 2 = fused chain (fails
 * with FGB_ERR_NOT_SUPPORTED when the chain does not fit on chip), 3 = the
 * butterfly chain kernel (fails unless every factor has a butterfly support:
 * entries r & ~h, r | h in row r, faust_butterfly.hpp:459-492).  Automatic
 * mode takes the butterfly kernel for butterfly chains with enough columns. */
fgb_status fgb_faust_mul(fgb_faust* F, const void* X, int ldx, int ncols, void* Y, int ldy, int mode);

// Y = op(F) X with op 'N' (as fgb_faust_mul), 'T' or 'H' (the adjoint; the
// transpose for real scalars): F^T X = S_J^T (... (S_1^T X)), X of
// rows(F) x ncols (ld >= rows(F)), Y of cols(F) x ncols.  CSR Fausts only;
// the factors' transposes are built on first use.  Replaces
// Transform<FPP,Cpu>::multiply(const MatDense&, char opThis)
// (CPU/faust_Transform.hpp:1754-1773, the 'T' / 'H' branches).
fgb_status fgb_faust_mul_op(fgb_faust* F, char op, const void* X, int ldx, int ncols, void* Y, int ldy, int mode);

/* Product orders: the values of FaustMulMode (CPU/faust_prod_opt.h:12-60)
 * that the device path runs. */
enum { FGB_ORDER_DEFAULT_L2R = 0, FGB_ORDER_DYNPROG = 5 };

/* Y = op(F) as a dense column-major matrix on the device (ldy >= its rows),
 * TransformHelper<FPP,Cpu>::get_product(mul_order_opt_mode)
 * (CPU/faust_TransformHelper.hpp:1132-1178):
 *   FGB_ORDER_DEFAULT_L2R  Transform::get_product (CPU/faust_Transform.hpp:598-656)
 *   FGB_ORDER_DYNPROG      dynprog_multiply (faust_prod_opt_gen.hpp:80-202)
 * op 'N', 'T' or 'H' ('H' = 'T' for real scalars).  CSR Fausts only. */
fgb_status fgb_faust_product(fgb_faust* F, char op, int order, void* Y, int ldy);

/* Y = op(F) X in the DYNPROG order, X dense (device, column-major) as the
 * last operand of the chain: TransformHelper::multiply(const MatDense&) with
 * mul_order_opt_mode == DYNPROG (CPU/faust_TransformHelper.hpp:373-379). */
fgb_status fgb_faust_mul_dynprog(fgb_faust* F, char op, const void* X, int ldx, int ncols, void* Y, int ldy);

/* Host-only: the DYNPROG split table for a chain of n leaves (stored rows,
 * cols, nonzeros, is_dense per leaf; op 'N' or 'T').  split[i*n + j] = k
 * for i < j means the product of leaves i..j is (i..k)(k+1..j); other cells
 * are -1.  The cost model is the reference's (CPU/faust_prod_opt.cpp:1-80,
 * faust_prod_opt_gen.hpp:113-190) in 32-bit two's complement arithmetic. */
fgb_status fgb_dynprog_plan(int n, const int* rows, const int* cols, const int* nnz, const int* is_dense, char op,
                            int* split);

/* Y = F X with X, Y in HOST memory: copy in, product, copy out, synchronous.
 * Operands of 32 MB or more go in up to four column chunks whose copies
 * (on two extra streams) overlap the products of their neighbours; with
 * pinned host buffers the copy engines then run beside the kernels.
 * Replaces TransformHelper<FPP,Cpu>::multiply(const FPP* A, int A_ncols,
 * FPP* C) (CPU/faust_TransformHelper.hpp:406-433) and
 * TransformHelper<FPP,GPU2>::multiply(const MatDense<FPP,Cpu>&)
 * (GPU2/faust_TransformHelper_gpu.hpp:439-444). */
fgb_status fgb_faust_mul_host(fgb_faust* F, const void* X, int ncols, void* Y);

/* 2-norm by power iteration in FP64, TransformHelper::spectralNorm
 * (CPU/faust_TransformHelper.hpp:1200-1218, CPU/faust_Transform.hpp:683-708,
 * faust_linear_algebra.hpp:806-899).  flag = iterations, or -1 when max_iter
 * was reached.  CSR Fausts only. */
fgb_status fgb_faust_spectral_norm(fgb_faust* F, int max_iter, double threshold, double* norm, int* flag);

/* Factor i copied to host: dense column-major (rows*cols values) or CSR
 * arrays (rowptr[rows+1], colind[nnz], values[nnz]; query nnz first). */
fgb_status fgb_faust_factor_info(const fgb_faust* F, int i, int* format, int* rows, int* cols, int* nnz);
fgb_status fgb_faust_factor_to_dense(fgb_faust* F, int i, void* host_dense);
fgb_status fgb_faust_factor_to_csr(fgb_faust* F, int i, int* host_rowptr, int* host_colind, void* host_values);
/* BSR factor i copied to host as stored: browptr[rows/bm + 1], bcolind[nblocks]
 * and nblocks column-major bm x bn blocks (MatBSR's layout, faust_MatBSR.h:41-145;
 * read back by the .mat writer, MatBSR::toMatIOVar, faust_MatBSR.hpp:387-470). */
fgb_status fgb_faust_factor_to_bsr(fgb_faust* F, int i, int* host_browptr, int* host_bcolind, void* host_blocks);

/* ------------------------------------------------------------------ projections
 * Constraint kinds: ConstraintName (faust_ConstraintGeneric.h:49-70). */
typedef enum fgb_cons_kind {
  FGB_SP = 0,       /* prox_sp        faust_prox.hpp:71-96   */
  FGB_SPCOL = 1,    /* prox_spcol     faust_prox.hpp:112-143 */
  FGB_SPLIN = 2,    /* prox_splin     faust_prox.hpp:145-177 */
  FGB_SPLINCOL = 3, /* prox_splincol  faust_prox.hpp:179-202 */
  FGB_NORMCOL = 4,  /* prox_normcol   faust_prox.hpp:204-246 */
  FGB_NORMLIN = 5,  /* prox_normlin   faust_prox.hpp:248-254 */
  FGB_SUPP = 6,     /* prox_supp      faust_prox.hpp:375-385 */
  FGB_SP_POS = 7    /* prox_sp with pos=true */
} fgb_cons_kind;

typedef struct fgb_constraint {
  int kind;           /* fgb_cons_kind */
  int rows, cols;     /* shape of the constrained factor */
  long long k;        /* sparsity level (SP, SPCOL, SPLIN, SPLINCOL, SP_POS) */
  double s;           /* norm value (NORMCOL, NORMLIN) */
  int normalized;     /* ConstraintGeneric normalizing flag */
  int pos;            /* ConstraintGeneric pos flag */
  const void* supp;   /* SUPP: rows*cols column-major support (HOST memory), same dtype */
} fgb_constraint;

/* In-place projection of the dense DEVICE matrix M (rows x cols,
 * column-major, ld = rows), ConstraintGeneric::project
 * (faust_ConstraintGeneric.hpp:229-246).  Replaces dsm_funcs->prox_sp /
 * prox_spcol / prox_splin (faust_MatDense_gpu.cpp.in:746-763) and the CPU
 * round trips of GPU2/faust_prox_gpu.hpp:102-149.  Supports are chosen as
 * std::partial_sort with comparator |a| > |b| chooses them
 * (faust_prox.hpp:52-69), ties included.  F32 and F64. */
fgb_status fgb_prox(fgb_ctx* ctx, fgb_dtype dtype, const fgb_constraint* cons, void* M);

/* Same projection as fgb_prox, for callers that cannot allocate device
 * memory: host applications that reserve all of a GPU's memory up front
 * (a fixed serving budget, an embedder whose pool owns the device) and
 * latency-critical loops that must not reach cudaMalloc / cudaFree, which
 * can synchronise the device.  No cudaMalloc/cudaFree or allocating library
 * call is made.  This entry point has no counterpart in the reference.  The
 * caller's current device is restored before returning.  Its scratch memory is one
 * fixed 6 MiB device array inside the library (every GPU that loads the
 * library holds it until the process exits), which limits it to
 * rows*cols <= 4194304, rows+cols <= 65536 and, for FGB_SP / FGB_SP_POS,
 * k <= 65536 (larger sizes return FGB_ERR_INVALID_ARG).  M is a DEVICE
 * matrix as in fgb_prox; for FGB_SUPP the support must be given in DEVICE
 * memory through supp_dev (cons->supp is ignored).  The first call on a
 * device looks up the array's device address: make that first call before
 * any stream capture.  All calls share the array, so calls that overlap on
 * the GPU (several streams or threads at once) race; the entry point
 * clears what must start at zero and synchronises the context's stream
 * before returning. */
fgb_status fgb_prox_noalloc(fgb_ctx* ctx, fgb_dtype dtype, const fgb_constraint* cons, void* M,
                            const void* supp_dev);

/* ------------------------------------------------------------------ PALM4MSA */
typedef struct fgb_palm_params {
  int nb_it;                 /* StoppingCriterion num_its (faust_StoppingCriterion.hpp:112-154) */
  int is_update_way_R2L;     /* default 0 */
  int packing_RL;            /* default 1 */
  int no_normalization;      /* default 0 */
  int no_lambda;             /* default 0 */
  double norm2_threshold;    /* default 1e-6 */
  int norm2_max_iter;        /* default 100 */
  int constant_step_size;    /* default 0 */
  double step_size;          /* default 1e-16 (pyfaust ParamsPalm4MSA) */
  int no_lambda_error;       /* the reference's NO_LAMBDA_ERROR environment switch */
  int norm2_fp64;            /* F32 runs: spectral norms in FP64 */
} fgb_palm_params;

fgb_status fgb_palm_params_default(fgb_palm_params* p);

/* palm4msa2 (src/algorithm/factorization/faust_palm4msa2020.h:45-72,
 * .hpp:46-301) with factors_format = AllDynamic and no MHTP, on the GPU.
 * A: rows x cols column-major in HOST memory.  init_facts: NULL (zero/eye
 * initialisation of :115-149) or an array of nfacts host pointers to dense
 * column-major factors.  lambda: in = initial lambda, out = final lambda.
 * out: the resulting Faust (device resident), to be released with
 * fgb_faust_destroy.  F32 and F64. */
fgb_status fgb_palm4msa2(fgb_ctx* ctx, fgb_dtype dtype, const void* A, int rows, int cols, int nfacts,
                         const fgb_constraint* cons, const fgb_palm_params* params, const void* const* init_facts,
                         double* lambda, fgb_faust** out);

/* Same with A already in DEVICE memory (column-major, ld = rows). */
fgb_status fgb_palm4msa2_device(fgb_ctx* ctx, fgb_dtype dtype, const void* A_dev, int rows, int cols, int nfacts,
                                const fgb_constraint* cons, const fgb_palm_params* params,
                                const void* const* init_facts, double* lambda, fgb_faust** out);

/* hierarchical (2020) factorization: Faust::hierarchical
 * (src/algorithm/factorization/faust_hierarchical.hpp:1-121, .h:6-24).
 * Step i = 0..nsteps-1 splits the current residual (the last factor, or the
 * first when is_fact_side_left) by palm4msa2 with constraints
 * (fac_cons[i], res_cons[i]) -- (res_cons[i], fac_cons[i]) on the left side --
 * and params_2facts (zero / identity start, lambda 1); the global lambda is
 * multiplied by that lambda; then palm4msa2 with params_global refines all
 * factors against A from the current factors and the global lambda.  A: rows
 * x cols column-major in HOST memory.  The result has nsteps + 1 factors;
 * lambda receives the final global lambda.  F32 and F64. */
fgb_status fgb_hierarchical(fgb_ctx* ctx, fgb_dtype dtype, const void* A, int rows, int cols, int nsteps,
                            const fgb_constraint* fac_cons, const fgb_constraint* res_cons,
                            const fgb_palm_params* params_2facts, const fgb_palm_params* params_global,
                            int is_fact_side_left, double* lambda, fgb_faust** out);

/* ------------------------------------------------------------------ batched PALM4MSA
 * Many independent palm4msa2 instances (uneven sizes) in ONE persistent
 * launch: each CTA takes the next instance from a device work queue and runs
 * its whole loop.  No reference counterpart exists as one call: it replaces
 * a host loop of palm4msa2 calls (src/FaustFact.hpp:579-673 per instance).
 * Supported constraints: SPCOL, SPLIN, SPLINCOL (k <= 64), NORMCOL, NORMLIN,
 * SUPP; at most 16 factors.  Every instance is bit-identical to a
 * single-instance run with the same parameters. */
typedef struct fgb_palm_problem {
  int rows, cols;                  /* shape of A */
  const void* A;                   /* DEVICE, column-major, ld = rows */
  int nfacts;
  const fgb_constraint* cons;      /* host array (SUPP supports in host memory) */
  const void* const* init_facts;   /* NULL or nfacts host dense factors */
  double init_lambda;
} fgb_palm_problem;

typedef struct fgb_palm_result {
  fgb_faust* faust;  /* release with fgb_faust_destroy */
  double lambda;
  int status;        /* fgb_status of this instance */
  long long cycles;  /* batched runs: SM clock cycles its CTA spent on the instance */
} fgb_palm_result;

typedef struct fgb_batch_opts {
  int ctas_per_sm;   /* resident instances per SM (0 = the tuned table's choice, else 2) */
  /* Seeding from values already on the device (the learned warm start):
   * when init_values is set, every instance has the same nfacts and the same
   * SUPP constraints (same shapes and support pointers); instance i starts
   * from factors whose entries on the supports are
   * init_values_scale * init_values[i * values_per_instance + q], q running
   * over the support entries factor by factor in row-major (CSR) order, and
   * problems[i].init_facts is ignored.  DEVICE memory, dtype of the run. */
  const void* init_values;
  int values_per_instance;
  double init_values_scale;
  /* 1: each instance starts from lambda = <A, S>_F / ||S||_F^2 with S the
   * product of its initial factors (in place of problems[i].init_lambda);
   * the same formula and summation order as update_lambda's. */
  int lambda_from_init;
} fgb_batch_opts;

fgb_status fgb_palm4msa2_batched(fgb_ctx* ctx, fgb_dtype dtype, int nprob, const fgb_palm_problem* problems,
                                 const fgb_palm_params* params, const fgb_batch_opts* opts,
                                 fgb_palm_result* results);

/* calc_rel_err (faust_palm4msa2020.hpp:35-44): ||lambda F - A||_F / ||A||_F
 * with A in DEVICE memory. */
fgb_status fgb_rel_err(fgb_faust* F, const void* A_dev, double lambda, double* out);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif

#endif /* FGB_H */
