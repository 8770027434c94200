/* fgb_diag.h — device rate probe used as a roofline denominator.  No
 * counterpart in the reference.  Same conventions as fgb.h. */
#ifndef FGB_DIAG_H
#define FGB_DIAG_H

#include "fgb.h"

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* Scalar FP64 fused multiply-add throughput of the whole device (the pipe
 * the CSR products and power iterations of FP64 palm4msa2 run on): a
 * dependent-FMA loop on every SM, eight independent chains per thread,
 * timed with CUDA events on the context's stream.  *flops = 2 * FMAs / s. */
fgb_status fgb_probe_fp64_fma(fgb_ctx* ctx, double* flops);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif
