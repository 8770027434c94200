// palm.cu — palm4msa2 driver (in progress).
#include "fgb_internal.cuh"

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
fgb_status fgb_prox(fgb_ctx* ctx, fgb_dtype, const fgb_constraint*, void*) {
  return fail(ctx, FGB_ERR_NOT_SUPPORTED, "not built yet");
}
fgb_status fgb_palm4msa2(fgb_ctx* ctx, fgb_dtype, const void*, int, int, int, const fgb_constraint*,
                         const fgb_palm_params*, const void* const*, double*, fgb_faust**) {
  return fail(ctx, FGB_ERR_NOT_SUPPORTED, "not built yet");
}
fgb_status fgb_palm4msa2_device(fgb_ctx* ctx, fgb_dtype, const void*, int, int, int, const fgb_constraint*,
                                const fgb_palm_params*, const void* const*, double*, fgb_faust**) {
  return fail(ctx, FGB_ERR_NOT_SUPPORTED, "not built yet");
}
fgb_status fgb_rel_err(fgb_faust* F, const void*, double, double*) {
  return fail(F ? F->ctx : nullptr, FGB_ERR_NOT_SUPPORTED, "not built yet");
}
}
