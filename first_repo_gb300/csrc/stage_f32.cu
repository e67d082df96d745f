// FP32 mixed form of the particle step (filled in below the FP64 drop-in).
#include "pstep_internal.cuh"

namespace pstep {
int f32_create(pstep_ctx *h) {
  snprintf(h->err, sizeof h->err, "the FP32 form is not available in this build");
  return PSTEP_ERR_CONFIG;
}
int f32_destroy(pstep_ctx *) { return PSTEP_OK; }
int f32_upload(pstep_ctx *, const double *, const double *, const double *, const double *, const double *,
               const double *, const double *, int) { return PSTEP_ERR_CONFIG; }
int f32_set_tau(pstep_ctx *, const double *, int) { return PSTEP_ERR_CONFIG; }
int f32_bind_fields(pstep_ctx *) { return PSTEP_ERR_CONFIG; }
int f32_prime(pstep_ctx *) { return PSTEP_ERR_CONFIG; }
int f32_stage(pstep_ctx *, int, double, double) { return PSTEP_ERR_CONFIG; }
int f32_end_stage(pstep_ctx *) { return PSTEP_ERR_CONFIG; }
int f32_end_step(pstep_ctx *) { return PSTEP_ERR_CONFIG; }
int f32_get_array(pstep_ctx *, int, void *, int) { return PSTEP_ERR_CONFIG; }
}  // namespace pstep
