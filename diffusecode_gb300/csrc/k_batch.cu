// Batched population (placeholder).
#include "dgpu_internal.h"

extern "C" int dgpu_batch_run(dgpu_ctx *ctx, int32_t, const dgpu_crystal *, const dgpu_grid *,
                              const dgpu_opts *, double *const *, const double *const *,
                              const double *const *, double *, double *const *, double *const *)
{
    return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "batch not built");
}

extern "C" double dgpu_batch_last_ms(const dgpu_ctx *ctx) { return ctx ? ctx->batch_ms : 0.0; }
