// Tensor-core engine (placeholder until the tcgen05 kernel lands).
#include "dgpu_internal.h"

bool dgpu_tc_available(dgpu_ctx *ctx) { (void)ctx; return false; }

int dgpu_tc_sums(dgpu_ctx *ctx, const uint64_t *, const uint64_t *, const uint64_t *, const uint64_t *,
                 const float *, const int64_t *, int32_t, const BoxSpec &, const dgpu_opts *, DevBuf &,
                 int32_t *)
{
    return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "tensor-core engine not built");
}
