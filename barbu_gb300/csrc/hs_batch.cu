// hs_batch.cu -- batched update of many grooms (placeholder until the
// batched path lands).
#include "hs_api_internal.h"

namespace hs {

struct BatchState {};

void destroy_ctx_extensions(hs_ctx* ctx) {
  delete ctx->batch;
  ctx->batch = nullptr;
}

}  // namespace hs
