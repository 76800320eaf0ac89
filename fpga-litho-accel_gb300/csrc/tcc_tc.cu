// Split-BF16 tensor-core TCC contraction (tcgen05).
#include "litho_internal.cuh"

namespace litho {

int tcc_split_bf16(litho_ctx* ctx, const float2* P, const float* J, int n, int ns, int ldp, double2* tcc) {
  set_error(ctx, LITHO_ERR_UNSUPPORTED, "split-BF16 TCC not built");
  return LITHO_ERR_UNSUPPORTED;
}

}  // namespace litho
