// Mixed-precision (tensor-core) window DFT and interpolation.
#include "litho_internal.cuh"

namespace litho {

bool tc_supported(const ImgGeom& g) { return false; }

int run_win_dft_tc(litho_ctx* ctx, const ImgPlan& p, const float* masks, float2* win_part) {
  set_error(ctx, LITHO_ERR_UNSUPPORTED, "tensor-core window DFT not built");
  return LITHO_ERR_UNSUPPORTED;
}

int run_fi_tc(litho_ctx* ctx, const ImgPlan& p, const float2* band_part, float* tm, float* images) {
  set_error(ctx, LITHO_ERR_UNSUPPORTED, "tensor-core interpolation not built");
  return LITHO_ERR_UNSUPPORTED;
}

}  // namespace litho
