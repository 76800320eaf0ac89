// SOCS kernel extraction (litho.cpp:579-645).
#include "litho_internal.cuh"

extern "C" int litho_calc_kernels(litho_ctx* ctx, const double* tcc, int tccSize, int nk, float* krn_r, float* krn_i,
                                  float* scales, double* krn64, double* scales64, int mem) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  litho::set_error(ctx, LITHO_ERR_UNSUPPORTED, "not built");
  return LITHO_ERR_UNSUPPORTED;
}
