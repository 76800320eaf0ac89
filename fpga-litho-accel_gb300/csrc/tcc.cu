// TCC assembly (litho.cpp:428-516).
#include "litho_internal.cuh"

extern "C" int litho_calc_tcc(litho_ctx* ctx, const float* src, int srcSize, float outerSigma, float wavelength,
                              float NA, float defocus, int Lx, int Ly, int Nx, int Ny, double* tcc, int tccPrecision,
                              int mem) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  litho::set_error(ctx, LITHO_ERR_UNSUPPORTED, "not built");
  return LITHO_ERR_UNSUPPORTED;
}
