// TCC-direct aerial image (litho.cpp:522-566 calcImage + 358-408 FT_c2r_padded).
//
//   imgf[ny2][nx2] = sum_{ny1,nx1} mskf[ny2+ny1][nx2+nx1] conj(mskf[ny1][nx1])
//                    * tcc[(ny1,nx1)][(ny2+ny1, nx2+nx1)]
// for |ny2| <= 2Ny, 0 <= nx2 <= 2Nx (indices relative to the spectrum centre,
// terms with |ny2+ny1| > Ny or |nx2+nx1| > Nx skipped), accumulated in FP64 as
// the reference does.  FT_c2r_padded completes nx2 < 0 by Hermitian symmetry;
// that completion is exactly the interpolation band used by the SOCS path
// (band[fy][d] = imgf[fy][d] for d >= 0, conj(imgf[-fy][-d]) for d < 0), so the
// image is produced by the same fi_prep/fi_out kernels.
#include "litho_internal.cuh"

#include <vector>

namespace litho {

__global__ void calc_image_band_kernel(const float* __restrict__ mr, const float* __restrict__ mi, int Fx, int Fy,
                                       const double2* __restrict__ tcc, int n, int Nx, int Ny,
                                       float2* __restrict__ band) {
  const int BW = 4 * Nx + 1;
  const int fy = blockIdx.x;               // 0..2Ny
  const int d = (int)threadIdx.x - 2 * Nx;  // -2Nx..2Nx
  if (fy > 2 * Ny || threadIdx.x >= (unsigned)BW) return;
  // imgf at (ny2, nx2) with nx2 >= 0; conjugate mirror for d < 0
  const bool neg = d < 0;
  const int ny2 = neg ? -fy : fy, nx2 = neg ? -d : d;
  const int th = (n - 1) / 2, KX = 2 * Nx + 1;
  const int cy = Fy / 2, cx = Fx / 2;
  double re = 0.0, im = 0.0;
  for (int ny1 = -Ny; ny1 <= Ny; ++ny1) {
    if (ny2 + ny1 < -Ny || ny2 + ny1 > Ny) continue;
    for (int nx1 = -Nx; nx1 <= Nx; ++nx1) {
      if (nx2 + nx1 < -Nx || nx2 + nx1 > Nx) continue;
      const size_t ia = (size_t)(ny2 + ny1 + cy) * Fx + (nx2 + nx1 + cx);
      const size_t ib = (size_t)(ny1 + cy) * Fx + (nx1 + cx);
      const double ar = mr[ia], ai = mi[ia], br = mr[ib], bi = mi[ib];
      // a * conj(b)
      const double pr = ar * br + ai * bi, pi = ai * br - ar * bi;
      const double2 t = tcc[(size_t)(ny1 * KX + nx1 + th) * n + ((ny2 + ny1) * KX + (nx2 + nx1) + th)];
      re += pr * t.x - pi * t.y;
      im += pr * t.y + pi * t.x;
    }
  }
  band[fy * BW + d + 2 * Nx] = neg ? make_float2((float)re, (float)-im) : make_float2((float)re, (float)im);
}

}  // namespace litho

using namespace litho;

extern "C" int litho_calc_image(litho_ctx* ctx, const float* mskf_r, const float* mskf_i, int fftLx, int fftLy,
                                const double* tcc, int tccSize, int Nx, int Ny, int physLx, int physLy, float* image,
                                int mem) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  LITHO_ARG_CHECK(ctx, mskf_r && mskf_i && tcc && image, "null pointer");
  LITHO_ARG_CHECK(ctx, Nx >= 0 && Ny >= 0 && Nx <= 16 && Ny <= 16, "Nx, Ny must be in [0, 16]");
  LITHO_ARG_CHECK(ctx, tccSize == (2 * Nx + 1) * (2 * Ny + 1), "tccSize must be (2Nx+1)(2Ny+1)");
  LITHO_ARG_CHECK(ctx, is_pow2(fftLx) && is_pow2(fftLy) && next_pow2(physLx) == fftLx && next_pow2(physLy) == fftLy,
                  "fft size must be nextPow2 of the physical size");
  LITHO_ARG_CHECK(ctx, 2 * Nx + 1 <= fftLx && 2 * Ny + 1 <= fftLy, "window exceeds the spectrum");
  LITHO_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  const size_t spec = (size_t)fftLx * fftLy * sizeof(float);
  const void *dr = nullptr, *di = nullptr, *dt = nullptr;
  LITHO_RET(stage_in(ctx, ctx->stage_in, mskf_r, spec, mem, &dr));
  LITHO_RET(stage_in(ctx, ctx->stage_x, mskf_i, spec, mem, &di));
  LITHO_RET(stage_in(ctx, ctx->tcc_c, tcc, (size_t)tccSize * tccSize * sizeof(double2), mem, &dt));
  ImgGeom g{physLx, physLy, fftLx, fftLy, Nx, Ny, 1, 32};
  ImgPlan p = make_plan(g, 1, ctx->sm_count);
  p.kpg = 1;
  p.ngroups = 1;
  const int BW = 4 * Nx + 1, BH = 2 * Ny + 1;
  LITHO_RET(ctx->band_part.ensure(ctx, (size_t)BH * BW * sizeof(float2)));
  LITHO_RET(ctx->tm.ensure(ctx, (size_t)(4 * Ny + 1) * physLx * sizeof(float)));
  float* dimg = image;
  const size_t img_bytes = (size_t)physLx * physLy * sizeof(float);
  if (mem == LITHO_MEM_HOST) {
    LITHO_RET(ctx->stage_out.ensure(ctx, img_bytes));
    dimg = ctx->stage_out.as<float>();
  }
  {
    StageScope sc(ctx, LITHO_STAGE_SOCS);
    calc_image_band_kernel<<<BH, ((BW + 31) / 32) * 32, 0, ctx->stream>>>(
        static_cast<const float*>(dr), static_cast<const float*>(di), fftLx, fftLy, static_cast<const double2*>(dt),
        tccSize, Nx, Ny, ctx->band_part.as<float2>());
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
  }
  LITHO_RET(run_fi(ctx, p, ctx->band_part.as<float2>(), ctx->tm.as<float>(), dimg));
  if (mem == LITHO_MEM_HOST) {
    LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(image, dimg, img_bytes, cudaMemcpyDeviceToHost, ctx->stream));
    LITHO_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return LITHO_OK;
}
