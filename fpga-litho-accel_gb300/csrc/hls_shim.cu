// C++-linkage shims with the reference's FPGA top-function signatures
// (include/litho_gb300_hls.hpp), backed by the GPU library.
#include "litho_internal.cuh"
#include "../../include/litho_gb300_hls.hpp"

#include <cmath>
#include <cstdio>
#include <limits>
#include <mutex>
#include <vector>

namespace litho {

// one process-wide context per device, created on first use
static litho_ctx* hls_ctx() {
  static std::mutex mu;
  static litho_ctx* ctxs[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (ctxs[dev] == nullptr && litho_ctx_create(dev, &ctxs[dev]) != LITHO_OK) ctxs[dev] = nullptr;
  return ctxs[dev];
}

static void fill_nan(float* p, size_t n) {
  if (p)
    for (size_t i = 0; i < n; ++i) p[i] = std::numeric_limits<float>::quiet_NaN();
}

}  // namespace litho

using namespace litho;

// socs_2048_stream_refactored_v18_hls_fft.cpp:287-388: 128 x 128 fftshifted
// intensity of nk kernels (before Fourier interpolation) into both outputs.
void calc_socs_2048_hls_stream_refactored_v18(float* mskf_r, float* mskf_i, float* krn_r, float* krn_i,
                                              float* scales, float* tmpImg_ddr, float* output, int nk,
                                              int nx_actual, int ny_actual, int Lx, int Ly) {
  constexpr int N = 128;  // MAX_FFT_X / MAX_FFT_Y of the v18 design
  litho_ctx* ctx = hls_ctx();
  const size_t out_n = (size_t)N * N;
  int rc = LITHO_ERR_CUDA;
  if (ctx != nullptr && mskf_r && mskf_i && krn_r && krn_i && scales && nk >= 1 && nx_actual >= 0 &&
      ny_actual >= 0 && 4 * nx_actual + 1 <= N && 4 * ny_actual + 1 <= N && Lx >= 2 * nx_actual + 1 &&
      Ly >= 2 * ny_actual + 1) {
    rc = [&]() -> int {
      const int kdim = (2 * nx_actual + 1) * (2 * ny_actual + 1);
      const size_t spec = (size_t)Lx * Ly * sizeof(float);
      const void *dr = nullptr, *di = nullptr;
      LITHO_RET(stage_in(ctx, ctx->stage_in, mskf_r, spec, LITHO_MEM_HOST, &dr));
      LITHO_RET(stage_in(ctx, ctx->stage_x, mskf_i, spec, LITHO_MEM_HOST, &di));
      LITHO_RET(ctx->stage_k.ensure(ctx, (size_t)nk * kdim * sizeof(float2)));
      LITHO_RET(ctx->stage_s.ensure(ctx, (size_t)nk * sizeof(float)));
      LITHO_RET(upload_kernels(ctx, krn_r, krn_i, scales, nk, kdim, LITHO_MEM_HOST, ctx->stage_k.as<float2>(),
                               ctx->stage_s.as<float>()));
      ImgGeom g{Lx, Ly, Lx, Ly, nx_actual, ny_actual, nk, N};
      ImgPlan p = make_plan(g, 1, ctx->sm_count);
      p.kpg = nk;
      p.ngroups = 1;
      LITHO_RET(ctx->band_part.ensure(ctx, (size_t)(2 * ny_actual + 1) * (4 * nx_actual + 1) * sizeof(float2)));
      LITHO_RET(ctx->stage_out.ensure(ctx, out_n * sizeof(float)));
      WindowSrc w;
      w.mskf_r = static_cast<const float*>(dr);
      w.mskf_i = static_cast<const float*>(di);
      LITHO_RET(run_socs(ctx, p, w, ctx->stage_k.as<float2>(), ctx->stage_s.as<float>(), ctx->band_part.as<float2>(),
                         ctx->stage_out.as<float>()));
      std::vector<float> h(out_n);
      LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(h.data(), ctx->stage_out.p, out_n * sizeof(float), cudaMemcpyDeviceToHost,
                                          ctx->stream));
      LITHO_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
      if (tmpImg_ddr) std::copy(h.begin(), h.end(), tmpImg_ddr);
      if (output) std::copy(h.begin(), h.end(), output);
      return LITHO_OK;
    }();
  }
  if (rc != LITHO_OK) {
    fprintf(stderr, "calc_socs_2048_hls_stream_refactored_v18: %s\n",
            ctx ? litho_last_error(ctx) : "no CUDA device");
    fill_nan(tmpImg_ddr, out_n);
    fill_nan(output, out_n);
  }
}

// calc_tcc.cpp:34-191: TCC (tccSize x tccSize, std::complex<float>) of the
// source with the caller's sh and oSgm.  Accumulated in FP64, stored as float.
void calc_tcc(data_t* src, int srcSize, cmpxData_t* tcc, OpticalParams& params, int tccSize, int sh, int oSgm) {
  litho_ctx* ctx = hls_ctx();
  const size_t nn = (size_t)tccSize * tccSize;
  int rc = LITHO_ERR_CUDA;
  if (ctx != nullptr && src && tcc && tccSize == (2 * params.Nx + 1) * (2 * params.Ny + 1)) {
    std::vector<double> t(2 * nn);
    rc = calc_tcc_impl(ctx, src, srcSize, params.outerSigma, params.lambda, params.NA, params.defocus,
                       (int)params.Lx, (int)params.Ly, params.Nx, params.Ny, t.data(), LITHO_TCC_FP64, LITHO_MEM_HOST,
                       sh, oSgm);
    if (rc == LITHO_OK)
      for (size_t i = 0; i < nn; ++i) tcc[i] = cmpxData_t((float)t[2 * i], (float)t[2 * i + 1]);
  }
  if (rc != LITHO_OK) {
    fprintf(stderr, "calc_tcc: %s\n", ctx ? litho_last_error(ctx) : "no CUDA device or tccSize mismatch");
    for (size_t i = 0; tcc && i < nn; ++i)
      tcc[i] = cmpxData_t(std::numeric_limits<float>::quiet_NaN(), std::numeric_limits<float>::quiet_NaN());
  }
}
