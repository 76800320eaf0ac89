// Internal declarations shared by the liblitho_gb300 translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <string>
#include <map>
#include <memory>
#include <tuple>
#include <vector>

#include "../../include/litho_gb300.h"
#include "win_tiles.hpp"

namespace litho {

// ---------------------------------------------------------------------------
// error plumbing
// ---------------------------------------------------------------------------
struct Status {
  int code = LITHO_OK;
  std::string msg;
};

void set_error(litho_ctx* ctx, int code, const char* fmt, ...);

#define LITHO_CUDA_TRY(ctx, call)                                                       \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      ::litho::set_error((ctx), LITHO_ERR_CUDA, "%s failed: %s (%s:%d)", #call,          \
                         cudaGetErrorString(e_), __FILE__, __LINE__);                   \
      return LITHO_ERR_CUDA;                                                            \
    }                                                                                   \
  } while (0)

#define LITHO_ARG_CHECK(ctx, cond, ...)                                                 \
  do {                                                                                  \
    if (!(cond)) {                                                                      \
      ::litho::set_error((ctx), LITHO_ERR_ARG, __VA_ARGS__);                            \
      return LITHO_ERR_ARG;                                                             \
    }                                                                                   \
  } while (0)

#define LITHO_RET(expr)             \
  do {                              \
    int r_ = (expr);                \
    if (r_ != LITHO_OK) return r_;  \
  } while (0)

// ---------------------------------------------------------------------------
// grow-only device buffer owned by a context
// ---------------------------------------------------------------------------
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  int ensure(litho_ctx* ctx, size_t need);
  void release();
  template <class T> T* as() const { return static_cast<T*>(p); }
};

// Sum of n float2 values p[0], p[stride], ... (partials written by an earlier
// kernel): eight independent loads in flight and a fixed summation order.
__device__ __forceinline__ float2 sum_strided(const float2* __restrict__ p, size_t stride, int n) {
  float2 a[8];
#pragma unroll
  for (int u = 0; u < 8; ++u) a[u] = make_float2(0.f, 0.f);
  int i = 0;
  for (; i + 8 <= n; i += 8) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const float2 t = __ldg(p + (size_t)(i + u) * stride);
      a[u].x += t.x;
      a[u].y += t.y;
    }
  }
#pragma unroll
  for (int u = 0; u < 7; ++u)
    if (i + u < n) {
      const float2 t = __ldg(p + (size_t)(i + u) * stride);
      a[u].x += t.x;
      a[u].y += t.y;
    }
  return make_float2(((a[0].x + a[1].x) + (a[2].x + a[3].x)) + ((a[4].x + a[5].x) + (a[6].x + a[7].x)),
                     ((a[0].y + a[1].y) + (a[2].y + a[3].y)) + ((a[4].y + a[5].y) + (a[6].y + a[7].y)));
}

// Autotuned shape of the split-BF16 TCC GEMM for one (n, Kp): column tile width, K
// slice, schedule (gemm_schedule's sched) and every candidate's measured time.
struct TccTune {
  struct Cand {
    int bn, bk, sched;
    float ms;
  };
  int bn = 128, bk = 64, sched = 0;
  std::vector<Cand> cands;
};

inline int next_pow2(int x) {
  int p = 1;
  while (p < x) p <<= 1;
  return p;
}
inline bool is_pow2(int x) { return x > 0 && (x & (x - 1)) == 0; }

}  // namespace litho

// The context.  One stream, a set of grow-only workspaces and cached tables.
// device staging slots each way of the host-buffer imaging pipeline (6 measured
// no faster: chunked copies, not slot reuse, bound the pipeline)
constexpr int HB_SLOTS = 3;

struct litho_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::string last_error;
  // imaging workspaces
  litho::DevBuf win_part, band_part, tm, stage_in, stage_out, stage_k, stage_s, stage_x, band_w;
  // how the SOCS band is formed for kernel sets that carry a TCC band table
  // (litho_ctx_set_band_method): LITHO_BAND_AUTO / _FFT / _TCC
  int band_method = 0;
  // mask bytes per chunk of the host-buffer path (litho_ctx_set_host_chunk); 0: default
  size_t host_chunk_bytes = 0;
  // window-DFT column twiddle tables keyed by (Lx, Fx, Nx, NJT)
  std::map<std::tuple<int, int, int, int>, litho::DevBuf> twx_tables;
  // TCC / eigensolver workspaces
  litho::DevBuf tcc_a, tcc_b, tcc_c, tcc_pq, eig_w, eig_v, eig_work, eig_info;
  // mixed-precision (tensor-core) workspaces
  litho::DevBuf mx_b, mx_c, mx_d;
  // host-buffer batches: copy streams and per-slot events of the staging pipeline
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  cudaEvent_t ev_in[HB_SLOTS] = {}, ev_comp[HB_SLOTS] = {}, ev_out[HB_SLOTS] = {}, ev_start = nullptr;
  // per-stage timers
  bool timing = false;
  double stage_ms[LITHO_STAGE_COUNT] = {};
  long long stage_launches[LITHO_STAGE_COUNT] = {};
  struct Pending { int stage; cudaEvent_t a, b; };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> event_pool;
  // split-BF16 TCC GEMM: tuned shape per (n, Kp) and device schedule tables per
  // (n, K slices, BN, split)
  std::map<std::pair<int, int>, litho::TccTune> tcc_tune;
  std::map<std::tuple<int, int, int, int>, std::shared_ptr<void>> gemm_tables;
  int tcc_force_bn = 0, tcc_force_bk = 64, tcc_force_sched = 0;  // litho_tcc_gemm_shape: bn > 0 bypasses the tuner
  // error-path test hook (litho_ctx_set_test_stall): >= 0 stops the mixed window
  // DFT's TMA producer at that chunk of every CTA's work; -1 = off
  int test_stall_chunk = -1;
};

struct litho_kernel_set {
  litho_ctx* ctx = nullptr;
  int nk = 0, Nx = 0, Ny = 0;
  float2* krn = nullptr;    // [nk][(2Ny+1)(2Nx+1)]
  float* scales = nullptr;  // [nk]
  // rank-K TCC over the window, T(p, q) = sum_k s_k K_k(p) conj(K_k(q)), laid out for
  // band_tcc_kernel in band_nc row chunks (band_tcc.cu); band_nc == 0: none
  float2* band_tab = nullptr;
  int band_nc = 0;
};

namespace litho {

// Brackets one stage's launches with CUDA events when timing is on and counts
// its kernel launches always.
struct StageScope {
  litho_ctx* ctx;
  int stage;
  cudaEvent_t b = nullptr;
  StageScope(litho_ctx* c, int s, int launches = 1);
  ~StageScope();
};

// ---------------------------------------------------------------------------
// imaging pipeline (imaging.cu)
// ---------------------------------------------------------------------------
struct ImgGeom {
  int Lx, Ly;   // physical size (image and mask)
  int Fx, Fy;   // padded FFT size (power of two >= L)
  int Nx, Ny;   // kernel half-support
  int nk;
  int convN;    // SOCS conv grid (power of two >= 4*max(N)+1)
};

// Launch plan for one batch of one size class.
struct ImgPlan {
  ImgGeom g;
  int batch = 1;
  int rowBlocks = 1, colSplits = 1;  // window-DFT partition -> nparts
  int kpg = 1, ngroups = 1;          // SOCS kernels per CTA -> ngroups
  int part_stride = 0;               // >0: window partials per image in a shared per-class array
  int sms = 0;                       // SMs of the device (launch sizing)
  int nparts() const { return rowBlocks * colSplits; }
};

ImgPlan make_plan(const ImgGeom& g, int batch, int sm_count);

// SOCS conv grid used by the imaging entry points: pow2 >= 4 max(Nx, Ny) + 1, at least 32.
int default_conv_n(int Nx, int Ny);

int calc_tcc_impl(litho_ctx* ctx, const float* src, int srcSize, float outerSigma, float wavelength, float NA,
                  float defocus, int Lx, int Ly, int Nx, int Ny, double* tcc, int tccPrecision, int mem, int sh_in,
                  int oSgm_in, float n_medium = 1.0f);

// Host input -> device staging buffer (device input passes through).
int stage_in(litho_ctx* ctx, DevBuf& buf, const void* src, size_t bytes, int mem, const void** dev);

// Window source for the SOCS stage.
struct WindowSrc {
  const float2* part = nullptr;  // [batch][nparts][2Ny+1][Nx+1] partial sums (fused path)
  int nparts = 0;
  const float* mskf_r = nullptr;  // or full spectrum planes [batch][Fy][Fx]
  const float* mskf_i = nullptr;
};

int run_win_dft(litho_ctx* ctx, const ImgPlan& p, const float* masks, float2* win_part);
int prepare_win_dft(litho_ctx* ctx, const ImgPlan& p);  // cached tables, on ctx->stream
int run_socs(litho_ctx* ctx, const ImgPlan& p, const WindowSrc& w, const float2* krn,
             const float* scales, float2* band_part, float* tmpImgp);
int run_fi(litho_ctx* ctx, const ImgPlan& p, const float2* band_part, float* tm, float* images);
// FI step 1 for both layouts (tmh == nullptr: plain tm; else K-major hi/lo + t0);
// twF == nullptr evaluates the column twiddles in the kernel
cudaError_t launch_fi_rows(cudaStream_t s, const ImgPlan& p, const float2* band_part, const float2* twF, int KP,
                           float* tm, float* tmh, float* tml, float* t0);
int fi_twiddles(litho_ctx* ctx, const ImgGeom& g, const float2** out);
int run_fft_mask(litho_ctx* ctx, const float* mask, int Lx, int Ly, float* mskf_r, float* mskf_i);
int upload_kernels(litho_ctx* ctx, const float* krn_r, const float* krn_i, const float* scales,
                   int nk, int kdim, int mem, float2* krn_dev, float* scales_dev);

// Full imaging pipeline on device pointers for one size class (window DFT ->
// SOCS -> FI), FP32 or mixed precision.
int image_pipeline(litho_ctx* ctx, const ImgGeom& g, int batch, const float* masks,
                   const litho_kernel_set* ks, float* images, int precision);

// the SOCS band as the bilinear form of the kernel set's rank-K TCC (band_tcc.cu)
int build_band_table(litho_ctx* ctx, litho_kernel_set* ks, cudaStream_t stream);
size_t band_wsum_bytes(const ImgGeom& g, int batch);
int run_band_tcc(litho_ctx* ctx, const ImgPlan& p, const WindowSrc& w, const litho_kernel_set* ks,
                 float2* wsum, float2* band_part);
// whether the TCC band may serve a kernel set under the context's band method
inline bool band_tcc_available(const litho_ctx* ctx, const litho_kernel_set* ks) {
  return ks->band_nc > 0 && ctx->band_method != LITHO_BAND_FFT;
}
// whether a batch of images takes the TCC band: LITHO_BAND_TCC wherever the table exists,
// LITHO_BAND_AUTO where the band cost model (band_sched.hpp) expects it to be faster
bool use_band_tcc(const litho_ctx* ctx, const litho_kernel_set* ks, int batch);

// mixed precision window DFT / interpolation (imaging_tc.cu)
int run_win_dft_tc(litho_ctx* ctx, const ImgPlan& p, const float* masks, float2* win_part);
// masks of one size for a multi-size window launch (at most WIN_MAX_SIZES, win_tiles.hpp):
// its plan, its masks and its first image
// in the shared partial array
struct WinPart {
  ImgPlan plan;
  const float* masks;
  int img0;
};
int run_win_dft_tc_multi(litho_ctx* ctx, const WinPart* parts, int n, float2* win_part);
int run_fi_tc(litho_ctx* ctx, const ImgPlan& p, const float2* band_part, float* tmT, float* images);
struct FiTcBufs {
  float *tmh, *tml, *t0;
};
FiTcBufs fi_tc_bufs(float* base, const ImgGeom& g, int total, int first);
int run_fi_rows_tc(litho_ctx* ctx, const ImgPlan& p, const float2* band_part, const FiTcBufs& b);
int run_fi_out_tc(litho_ctx* ctx, const ImgPlan& p, const FiTcBufs& b, float* images);
size_t fi_tc_workspace_bytes(const ImgGeom& g, int batch);
bool tc_supported(const ImgGeom& g);
int tc_check_flag(litho_ctx* ctx);

}  // namespace litho
