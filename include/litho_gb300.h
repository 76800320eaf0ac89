/*
 * litho_gb300.h -- C ABI of liblitho_gb300.so, a GB300 (sm_103a) implementation
 * of the Hopkins/SOCS aerial-image path: TCC assembly, SOCS kernel extraction
 * and calcSOCS imaging (with Fourier interpolation).
 *
 * Every entry point replaces one function of the reference program
 * validation/golden/src/litho.cpp (or of its FPGA top functions) and keeps its
 * data conventions:
 *   - all arrays are row-major, float32 unless stated;
 *   - complex data is passed as separate real/imaginary planes (the BIN layout
 *     of mskf_r.bin / mskf_i.bin / kernels/krn_{k}_{r,i}.bin), or interleaved
 *     (re, im) float64 for the TCC (std::complex<double> layout);
 *   - SOCS kernels are concatenated k-major: kernel k occupies
 *     [k*(2Ny+1)*(2Nx+1), (k+1)*(2Ny+1)*(2Nx+1)), element ky*(2Nx+1)+kx,
 *     exactly as litho.cpp:1420-1425 writes them and the HLS top reads them
 *     (socs_2048_stream_refactored_v18_hls_fft.cpp:78);
 *   - the mask spectrum has DC at (fftLy/2, fftLx/2) and is divided by
 *     fftLx*fftLy (litho.cpp:242-318);
 *   - callers allocate every output; the library never exits the process and
 *     reports failures as LITHO_ERR_* status codes.
 *
 * Pointer location: entry points taking `int mem` accept either host pointers
 * (LITHO_MEM_HOST: the library stages them through its own device buffers and
 * returns after the results are back on the host) or device pointers
 * (LITHO_MEM_DEVICE: work is enqueued on the context's stream and the call
 * returns without synchronising).
 *
 * Threading: a litho_ctx is not re-entrant; use one context per host thread.
 */
#ifndef LITHO_GB300_H
#define LITHO_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define LITHO_OK               0
#define LITHO_ERR_ARG          1  /* invalid argument (size, pointer, nk > tccSize ...) */
#define LITHO_ERR_CUDA         2  /* a CUDA runtime call failed (see litho_last_error) */
#define LITHO_ERR_NOCONVERGE   3  /* eigensolver iteration cap reached */
#define LITHO_ERR_NAN          4  /* non-finite input or output detected */
#define LITHO_ERR_NOMEM        5  /* device or pinned allocation failed */
#define LITHO_ERR_IO           6  /* file read/write failed (BIN / JSON helpers) */
#define LITHO_ERR_UNSUPPORTED  7  /* size or mode outside what the library implements */
#define LITHO_ERR_TIMEOUT      8  /* a bounded device-side wait gave up */

#define LITHO_MEM_HOST   0
#define LITHO_MEM_DEVICE 1

/* Arithmetic of the imaging pipeline.
 * LITHO_PREC_FP32  : window DFT, FFTs, intensity sum and interpolation in FP32
 *                    on the CUDA cores (the plain path).
 * LITHO_PREC_MIXED : the two dense DFT contractions (mask -> spectrum window,
 *                    intensity band -> image) on the tensor cores with
 *                    split-operand TF32 products and FP32 accumulation; FFTs
 *                    and intensity sum in FP32.                               */
#define LITHO_PREC_FP32  0
#define LITHO_PREC_MIXED 1

/* How the SOCS band is formed for a kernel set (litho_ctx_set_band_method).
 * calcSOCS (litho.cpp:795-1006) sums s_k |IFFT(K_k . M)|^2 on the conv grid and the
 * interpolation (FI, litho.cpp:674-754) keeps the band |f| <= 2N of that intensity.
 * LITHO_BAND_FFT : per kernel a 2-D inverse FFT on the conv grid, |E|^2 summed,
 *                  one forward FFT of the intensity (the reference's order).
 * LITHO_BAND_TCC : the same band as the bilinear form of the rank-K TCC
 *                  T(p, q) = sum_k s_k K_k(p) conj(K_k(q)) over the kernel window,
 *                  band(f) = sum_{p-q=f} M(p) conj(M(q)) T(p, q); T is built once
 *                  per kernel set (FP64 sums, rounded to FP32), the sums in FP32.
 * LITHO_BAND_AUTO: per batch, the form a cost model fitted on GB300 expects to be
 *                  faster (TCC only where the kernel set has a table: 1 <= Nx <= 16,
 *                  Ny <= 16).  At K = 24 and 256 masks: TCC for Nx = Ny <= 10 and
 *                  16, FFT for 11..15 and for small batches (the default).         */
#define LITHO_BAND_AUTO 0
#define LITHO_BAND_FFT  1
#define LITHO_BAND_TCC  2

/* Arithmetic of the TCC contraction (litho.cpp:428-516).
 * LITHO_TCC_FP64      : pupil in FP32 exactly as the reference, FP64 accumulation.
 * LITHO_TCC_SPLIT_BF16: pupil split into three BF16 terms (hi*hi + hi*lo + lo*hi),
 *                       tensor-core (tcgen05) contraction with FP32 accumulation. */
#define LITHO_TCC_FP64       0
#define LITHO_TCC_SPLIT_BF16 1

typedef struct litho_ctx litho_ctx;

/* ---- context ----------------------------------------------------------- */
/* Create a context on CUDA device `device` with its own non-blocking stream. */
int litho_ctx_create(int device, litho_ctx** out);
int litho_ctx_destroy(litho_ctx* ctx);
/* Use a caller-owned stream (cudaStream_t passed as void*); NULL restores the
 * context's own stream (pass cudaStreamLegacy for the legacy default stream). */
int litho_ctx_set_stream(litho_ctx* ctx, void* stream);
void* litho_ctx_get_stream(litho_ctx* ctx);
/* Block until all work queued on the context's stream has finished. */
int litho_ctx_synchronize(litho_ctx* ctx);
/* Text of the last failure on this context (empty string if none). */
const char* litho_last_error(const litho_ctx* ctx);
const char* litho_status_string(int status);
/* Library version as major*10000 + minor*100 + patch. */
int litho_version(void);

/* ---- per-stage device timers ---------------------------------------------
 * The GPU counterpart of litho.cpp's per-module [TIME] lines
 * (litho.cpp:1259-1474).  When enabled, every stage launch is bracketed by CUDA
 * events on the context's stream.  Launch counts are kept whether or not timing
 * is enabled. */
#define LITHO_STAGE_WIN_DFT   0  /* mask -> spectrum window (partial DFT)        */
#define LITHO_STAGE_SOCS      1  /* K inverse FFTs + intensity + band            */
#define LITHO_STAGE_FI_PREP   2  /* band -> per-column interpolation rows        */
#define LITHO_STAGE_FI_OUT    3  /* interpolation contraction, image write       */
#define LITHO_STAGE_FFT_MASK  4  /* full centred mask spectrum                   */
#define LITHO_STAGE_TCC       5  /* pupil build + TCC contraction                */
#define LITHO_STAGE_EIG       6  /* Hermitian eigensolve                         */
#define LITHO_STAGE_UPLOAD    7  /* kernel packing and other small helpers       */
#define LITHO_STAGE_SURROGATE 8  /* FNO surrogate forward / backward / update    */
#define LITHO_STAGE_COUNT     9
int litho_ctx_enable_timing(litho_ctx* ctx, int enable);
/* Synchronise the stream; fill ms[LITHO_STAGE_COUNT] (summed device time) and
 * launches[LITHO_STAGE_COUNT] (kernel launches) since the last reset; either
 * output may be NULL.  reset != 0 clears the counters afterwards. */
int litho_ctx_stage_times(litho_ctx* ctx, double* ms, long long* launches, int reset);

/* ---- error-path test hook for the bounded device-side waits ----------------
 * No counterpart in the reference, whose failure handling is assert and exit
 * (common/file_io.cpp:137-150, litho.cpp:246-248).  chunk >= 0 makes the TMA
 * producer of the mixed-precision window DFT (LITHO_PREC_MIXED imaging) stop
 * issuing loads at that 64-column chunk of every CTA's share of the work, as if
 * it had been lost.  The consumers' waits then give up after their limit (about
 * one second), every role of the kernel leaves, the kernel frees its tensor
 * memory, and the call (or the next litho_ctx_synchronize, for device pointers)
 * returns LITHO_ERR_TIMEOUT; the images of that call are undefined.  -1, the
 * default, turns the hook off.  The value is read when a window DFT is launched
 * (and baked into a batch plan's graph when the plan is created).  For tests of
 * the error path only. */
int litho_ctx_set_test_stall(litho_ctx* ctx, int chunk);

/* ---- band method -------------------------------------------------------------
 * No reference counterpart (the reference has the FFT form only): selects
 * LITHO_BAND_AUTO / _FFT / _TCC for this context's batched imaging
 * (litho_image_batch, litho_batch_plan_create, the surrogate's fallback).  _TCC
 * with a kernel set that has no table images with the FFT form.  Read when work is
 * enqueued (and when a batch plan is created). */
int litho_ctx_set_band_method(litho_ctx* ctx, int method);

/* ---- host-buffer chunks -----------------------------------------------------
 * No reference counterpart.  litho_image_batch with LITHO_MEM_HOST moves the batch
 * through the device in chunks of at most `bytes` of masks (at least one mask, and at
 * least about eight chunks per batch), copies in and out overlapping the imaging.
 * The device holds three staging slots of a chunk each way.  Larger chunks move
 * faster over the host link; 0 restores the default, 128 MB (768 MB of slots). */
int litho_ctx_set_host_chunk(litho_ctx* ctx, size_t bytes);

/* ---- optics helpers (litho.cpp:414-426, 1297-1302) --------------------- */
/* getOuterSigma: max lit-pixel radius / ((srcSize-1)/2), clamped to 1 as
 * litho.cpp:1298 does.  Host pointer. */
float litho_outer_sigma(const float* src, int srcSize);
/* Nx = floor(NA * L * (1 + outerSigma) / lambda) evaluated in float32. */
int litho_optics_n(float NA, int L, float outerSigma, float wavelength);

/* ---- sources, masks and files (host only; validation/golden/src/common/) --- */
#define LITHO_SRC_ANNULAR          0  /* params: innerRadius, outerRadius          source.cpp:5-23  */
#define LITHO_SRC_DIPOLE           1  /* params: radius, offset, onXAxis (0/1)     source.cpp:58-87 */
#define LITHO_SRC_CROSS_QUADRUPOLE 2  /* params: radius, offset                    source.cpp:25-56 */
#define LITHO_SRC_POINT            3  /* params: x, y                              source.cpp:121-128 */
#define LITHO_SRC_KEEP             4  /* reserved: an imported source is normalised with litho_normalize_source */
/* createSource (source.cpp:105-141): fill src (S x S) and, if normalize, scale to
 * unit sum with the reference's sequential float32 sum. */
int litho_create_source(float* src, int srcSize, int type, const float* params, int normalize);
int litho_normalize_source(float* src, int srcSize);
/* generateLineSpace (mask.cpp:5-29) */
int litho_create_linespace(float* mask, int sizeX, int sizeY, int lineWidth, int spaceWidth, int horizontal);
/* createMask placement (mask.cpp:52-59): centre maskX x maskY in the Lx x Ly period, times dose */
int litho_place_mask(const float* in, int maskX, int maskY, float dose, float* out, int Lx, int Ly);
/* BIN files (file_io.cpp:137-150, 232-259): raw float32; reading a file of the
 * wrong size warns and truncates / zero-pads, as the reference does */
int litho_write_bin(const char* path, const float* data, long long n);
int litho_read_bin(const char* path, float* data, long long n);
/* kernels/kernel_info.txt (file_io.cpp:262-307) */
int litho_write_kernel_info(const char* path, int krnX, int krnY, int nk, const float* scales);
int litho_read_kernel_info(const char* path, int* krnX, int* krnY, int* nk, float* scales, int cap);

/* ---- mask spectrum (litho.cpp:242-318 FT_r2c_padded) --------------------
 * mask: Ly x Lx.  Outputs fftLy x fftLx planes with fftL = nextPow2(L); DC at
 * (fftLy/2, fftLx/2), divided by fftLx*fftLy. */
int litho_fft_mask(litho_ctx* ctx, const float* mask, int Lx, int Ly,
                   float* mskf_r, float* mskf_i, int mem);

/* ---- SOCS imaging from a mask spectrum (litho.cpp:795-1006 calcSOCS) ----
 * mskf_r/mskf_i: fftLy x fftLx planes (litho_fft_mask output).
 * krn_r/krn_i: nk kernels, k-major, (2Ny+1)*(2Nx+1) each.  scales: nk.
 * image: physLy x physLx output (calcSOCS + FI + centred crop).
 * tmpImgp (optional, NULL to skip): convN x convN fftshifted intensity before
 * interpolation (litho.cpp:934, the tmpImgp_full_{N}.bin dump).
 * convN: conv grid; 0 selects 128 as litho.cpp:815-816 forces.  Any power of
 * two >= 4*max(Nx,Ny)+1 gives the same image (the embed position only adds a
 * linear phase before |.|^2). */
int litho_calc_socs(litho_ctx* ctx, const float* mskf_r, const float* mskf_i,
                    int fftLx, int fftLy, const float* krn_r, const float* krn_i,
                    const float* scales, int nk, int Nx, int Ny, int physLx, int physLy,
                    float* image, float* tmpImgp, int convN, int mem);

/* ---- TCC-direct image (litho.cpp:522-566 calcImage + 358-408 FT_c2r_padded)
 * mskf planes (fftLy x fftLx) and the interleaved float64 TCC -> physLy x physLx
 * image, accumulated in FP64 exactly as calcImage orders the terms. */
int litho_calc_image(litho_ctx* ctx, const float* mskf_r, const float* mskf_i, int fftLx, int fftLy,
                     const double* tcc, int tccSize, int Nx, int Ny, int physLx, int physLy, float* image, int mem);

/* ---- fused mask -> aerial image (FT_r2c_padded + calcSOCS, litho.cpp:1318-1451)
 * One mask (Ly x Lx) to one image (Ly x Lx).  Only the (2Ny+1)x(2Nx+1) window
 * of the spectrum is formed (a partial DFT), so the full spectrum never
 * touches HBM.  precision: LITHO_PREC_FP32 or LITHO_PREC_MIXED. */
int litho_image(litho_ctx* ctx, const float* mask, int Lx, int Ly,
                const float* krn_r, const float* krn_i, const float* scales, int nk,
                int Nx, int Ny, float* image, int precision, int mem);

/* ---- batched imaging ------------------------------------------------------
 * A kernel set is uploaded once and reused by every batch (kernels fixed, as in
 * the reference's FPGA flow).  Masks of one batch share (Lx, Ly); masks are
 * packed back to back (image i at offset i*Lx*Ly), outputs likewise.  Creating a
 * set with 1 <= Nx <= 16 and Ny <= 16 also builds its rank-K TCC band table on the
 * device (LITHO_BAND_TCC; 0.37 MB at Nx = Ny = 8, 5.0 MB at 16). */
typedef struct litho_kernel_set litho_kernel_set;
int litho_kernel_set_create(litho_ctx* ctx, const float* krn_r, const float* krn_i,
                            const float* scales, int nk, int Nx, int Ny, int mem,
                            litho_kernel_set** out);
int litho_kernel_set_destroy(litho_kernel_set* ks);
int litho_image_batch(litho_ctx* ctx, const litho_kernel_set* ks, const float* masks,
                      int batch, int Lx, int Ly, float* images, int precision, int mem);

/* ---- batched imaging of masks of uneven sizes in one CUDA graph -----------
 * No single reference function: the reference images one mask per litho run
 * (validation/batch_test_runner.py:30-171 loops over masks).  Each item names
 * a size class (a kernel set and its period L, a power of two) and its mask
 * size mLx x mLy <= L; as common/mask.cpp:31-60 createMask does, a smaller mask
 * is centred in the period and the image is L x L.  The plan owns device slots
 * for every mask and image, chooses per size class the conv grid (FFT plan),
 * the kernels per CTA and the window-DFT split by timing candidates on the
 * device (LITHO_BATCH_AUTOTUNE), and captures all stages of all classes in one
 * CUDA graph (LITHO_BATCH_GRAPH) that litho_batch_plan_run launches. */
typedef struct {
  int cls;        /* index into the kernel-set / period arrays */
  int mLx, mLy;   /* mask size, <= the class period */
} litho_batch_item;
typedef struct litho_batch_plan litho_batch_plan;
#define LITHO_BATCH_AUTOTUNE 1
#define LITHO_BATCH_GRAPH    2
int litho_batch_plan_create(litho_ctx* ctx, const litho_kernel_set* const* sets, const int* periods, int nsets,
                            const litho_batch_item* items, int n, int precision, int flags,
                            litho_batch_plan** out);
/* device slot of item i's mask (mLy x mLx float32) and image (L x L float32) */
float* litho_batch_plan_mask(litho_batch_plan* plan, int i);
float* litho_batch_plan_image(litho_batch_plan* plan, int i);
/* image every item: one graph launch (or the plain launch sequence) on the context's stream */
int litho_batch_plan_run(litho_batch_plan* plan);
/* JSON description of the tuned choices per size class; returns the length written */
int litho_batch_plan_describe(const litho_batch_plan* plan, char* buf, int cap);
int litho_batch_plan_destroy(litho_batch_plan* plan);

/* ---- mask -> image with no device allocation ------------------------------
 * No counterpart in the reference.  For callers that cannot let a library call
 * cudaMalloc/cudaFree: those calls synchronise the whole device (a latency-
 * critical loop on several streams cannot afford that), and a plugin whose host
 * application owns the device memory budget through its own allocator must not
 * allocate behind it.  The same FP32 pipeline as litho_image, but its
 * intermediates live in one fixed 6 MiB __device__ array compiled into the
 * library (held by every GPU that loads it until the process exits).
 * All pointers are device pointers on the current device; work is queued on
 * `stream` (cudaStream_t as void*, NULL = legacy default stream) and the call
 * returns without synchronising.  Limits: 2 <= Lx, Ly <= 4096, Nx, Ny <= 16,
 * 1 <= nk <= 64; anything beyond returns LITHO_ERR_ARG.  The first call on a
 * device looks up the array's device address (make it before any stream
 * capture); the address is kept for the life of the process, so do not reset
 * the device (cudaDeviceReset) between calls.  Calls share the array: calls whose work overlaps on the GPU race
 * and must be serialised by the caller. */
int litho_image_noalloc(const float* mask, int Lx, int Ly, const float* krn_r, const float* krn_i,
                        const float* scales, int nk, int Nx, int Ny, float* image, void* stream);

/* ---- learned surrogate (no reference counterpart) -------------------------
 * FNO-2d (Li et al. 2021) of the SOCS map mask -> aerial image on an L x L
 * grid: one input channel, LITHO_FNO_WIDTH channels, LITHO_FNO_MODES retained
 * modes per axis, LITHO_FNO_LAYERS Fourier layers, a width -> HIDDEN -> 1
 * projection.  FP32 master weights; GEMMs in BF16 on the tensor cores.
 * Masks, images and targets are DEVICE pointers ([batch][L][L] float32),
 * launched on the context's stream.  Parameters are one flat float32 vector:
 *   Pw[32] Pb[32] | W[4][32 o][32 c] | Wb[4][32] |
 *   R[4][32 ky-slot][16 kx][32 c][32 o][re,im] (ky = j for j < 16, L-32+j else) |
 *   Q1[128][32] | q1b[128] | Q2[128] | q2b[1]                                    */
#define LITHO_FNO_WIDTH  32
#define LITHO_FNO_MODES  16
#define LITHO_FNO_HIDDEN 128
#define LITHO_FNO_LAYERS 4
typedef struct litho_fno litho_fno;

long long litho_surrogate_num_params(void);
/* L in {64, 128, 256}; parameters initialised from `seed` (Kaiming-uniform
 * linear layers, spectral weights U[0,1)/width^2). */
int  litho_surrogate_create(litho_ctx* ctx, int L, unsigned long long seed, litho_fno** out);
void litho_surrogate_destroy(litho_fno* f);
int  litho_surrogate_get_params(litho_fno* f, float* host, long long n);
/* also resets the Adam state */
int  litho_surrogate_set_params(litho_fno* f, const float* host, long long n);
int  litho_surrogate_forward(litho_fno* f, const float* masks, int batch, float* images);
/* loss = mean_b ||F(m_b) - t_b|| / ||t_b|| (host float, optional) and its
 * gradient (host copy into grad_host[num_params], optional). */
int  litho_surrogate_loss_grad(litho_fno* f, const float* masks, const float* targets, int batch,
                               float* loss, float* grad_host);
/* one Adam step (beta 0.9/0.999, eps 1e-8, L2 weight decay added to the gradient). */
int  litho_surrogate_train_step(litho_fno* f, const float* masks, const float* targets, int batch,
                                float lr, float weight_decay, float* loss);
/* Seeded rectangle masks first .. first+count-1 of the stream `seed`: nrect in
 * [nmin, nmax] (<= 256) axis-aligned rectangles, sides in [wmin, wmax] (<= L),
 * value 1 on 0.  SplitMix64 counters, so any sub-range is reproducible. */
int  litho_rect_masks(litho_ctx* ctx, unsigned long long seed, long long first, int count, int L,
                      int nmin, int nmax, int wmin, int wmax, float* masks);
/* Band projection and error estimates.  Every SOCS image of kernels with half
 * widths (Nx, Ny) is band-limited to |kx| <= 2 Nx, |ky| <= 2 Ny (in 1/L), so
 * the surrogate's image is replaced by its band part (in place; the L2 error
 * can only shrink).  litho_surrogate_project writes est[b] = alpha * ||removed
 * part|| / ||band part||.  litho_surrogate_predict runs the network, the
 * projection and the estimator: the image's coefficients at the lowest
 * frequencies q in {-1,0,1}^2 are computed exactly from the mask's window
 * spectrum and the kernels, I(q) = 1/L^2 sum_k s_k sum_f B_k(f+q) conj(B_k(f)),
 * B_k = krn_k * DFT(mask), and est[b] = alpha * ||I_net(q) - I(q)|| / ||image||
 * (Parseval-weighted).  Arrays are DEVICE pointers; 2 Nx, 2 Ny <= 15, nk <= 64. */
int   litho_surrogate_set_alpha(litho_fno* f, float alpha);
float litho_surrogate_get_alpha(const litho_fno* f);
int   litho_surrogate_project(litho_fno* f, int Nx, int Ny, float* images, int batch, float* est);
int   litho_surrogate_predict(litho_fno* f, const litho_kernel_set* ks, const float* masks, int batch,
                              float* images, float* est);
/* Surrogate imaging with fallback: litho_surrogate_predict, then masks whose
 * estimate is above `threshold` (or NaN) are imaged by the plain FP32 SOCS
 * path with the kernel set instead.  est_host[batch] and used_socs[batch]
 * (host, optional) report the estimate and the choice. */
int   litho_surrogate_image(litho_fno* f, const litho_kernel_set* ks, const float* masks, int batch,
                            float threshold, float* images, float* est_host, int* used_socs);

/* ---- TCC (litho.cpp:428-516 calcTCC) --------------------------------------
 * src: srcSize x srcSize normalised source (host or device per mem).
 * tcc: tccSize x tccSize interleaved (re, im) float64, tccSize=(2Nx+1)(2Ny+1);
 * Hermitian, upper triangle accumulated then mirrored as the reference. */
int litho_calc_tcc(litho_ctx* ctx, const float* src, int srcSize, float outerSigma,
                   float wavelength, float NA, float defocus, int Lx, int Ly, int Nx, int Ny,
                   double* tcc, int tccPrecision, int mem);

/* Shape of the split-BF16 TCC GEMM (no reference counterpart: the reference
 * accumulates the TCC in scalar loops, litho.cpp:477-515).  By default the
 * shape is chosen per (tccSize, padded source count) by timing every candidate
 * on the device the first time that size is seen, and cached on the context:
 * the column tile width bn of the 128-row output tiles and the K slice bk of
 * one pipeline stage, (bn, bk) in {(64, 64), (128, 64), (256, 64), (128, 32),
 * (256, 32)}, and the schedule of the persistent CTAs: 0 = whole tiles only;
 * 1 = whole tiles for all but the last one or two rounds, whose tiles are split
 * along K over all SMs; 2 = whole tiles for every full round, only the last
 * partial round split along K.  litho_tcc_gemm_shape fixes them instead
 * (bn = 0 restores the tuner); litho_tcc_gemm_describe writes the cached
 * choices and every candidate's time as JSON and returns the length written. */
int litho_tcc_gemm_shape(litho_ctx* ctx, int bn, int bk, int sched);
int litho_tcc_gemm_describe(const litho_ctx* ctx, char* buf, int cap);

/* Immersion extension (no reference counterpart): the pupil phase is
 * dz k sqrt(n_medium^2 - rho^2 NA^2) instead of litho.cpp:463's sqrt(1 - rho^2 NA^2),
 * so NA > 1 (immersion optics) gives a finite TCC when n_medium >= NA.
 * n_medium = 1 is litho_calc_tcc. */
int litho_calc_tcc_medium(litho_ctx* ctx, const float* src, int srcSize, float outerSigma,
                          float wavelength, float NA, float defocus, float n_medium, int Lx, int Ly,
                          int Nx, int Ny, double* tcc, int tccPrecision, int mem);

/* ---- SOCS kernels (litho.cpp:579-645 calcKernels) --------------------------
 * Top-nk eigenpairs of the Hermitian tcc (interleaved float64, upper triangle
 * used as zheevr 'U').  scales descending (float32, and optionally float64);
 * kernel i is eigenvector i stored reversed: krn[i][j] = v_i[n-1-j].
 * krn64 (optional): nk*tccSize interleaved float64 kernels. */
int litho_calc_kernels(litho_ctx* ctx, const double* tcc, int tccSize, int nk,
                       float* krn_r, float* krn_i, float* scales,
                       double* krn64, double* scales64, int mem);

#ifdef __cplusplus
}
#endif
#endif /* LITHO_GB300_H */
