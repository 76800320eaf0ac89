// C ABI of liblitho_gb300.so: contexts, host/device staging and the imaging
// entry points.  TCC and eigensolver entry points live in tcc.cu / eig.cu.
#include "litho_internal.cuh"
#include "host_chunks.hpp"

#include <cmath>
#include <cstring>
#include <vector>

namespace litho {

void set_error(litho_ctx* ctx, int code, const char* fmt, ...) {
  if (ctx == nullptr) return;
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  ctx->last_error = std::string(litho_status_string(code)) + ": " + buf;
}

int DevBuf::ensure(litho_ctx* ctx, size_t need) {
  if (need <= bytes && p != nullptr) return LITHO_OK;
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
  size_t n = need < 256 ? 256 : need;
  cudaError_t e = cudaMalloc(&p, n);
  if (e != cudaSuccess) {
    p = nullptr;
    set_error(ctx, LITHO_ERR_NOMEM, "cudaMalloc(%zu) failed: %s", n, cudaGetErrorString(e));
    return LITHO_ERR_NOMEM;
  }
  bytes = n;
  return LITHO_OK;
}

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

static cudaEvent_t pool_get(litho_ctx* ctx) {
  if (!ctx->event_pool.empty()) {
    cudaEvent_t e = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

StageScope::StageScope(litho_ctx* c, int s, int launches) : ctx(c), stage(s) {
  ctx->stage_launches[stage] += launches;
  if (ctx->timing) {
    cudaEvent_t a = pool_get(ctx);
    b = pool_get(ctx);
    cudaEventRecord(a, ctx->stream);
    ctx->pending.push_back({stage, a, b});
  }
}

StageScope::~StageScope() {
  if (b) cudaEventRecord(b, ctx->stream);
}

// Copy a host or device input into a device pointer usable by kernels.
int stage_in(litho_ctx* ctx, DevBuf& buf, const void* src, size_t bytes, int mem, const void** dev) {
  if (mem == LITHO_MEM_DEVICE) {
    *dev = src;
    return LITHO_OK;
  }
  LITHO_RET(buf.ensure(ctx, bytes));
  LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(buf.p, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
  *dev = buf.p;
  return LITHO_OK;
}

}  // namespace litho

using namespace litho;

extern "C" {

const char* litho_status_string(int s) {
  switch (s) {
    case LITHO_OK: return "LITHO_OK";
    case LITHO_ERR_ARG: return "LITHO_ERR_ARG";
    case LITHO_ERR_CUDA: return "LITHO_ERR_CUDA";
    case LITHO_ERR_NOCONVERGE: return "LITHO_ERR_NOCONVERGE";
    case LITHO_ERR_NAN: return "LITHO_ERR_NAN";
    case LITHO_ERR_NOMEM: return "LITHO_ERR_NOMEM";
    case LITHO_ERR_IO: return "LITHO_ERR_IO";
    case LITHO_ERR_UNSUPPORTED: return "LITHO_ERR_UNSUPPORTED";
    case LITHO_ERR_TIMEOUT: return "LITHO_ERR_TIMEOUT";
    default: return "LITHO_ERR_UNKNOWN";
  }
}

int litho_version(void) { return 10000; }

int litho_ctx_create(int device, litho_ctx** out) {
  if (out == nullptr) return LITHO_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return LITHO_ERR_CUDA;
  if (cudaSetDevice(device) != cudaSuccess) return LITHO_ERR_CUDA;
  litho_ctx* c = new litho_ctx();
  c->device = device;
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return LITHO_ERR_CUDA;
  }
  c->stream = c->own_stream;
  *out = c;
  return LITHO_OK;
}

int litho_ctx_destroy(litho_ctx* ctx) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  DevBuf* bufs[] = {&ctx->win_part, &ctx->band_part, &ctx->tm,     &ctx->stage_in, &ctx->stage_out,
                    &ctx->stage_k,  &ctx->stage_s,   &ctx->stage_x, &ctx->tcc_a,   &ctx->tcc_b,
                    &ctx->tcc_c,    &ctx->tcc_pq,  &ctx->eig_w,     &ctx->eig_v,   &ctx->eig_work, &ctx->eig_info,
                    &ctx->mx_b,     &ctx->mx_c,      &ctx->mx_d,    &ctx->band_w};
  for (DevBuf* b : bufs) b->release();
  for (auto& kv : ctx->twx_tables) kv.second.release();
  for (auto& p : ctx->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
  for (cudaStream_t st : {ctx->copy_in, ctx->copy_out})
    if (st) {
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
    }
  for (int i = 0; i < HB_SLOTS; ++i)
    for (cudaEvent_t e : {ctx->ev_in[i], ctx->ev_comp[i], ctx->ev_out[i]})
      if (e) cudaEventDestroy(e);
  if (ctx->ev_start) cudaEventDestroy(ctx->ev_start);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return LITHO_OK;
}

int litho_ctx_set_stream(litho_ctx* ctx, void* stream) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
  return LITHO_OK;
}

void* litho_ctx_get_stream(litho_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int litho_ctx_synchronize(litho_ctx* ctx) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  LITHO_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return tc_check_flag(ctx);
}

int litho_ctx_enable_timing(litho_ctx* ctx, int enable) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  ctx->timing = enable != 0;
  return LITHO_OK;
}

int litho_ctx_set_test_stall(litho_ctx* ctx, int chunk) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  LITHO_ARG_CHECK(ctx, chunk >= -1, "chunk must be >= -1 (-1 turns the hook off)");
  ctx->test_stall_chunk = chunk;
  return LITHO_OK;
}

int litho_ctx_set_band_method(litho_ctx* ctx, int method) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  LITHO_ARG_CHECK(ctx, method == LITHO_BAND_AUTO || method == LITHO_BAND_FFT || method == LITHO_BAND_TCC,
                  "bad band method %d", method);
  ctx->band_method = method;
  return LITHO_OK;
}

int litho_ctx_set_host_chunk(litho_ctx* ctx, size_t bytes) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  ctx->host_chunk_bytes = bytes;
  return LITHO_OK;
}

int litho_ctx_stage_times(litho_ctx* ctx, double* ms, long long* launches, int reset) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  LITHO_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  for (auto& p : ctx->pending) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess) ctx->stage_ms[p.stage] += t;
    ctx->event_pool.push_back(p.a);
    ctx->event_pool.push_back(p.b);
  }
  ctx->pending.clear();
  for (int i = 0; i < LITHO_STAGE_COUNT; ++i) {
    if (ms) ms[i] = ctx->stage_ms[i];
    if (launches) launches[i] = ctx->stage_launches[i];
    if (reset) {
      ctx->stage_ms[i] = 0.0;
      ctx->stage_launches[i] = 0;
    }
  }
  return LITHO_OK;
}

const char* litho_last_error(const litho_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

float litho_outer_sigma(const float* src, int srcSize) {
  // litho.cpp:414-426 (getOuterSigma) with the clamp of litho.cpp:1298
  if (src == nullptr || srcSize <= 0) return 0.f;
  const int c = (srcSize - 1) / 2;
  float maxd = 0.f;
  for (int y = 0; y < srcSize; ++y)
    for (int x = 0; x < srcSize; ++x)
      if (src[y * srcSize + x] != 0.0f) {
        const float d = (float)std::sqrt((double)((y - c) * (y - c) + (x - c) * (x - c)));
        if (d > maxd) maxd = d;
      }
  float s = (c == 0) ? 0.0f : (maxd / (float)c);
  return s > 1.f ? 1.f : s;
}

int litho_optics_n(float NA, int L, float outerSigma, float wavelength) {
  // litho.cpp:1300 in float32
  volatile float a = NA * (float)L;
  volatile float b = a * (1.0f + outerSigma);
  volatile float v = b / wavelength;
  return (int)std::floor(v);
}

int litho_fft_mask(litho_ctx* ctx, const float* mask, int Lx, int Ly, float* mskf_r, float* mskf_i, int mem) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  LITHO_ARG_CHECK(ctx, mask && mskf_r && mskf_i, "null pointer");
  LITHO_ARG_CHECK(ctx, Lx >= 2 && Ly >= 2 && Lx <= 8192 && Ly <= 8192, "mask size %dx%d outside [2, 8192]", Lx, Ly);
  LITHO_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  const int Fx = next_pow2(Lx), Fy = next_pow2(Ly);
  const void* dmask = nullptr;
  LITHO_RET(stage_in(ctx, ctx->stage_in, mask, (size_t)Lx * Ly * sizeof(float), mem, &dmask));
  float *dr = mskf_r, *di = mskf_i;
  if (mem == LITHO_MEM_HOST) {
    LITHO_RET(ctx->stage_out.ensure(ctx, (size_t)2 * Fx * Fy * sizeof(float)));
    dr = ctx->stage_out.as<float>();
    di = dr + (size_t)Fx * Fy;
  }
  LITHO_RET(run_fft_mask(ctx, static_cast<const float*>(dmask), Lx, Ly, dr, di));
  if (mem == LITHO_MEM_HOST) {
    LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(mskf_r, dr, (size_t)Fx * Fy * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(mskf_i, di, (size_t)Fx * Fy * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    LITHO_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return LITHO_OK;
}

}  // extern "C"

namespace litho {

// kernel planes (k-major, separate re/im) -> interleaved device float2
__global__ void pack_kernels_kernel(const float* __restrict__ kr, const float* __restrict__ ki, int n,
                                    float2* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_float2(kr[i], ki[i]);
}

int upload_kernels(litho_ctx* ctx, const float* krn_r, const float* krn_i, const float* scales, int nk,
                   int kdim, int mem, float2* krn_dev, float* scales_dev) {
  const size_t n = (size_t)nk * kdim;
  if (mem == LITHO_MEM_HOST) {
    std::vector<float2> tmp(n);
    for (size_t i = 0; i < n; ++i) tmp[i] = make_float2(krn_r[i], krn_i[i]);
    LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(krn_dev, tmp.data(), n * sizeof(float2), cudaMemcpyHostToDevice, ctx->stream));
    LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(scales_dev, scales, nk * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    // tmp must outlive the copy
    LITHO_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  } else {
    StageScope sc(ctx, LITHO_STAGE_UPLOAD);
    pack_kernels_kernel<<<(int)((n + 255) / 256), 256, 0, ctx->stream>>>(krn_r, krn_i, (int)n, krn_dev);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
    LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(scales_dev, scales, nk * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
  }
  return LITHO_OK;
}

static int check_geom(litho_ctx* ctx, int Lx, int Ly, int Nx, int Ny, int nk) {
  LITHO_ARG_CHECK(ctx, Lx >= 2 && Ly >= 2 && Lx <= 16384 && Ly <= 16384, "image size %dx%d outside [2, 16384]", Lx, Ly);
  LITHO_ARG_CHECK(ctx, Nx >= 0 && Ny >= 0, "negative Nx/Ny");
  LITHO_ARG_CHECK(ctx, nk >= 1, "nk must be >= 1 (got %d)", nk);
  if (Nx > 16 || Ny > 16) {
    set_error(ctx, LITHO_ERR_UNSUPPORTED, "imaging supports Nx, Ny <= 16 (got %d, %d)", Nx, Ny);
    return LITHO_ERR_UNSUPPORTED;
  }
  const int Fx = next_pow2(Lx), Fy = next_pow2(Ly);
  LITHO_ARG_CHECK(ctx, 2 * Nx + 1 <= Fx && 2 * Ny + 1 <= Fy, "kernel support exceeds the spectrum");
  return LITHO_OK;
}

int default_conv_n(int Nx, int Ny) {
  const int n = next_pow2(4 * (Nx > Ny ? Nx : Ny) + 1);
  return n < 32 ? 32 : n;
}

}  // namespace litho

// Host buffers: the batch moves in chunks of up to 128 MB (host_chunks.hpp) through HB_SLOTS
// device staging slots each way.  Host->device copies run on one copy stream
// and device->host copies on another, so chunk k+1 arrives and chunk k-1 leaves
// while chunk k is imaged on the context's stream; events order the reuse of
// every slot, and both copy streams join the context's stream at the end.
// Nothing overlaps the first chunk's copy in or the last chunk's copy out, so
// the chunk sizes ramp 1, 2, 4, ... masks up at the start and back down at the
// end (the host link, not the copy engines, bounds both directions: SM loads
// and stores on mapped host memory reach the same rates).
static int host_batch(litho_ctx* ctx, const ImgGeom& g, int batch, const float* masks, const litho_kernel_set* ks,
                      float* images, int precision, size_t img) {
  constexpr int NS = HB_SLOTS;
  const int CH = litho::host_chunk_masks(batch, img,
                                         ctx->host_chunk_bytes ? ctx->host_chunk_bytes : litho::HOST_CHUNK_BYTES);
  std::vector<int> sizes;
  litho::chunk_schedule(batch, CH, sizes);
  if (ctx->copy_in == nullptr) {
    LITHO_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&ctx->copy_in, cudaStreamNonBlocking));
    LITHO_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&ctx->copy_out, cudaStreamNonBlocking));
    for (int i = 0; i < NS; ++i) {
      LITHO_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->ev_in[i], cudaEventDisableTiming));
      LITHO_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->ev_comp[i], cudaEventDisableTiming));
      LITHO_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->ev_out[i], cudaEventDisableTiming));
    }
    LITHO_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->ev_start, cudaEventDisableTiming));
  }
  const int nchunk = (int)sizes.size();
  const int nslot = nchunk < NS ? nchunk : NS;
  LITHO_RET(ctx->stage_in.ensure(ctx, (size_t)nslot * CH * img));
  LITHO_RET(ctx->stage_out.ensure(ctx, (size_t)nslot * CH * img));
  char* din = ctx->stage_in.as<char>();
  char* dout = ctx->stage_out.as<char>();
  // both copy streams start after the caller's earlier work
  LITHO_CUDA_TRY(ctx, cudaEventRecord(ctx->ev_start, ctx->stream));
  LITHO_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->copy_in, ctx->ev_start, 0));
  LITHO_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->copy_out, ctx->ev_start, 0));
  size_t off = 0;
  for (int k = 0; k < nchunk; off += (size_t)sizes[k] * img, ++k) {
    const int sl = k % NS, nb = sizes[k];
    const size_t bytes = (size_t)nb * img;
    char* in = din + (size_t)sl * CH * img;
    char* out = dout + (size_t)sl * CH * img;
    if (k >= NS) LITHO_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->copy_in, ctx->ev_comp[sl], 0));  // slot read
    LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(in, reinterpret_cast<const char*>(masks) + off, bytes,
                                        cudaMemcpyHostToDevice, ctx->copy_in));
    LITHO_CUDA_TRY(ctx, cudaEventRecord(ctx->ev_in[sl], ctx->copy_in));
    LITHO_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_in[sl], 0));
    if (k >= NS) LITHO_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_out[sl], 0));  // slot drained
    LITHO_RET(image_pipeline(ctx, g, nb, reinterpret_cast<const float*>(in), ks,
                             reinterpret_cast<float*>(out), precision));
    LITHO_CUDA_TRY(ctx, cudaEventRecord(ctx->ev_comp[sl], ctx->stream));
    LITHO_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->copy_out, ctx->ev_comp[sl], 0));
    LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(reinterpret_cast<char*>(images) + off, out, bytes, cudaMemcpyDeviceToHost,
                                        ctx->copy_out));
    LITHO_CUDA_TRY(ctx, cudaEventRecord(ctx->ev_out[sl], ctx->copy_out));
  }
  // join: the context's stream continues after the last copy out
  for (int i = 0; i < nslot; ++i) LITHO_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_out[i], 0));
  return LITHO_OK;
}

extern "C" {

int litho_calc_socs(litho_ctx* ctx, const float* mskf_r, const float* mskf_i, int fftLx, int fftLy,
                    const float* krn_r, const float* krn_i, const float* scales, int nk, int Nx, int Ny,
                    int physLx, int physLy, float* image, float* tmpImgp, int convN, int mem) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  LITHO_ARG_CHECK(ctx, mskf_r && mskf_i && krn_r && krn_i && scales && image, "null pointer");
  LITHO_RET(check_geom(ctx, physLx, physLy, Nx, Ny, nk));
  LITHO_ARG_CHECK(ctx, is_pow2(fftLx) && is_pow2(fftLy) && fftLx >= physLx && fftLy >= physLy,
                  "fft size %dx%d must be powers of two >= the physical size", fftLx, fftLy);
  LITHO_ARG_CHECK(ctx, next_pow2(physLx) == fftLx && next_pow2(physLy) == fftLy,
                  "fft size must be nextPow2 of the physical size");
  if (convN == 0) convN = 128;  // litho.cpp:815-816
  LITHO_ARG_CHECK(ctx, convN == 32 || convN == 64 || convN == 128, "convN %d not in {32, 64, 128}", convN);
  LITHO_ARG_CHECK(ctx, convN >= 4 * Nx + 1 && convN >= 4 * Ny + 1, "convN %d < 4N+1: the intensity would alias", convN);
  LITHO_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  ImgGeom g{physLx, physLy, fftLx, fftLy, Nx, Ny, nk, convN};
  ImgPlan p = make_plan(g, 1, ctx->sm_count);
  if (tmpImgp) {
    p.kpg = nk;
    p.ngroups = 1;
  }
  const int kdim = (2 * Nx + 1) * (2 * Ny + 1);
  const size_t spec = (size_t)fftLx * fftLy * sizeof(float);
  const void *dr = nullptr, *di = nullptr;
  LITHO_RET(stage_in(ctx, ctx->stage_in, mskf_r, spec, mem, &dr));
  LITHO_RET(stage_in(ctx, ctx->stage_x, mskf_i, spec, mem, &di));
  LITHO_RET(ctx->stage_k.ensure(ctx, (size_t)nk * kdim * sizeof(float2)));
  LITHO_RET(ctx->stage_s.ensure(ctx, (size_t)nk * sizeof(float)));
  LITHO_RET(upload_kernels(ctx, krn_r, krn_i, scales, nk, kdim, mem, ctx->stage_k.as<float2>(), ctx->stage_s.as<float>()));
  const size_t img_bytes = (size_t)physLx * physLy * sizeof(float);
  const size_t tmp_bytes = (size_t)convN * convN * sizeof(float);
  float* dimg = image;
  float* dtmp = tmpImgp;
  if (mem == LITHO_MEM_HOST) {
    LITHO_RET(ctx->stage_out.ensure(ctx, img_bytes + tmp_bytes));
    dimg = ctx->stage_out.as<float>();
    dtmp = tmpImgp ? dimg + (size_t)physLx * physLy : nullptr;
  }
  const int KY = 2 * Ny + 1;
  LITHO_RET(ctx->band_part.ensure(ctx, (size_t)p.ngroups * KY * (4 * Nx + 1) * sizeof(float2)));
  LITHO_RET(ctx->tm.ensure(ctx, (size_t)(4 * Ny + 1) * physLx * sizeof(float)));
  WindowSrc w;
  w.mskf_r = static_cast<const float*>(dr);
  w.mskf_i = static_cast<const float*>(di);
  LITHO_RET(run_socs(ctx, p, w, ctx->stage_k.as<float2>(), ctx->stage_s.as<float>(), ctx->band_part.as<float2>(), dtmp));
  LITHO_RET(run_fi(ctx, p, ctx->band_part.as<float2>(), ctx->tm.as<float>(), dimg));
  if (mem == LITHO_MEM_HOST) {
    LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(image, dimg, img_bytes, cudaMemcpyDeviceToHost, ctx->stream));
    if (tmpImgp) LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(tmpImgp, dtmp, tmp_bytes, cudaMemcpyDeviceToHost, ctx->stream));
    LITHO_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return LITHO_OK;
}

int litho_kernel_set_create(litho_ctx* ctx, const float* krn_r, const float* krn_i, const float* scales, int nk,
                            int Nx, int Ny, int mem, litho_kernel_set** out) {
  if (ctx == nullptr || out == nullptr) return LITHO_ERR_ARG;
  *out = nullptr;
  LITHO_ARG_CHECK(ctx, krn_r && krn_i && scales, "null pointer");
  LITHO_ARG_CHECK(ctx, nk >= 1 && Nx >= 0 && Ny >= 0, "bad kernel set shape");
  LITHO_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  const int kdim = (2 * Nx + 1) * (2 * Ny + 1);
  litho_kernel_set* ks = new litho_kernel_set();
  ks->ctx = ctx;
  ks->nk = nk;
  ks->Nx = Nx;
  ks->Ny = Ny;
  if (cudaMalloc(&ks->krn, (size_t)nk * kdim * sizeof(float2)) != cudaSuccess ||
      cudaMalloc(&ks->scales, (size_t)nk * sizeof(float)) != cudaSuccess) {
    if (ks->krn) cudaFree(ks->krn);
    delete ks;
    set_error(ctx, LITHO_ERR_NOMEM, "kernel set allocation failed");
    return LITHO_ERR_NOMEM;
  }
  int rc = upload_kernels(ctx, krn_r, krn_i, scales, nk, kdim, mem, ks->krn, ks->scales);
  if (rc == LITHO_OK) rc = build_band_table(ctx, ks, ctx->stream);
  if (rc == LITHO_OK) rc = cudaStreamSynchronize(ctx->stream) == cudaSuccess ? LITHO_OK : LITHO_ERR_CUDA;
  if (rc != LITHO_OK) {
    cudaFree(ks->krn);
    cudaFree(ks->scales);
    if (ks->band_tab) cudaFree(ks->band_tab);
    delete ks;
    return rc;
  }
  *out = ks;
  return LITHO_OK;
}

int litho_kernel_set_destroy(litho_kernel_set* ks) {
  if (ks == nullptr) return LITHO_ERR_ARG;
  cudaSetDevice(ks->ctx->device);
  cudaFree(ks->krn);
  cudaFree(ks->scales);
  if (ks->band_tab) cudaFree(ks->band_tab);
  delete ks;
  return LITHO_OK;
}

int litho_image_batch(litho_ctx* ctx, const litho_kernel_set* ks, const float* masks, int batch, int Lx, int Ly,
                      float* images, int precision, int mem) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  LITHO_ARG_CHECK(ctx, ks && masks && images, "null pointer");
  LITHO_ARG_CHECK(ctx, ks->ctx == ctx, "kernel set belongs to another context");
  LITHO_ARG_CHECK(ctx, batch >= 1, "batch must be >= 1");
  LITHO_ARG_CHECK(ctx, precision == LITHO_PREC_FP32 || precision == LITHO_PREC_MIXED, "bad precision %d", precision);
  LITHO_RET(check_geom(ctx, Lx, Ly, ks->Nx, ks->Ny, ks->nk));
  LITHO_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  ImgGeom g{Lx, Ly, next_pow2(Lx), next_pow2(Ly), ks->Nx, ks->Ny, ks->nk, default_conv_n(ks->Nx, ks->Ny)};
  if (precision == LITHO_PREC_MIXED && !tc_supported(g)) {
    set_error(ctx, LITHO_ERR_UNSUPPORTED, "mixed precision needs Lx %% 32 == 0 and Nx <= 16 (Lx=%d)", Lx);
    return LITHO_ERR_UNSUPPORTED;
  }
  const size_t img = (size_t)Lx * Ly * sizeof(float);
  if (mem == LITHO_MEM_DEVICE) {
    return image_pipeline(ctx, g, batch, masks, ks, images, precision);
  }
  LITHO_RET(host_batch(ctx, g, batch, masks, ks, images, precision, img));
  LITHO_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (precision == LITHO_PREC_MIXED) LITHO_RET(tc_check_flag(ctx));
  return LITHO_OK;
}

int litho_image(litho_ctx* ctx, const float* mask, int Lx, int Ly, const float* krn_r, const float* krn_i,
                const float* scales, int nk, int Nx, int Ny, float* image, int precision, int mem) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  LITHO_ARG_CHECK(ctx, mask && krn_r && krn_i && scales && image, "null pointer");
  LITHO_RET(check_geom(ctx, Lx, Ly, Nx, Ny, nk));
  LITHO_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  const int kdim = (2 * Nx + 1) * (2 * Ny + 1);
  LITHO_RET(ctx->stage_k.ensure(ctx, (size_t)nk * kdim * sizeof(float2)));
  LITHO_RET(ctx->stage_s.ensure(ctx, (size_t)nk * sizeof(float)));
  LITHO_RET(upload_kernels(ctx, krn_r, krn_i, scales, nk, kdim, mem, ctx->stage_k.as<float2>(), ctx->stage_s.as<float>()));
  litho_kernel_set ks;
  ks.ctx = ctx;
  ks.nk = nk;
  ks.Nx = Nx;
  ks.Ny = Ny;
  ks.krn = ctx->stage_k.as<float2>();
  ks.scales = ctx->stage_s.as<float>();
  return litho_image_batch(ctx, &ks, mask, 1, Lx, Ly, image, precision, mem);
}

}  // extern "C"
