// litho_image_noalloc: mask -> aerial image without any device allocation.
//
// Who needs it.  Some callers cannot let a library call cudaMalloc/cudaFree:
// cudaMalloc and cudaFree synchronise the whole device, so a latency-critical
// inspection or OPC loop that keeps several streams busy cannot afford them;
// and a plugin embedded in a host application whose own allocator owns the
// device memory budget (a caching allocator, a fixed pool, an FPGA-style host
// that hands every DDR buffer to the accelerator as the reference's
// calc_socs_2048_hls_stream_refactored_v18 top function does) must not take
// memory behind that allocator's back.  This entry point takes its
// intermediate buffers from one fixed array compiled into the library instead.
//
// The scratch array.  g_noalloc_scratch is a file-scope __device__ array of
// LITHO_NOALLOC_SCRATCH_BYTES (6 MiB).  Every GPU that loads the library holds
// it until the process exits.  In host code its name is only a host-side
// stand-in, not a device address, so the address is looked up once per device
// with cudaGetSymbolAddress while that device is current; the first call on a
// device does this set-up, so make that first call before any stream capture.
// The looked-up address stays valid for the life of the device's context: a
// process that destroys the context between calls (cudaDeviceReset) must not
// call this entry point again on that device, since the cached address would
// then name memory of a context that no longer exists.
// All calls on a device share the array and it keeps the previous call's
// contents: every region is fully written before it is read in a call, so
// nothing has to start at zero, but calls whose work overlaps on the GPU
// (different streams, or different host threads) race on the array and must be
// serialised by the caller.
#include "litho_internal.cuh"

#include <mutex>

namespace litho {

size_t noctx_scratch_layout(const ImgPlan& p, size_t off[6]);
cudaError_t image_pipeline_noctx(cudaStream_t s, const ImgPlan& p, const float* mask, const float* krn_r,
                                 const float* krn_i, const float* scales, char* scratch, float* image);

constexpr size_t LITHO_NOALLOC_SCRATCH_BYTES = size_t(6) << 20;
constexpr int NOALLOC_MAX_L = 4096;
constexpr int NOALLOC_MAX_N = 16;
constexpr int NOALLOC_MAX_NK = 64;
constexpr int NOALLOC_MAX_PARTS = 256;
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[LITHO_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mu;
static void* g_noalloc_addr[NOALLOC_MAX_DEVICES] = {};

// Device address of g_noalloc_scratch on the current device (looked up once).
static cudaError_t noalloc_scratch(int dev, void** out) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (g_noalloc_addr[dev] == nullptr) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return cudaSuccess;
}

}  // namespace litho

using namespace litho;

extern "C" int litho_image_noalloc(const float* mask, int Lx, int Ly, const float* krn_r, const float* krn_i,
                                   const float* scales, int nk, int Nx, int Ny, float* image, void* stream) {
  if (!mask || !krn_r || !krn_i || !scales || !image) return LITHO_ERR_ARG;
  if (Lx < 2 || Ly < 2 || Lx > NOALLOC_MAX_L || Ly > NOALLOC_MAX_L) return LITHO_ERR_ARG;
  if (Nx < 0 || Ny < 0 || Nx > NOALLOC_MAX_N || Ny > NOALLOC_MAX_N) return LITHO_ERR_ARG;
  if (nk < 1 || nk > NOALLOC_MAX_NK) return LITHO_ERR_ARG;
  const int Fx = next_pow2(Lx), Fy = next_pow2(Ly);
  if (2 * Nx + 1 > Fx || 2 * Ny + 1 > Fy) return LITHO_ERR_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES) return LITHO_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return LITHO_ERR_CUDA;
  int cn = next_pow2(4 * (Nx > Ny ? Nx : Ny) + 1);
  if (cn < 32) cn = 32;
  ImgGeom g{Lx, Ly, Fx, Fy, Nx, Ny, nk, cn};
  ImgPlan p = make_plan(g, 1, sms);
  while (p.nparts() > NOALLOC_MAX_PARTS && p.colSplits > 1) --p.colSplits;
  if (p.nparts() > NOALLOC_MAX_PARTS) return LITHO_ERR_ARG;
  size_t off[6];
  if (noctx_scratch_layout(p, off) > LITHO_NOALLOC_SCRATCH_BYTES) return LITHO_ERR_ARG;
  void* scratch = nullptr;
  if (noalloc_scratch(dev, &scratch) != cudaSuccess) return LITHO_ERR_CUDA;
  const cudaError_t e = image_pipeline_noctx(static_cast<cudaStream_t>(stream), p, mask, krn_r, krn_i, scales,
                                             static_cast<char*>(scratch), image);
  return e == cudaSuccess ? LITHO_OK : LITHO_ERR_CUDA;
}
