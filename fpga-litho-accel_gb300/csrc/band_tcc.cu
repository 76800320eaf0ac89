// The SOCS band of an image as the bilinear form of the rank-K TCC.
//
// calcSOCS (litho.cpp:795-1006) sums, over the K kernels, s_k |IFFT(K_k . W)|^2 on
// the conv grid; the interpolation then needs only the band |f| <= 2N of that
// intensity's spectrum.  With A_k = K_k . W (both supported on the (2Ny+1) x (2Nx+1)
// window of frequencies p),
//   band(f) = sum_k s_k sum_{p - q = f} A_k(p) conj(A_k(q))
//           = sum_{p - q = f} W(p) conj(W(q)) T(p, q),   T(p, q) = sum_k s_k K_k(p) conj(K_k(q)),
// the same quantity the grid FFTs produce divided by the grid size squared (the
// transforms are unnormalised; the grid only has to avoid aliasing, |f| <= 2N).
// T depends on the kernel set alone and is built once; per image the band is
// sum over the window's pairs (p, q) with fy >= 0 -- ~44K products at Nx = Ny = 8
// instead of K inverse 2-D FFTs, |E|^2 and one forward FFT.
//
// Work layout (band_sched.hpp).  Rows fy and 2Ny - fy pair into one task of 2Ny+2 window
// rows (fy = Ny alone has Ny+1); a task's rows may be cut into chunks whose partial bands
// go to separate groups (summed by the interpolation in order).  Within a window row, lane
// j of an image owns the p column j and walks the q columns (plus a share of the last p
// column): its p value stays in a register, every q value is one load broadcast to the
// image's lanes, and its 2Nx+1 running sums (one per q column, band column j - qx) are
// summed along the band diagonals by warp shuffles once per band row.  T is stored
// per task-chunk in the order the lanes consume it ([row][slot][lane]), so that a CTA
// holds its chunk in shared memory and every warp streams it while imaging its own
// images: 2Nx lanes per image, 32 / (2Nx) images per warp.
#include "litho_internal.cuh"
#include "band_sched.hpp"

#include <algorithm>

namespace litho {

constexpr int BT_THREADS = 256, BT_WARPS = BT_THREADS / 32;

// 16-byte asynchronous global -> shared copies (zero fill when src_bytes is 0)
__device__ __forceinline__ void cp_async16(void* dst, const void* src, int src_bytes) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// T entries of task-chunk blockIdx.x in consumption order, accumulated in FP64 over
// the kernels in order and rounded once; zero for idle slots.
__global__ void band_tab_kernel(const float2* __restrict__ krn, const float* __restrict__ scales, int nk, int Nx,
                                int Ny, int nc, float2* __restrict__ tab) {
  const BandTask d = bt_task(blockIdx.x, Nx, Ny, nc);
  const int KX = 2 * Nx + 1, KD = KX * (2 * Ny + 1), NL = 2 * Nx, NS = bt_slots(Nx);
  for (int e = threadIdx.x; e < d.size; e += blockDim.x) {
    const int j = e % NL, rest = e / NL, sl = rest % NS, rr = rest / NS;
    const int l = rr >= d.npy[0] ? 1 : 0, r = rr - (l ? d.npy[0] : 0);
    const int py0 = l ? d.py0[1] : d.py0[0], fy = l ? d.fy[1] : d.fy[0];
    int px, qx;
    double tr = 0.0, ti = 0.0;
    if (bt_slot(j, sl, Nx, &px, &qx)) {
      const int py = py0 + r, qy = py - fy;
      for (int k = 0; k < nk; ++k) {
        const float2 a = krn[(size_t)k * KD + py * KX + px], b = krn[(size_t)k * KD + qy * KX + qx];
        const double sk = scales[k];
        // a * conj(b)
        tr += sk * ((double)a.x * b.x + (double)a.y * b.y);
        ti += sk * ((double)a.y * b.x - (double)a.x * b.y);
      }
    }
    tab[d.toff + e] = make_float2((float)tr, (float)ti);
  }
}

// W[img][ky][kx] (rows of 2Nx+1, KDP entries per image, the pad zero): the window of
// the mask spectrum, summed over the window DFT's partials in a fixed order with the
// u < 0 half from Hermitian symmetry, or read from full spectrum planes.
__global__ void win_sum_kernel(const float2* __restrict__ win_part, int nparts, const float* __restrict__ mskf_r,
                               const float* __restrict__ mskf_i, int Fx, int Fy, int Nx, int Ny, int KDP, int batch,
                               float2* __restrict__ wsum) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int KX = 2 * Nx + 1, KY = 2 * Ny + 1, KD = KX * KY;
  if (idx >= KDP) return;
  // several images per thread: their partial loads are in flight together
#pragma unroll 4
  for (int img = blockIdx.y; img < batch; img += gridDim.y) {
    float2 w = make_float2(0.f, 0.f);
    if (idx < KD) {
      const int ky = idx / KX, kx = idx - ky * KX;
      const int v = ky - Ny, u = kx - Nx;
      if (mskf_r != nullptr) {
        const size_t off = (size_t)img * Fx * Fy + (size_t)(Fy / 2 + v) * Fx + (Fx / 2 + u);
        w = make_float2(mskf_r[off], mskf_i[off]);
      } else {
        const bool neg = u < 0;
        const int vv = neg ? -v : v, uu = neg ? -u : u;
        const float2* P = win_part + (size_t)img * nparts * KY * (Nx + 1) + (size_t)(vv + Ny) * (Nx + 1) + uu;
        const float2 s = sum_strided(P, (size_t)KY * (Nx + 1), nparts);
        w = make_float2(s.x, neg ? -s.y : s.y);
      }
    }
    wsum[(size_t)img * KDP + idx] = w;
  }
}

// Per-lane register staging of a warp's windows (16-byte pieces): up to PF pieces per
// lane are loaded one pass ahead; the rest of a larger window set is loaded when stored.
__device__ __forceinline__ float4 bt_window_piece(const float2* __restrict__ wsum, int ibase, int e, int h,
                                                  int batch) {
  const int si = e / h, img = ibase + si;
  if (img >= batch) return make_float4(0.f, 0.f, 0.f, 0.f);
  return *reinterpret_cast<const float4*>(wsum + (size_t)img * 2 * h + 2 * (e - si * h));
}

// acc += (a conj(b)) t
__device__ __forceinline__ void bt_term(float2 a, float2 b, float2 t, float2& acc) {
  const float ux = fmaf(a.x, b.x, a.y * b.y), uy = fmaf(a.y, b.x, -a.x * b.y);
  acc.x = fmaf(ux, t.x, fmaf(-uy, t.y, acc.x));
  acc.y = fmaf(ux, t.y, fmaf(uy, t.x, acc.y));
}

__device__ __forceinline__ float2 bt_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }

// One CTA per (task-chunk, image group): its T chunk in shared memory, each warp imaging
// 32 / (2Nx) images at a time (2Nx lanes each) from its own window copies, the next images'
// windows in flight in registers meanwhile.  Lane j owns p column j of every window row
// (band_sched.hpp): per row its p value and the shared last-column value are two loads,
// then 2Nx+3 slots of one broadcast q load, one T load and eight FP32 operations each.
// Per band row the lanes' running sums (slot s: band column j - s) are added along the
// band diagonals by shuffles within the image's lanes, in a fixed order: for the band
// column j - c of lane j, round k takes slot k + c of lane j + k (the same register in
// every lane).
template <int NXC>
__global__ void __launch_bounds__(BT_THREADS, 2) band_tcc_kernel(const float2* __restrict__ tab,
                                                                 const float2* __restrict__ wsum, int KDP, int Ny,
                                                                 int nc, int batch, float2* __restrict__ band_part) {
  constexpr int Nx = NXC, KX = 2 * Nx + 1, NL = 2 * Nx, NS = KX + 2, BW = 4 * Nx + 1, IPW = 32 / NL;
  constexpr int PF = Nx <= 8 ? 10 : 4;  // window pieces prefetched per lane
  extern __shared__ __align__(16) float2 bts[];
  const BandTask d = bt_task(blockIdx.x, Nx, Ny, nc);
  const int KY = 2 * Ny + 1;
  const int tsz = d.size;                              // even: whole 16-byte pairs
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  float2* sT = bts;                                   // [tsz]
  float2* sW = bts + tsz;                             // [warps][IPW][KDP]
  {
    const float2* src = tab + d.toff;
    for (int e = tid; e < tsz / 2; e += blockDim.x) cp_async16(sT + 2 * e, src + 2 * e, 16);
    cp_async_commit();
  }
  const bool active = lane < IPW * NL;
  const int sub = active ? lane / NL : 0, j = active ? lane - sub * NL : lane % NL;
  float4* myW = reinterpret_cast<float4*>(sW + (size_t)warp * IPW * KDP);
  const float2* W = sW + (size_t)warp * IPW * KDP + (size_t)sub * KDP;
  const int h = KDP / 2, n4 = IPW * h;
  const int istep = gridDim.y * nw * IPW;
  int ibase = (blockIdx.y * nw + warp) * IPW;
  float4 pf[PF];
#pragma unroll
  for (int k = 0; k < PF; ++k)
    pf[k] = (lane + 32 * k < n4 && ibase < batch) ? bt_window_piece(wsum, ibase, lane + 32 * k, h, batch)
                                                  : make_float4(0.f, 0.f, 0.f, 0.f);
  cp_async_wait<0>();
  __syncthreads();
  for (; ibase < batch; ibase += istep) {
    __syncwarp();  // the previous images' windows are no longer read
#pragma unroll
    for (int k = 0; k < PF; ++k)
      if (lane + 32 * k < n4) myW[lane + 32 * k] = pf[k];
    for (int e = lane + 32 * PF; e < n4; e += 32) myW[e] = bt_window_piece(wsum, ibase, e, h, batch);
    __syncwarp();
    const int inext = ibase + istep;
#pragma unroll
    for (int k = 0; k < PF; ++k)
      if (lane + 32 * k < n4 && inext < batch) pf[k] = bt_window_piece(wsum, inext, lane + 32 * k, h, batch);
    const int img = ibase + sub;
    const bool live = active && img < batch;
#pragma unroll 1
    for (int l = 0; l < d.nfy; ++l) {
      const int fy = l ? d.fy[1] : d.fy[0], np = l ? d.npy[1] : d.npy[0], py0 = l ? d.py0[1] : d.py0[0];
      float2 acc[KX];
#pragma unroll
      for (int k = 0; k < KX; ++k) acc[k] = make_float2(0.f, 0.f);
      float2 e1 = make_float2(0.f, 0.f), e2 = e1;
      const float2* tt = sT + (size_t)bt_entry(d, l, 0, 0, j, Nx);
#pragma unroll 1
      for (int r = 0; r < np; ++r, tt += NS * NL) {
        const int py = py0 + r, qy = py - fy;
        const float2* wq = W + qy * KX;
        const float2 wp = W[py * KX + j], wl = W[py * KX + 2 * Nx];
#pragma unroll
        for (int sl = 0; sl < KX; ++sl) bt_term(wp, wq[sl], tt[sl * NL], acc[sl]);
        bt_term(wl, wq[j], tt[KX * NL], e1);
        bt_term(wl, wq[2 * Nx], tt[(KX + 1) * NL], e2);  // T is zero here but for lane 0
      }
      // band column f: the sum over lanes j' of acc_j'[j' - f], plus the last column's terms
      const unsigned full = 0xffffffffu;
      const int base = lane - j;  // this image's first lane (2Nx need not be a power of two)
      auto from = [&](float2 v, int src) {
        return make_float2(__shfl_sync(full, v.x, src), __shfl_sync(full, v.y, src));
      };
      float2 vneg = acc[2 * Nx], vpos = make_float2(0.f, 0.f), vz = acc[0];
#pragma unroll
      for (int k = 1; k <= 2 * Nx; ++k) {  // f = j - 2Nx: lanes j - k, slot 2Nx - k
        const float2 v = from(acc[2 * Nx - k], j >= k ? lane - k : lane);
        if (j >= k) vneg = bt_add(vneg, v);
      }
#pragma unroll
      for (int k = 1; k < NL; ++k) {  // f = j + 1: lanes j + k, slot k - 1; f = 0 (lane 0): slot k
        const int src = j + k < NL ? lane + k : lane;
        const float2 v = from(acc[k - 1], src), w = from(acc[k], src);
        if (j + k < NL) {
          vpos = bt_add(vpos, v);
          vz = bt_add(vz, w);
        }
      }
      // (2Nx, qx) of lane qx is band column 2Nx - qx: lane j takes lane 2Nx - 1 - j's
      const float2 ex = from(e1, base + NL - 1 - j);
      if (live) {
        float2* out = band_part + (((size_t)img * nc + d.group) * KY + fy) * BW + 2 * Nx;
        out[j - 2 * Nx] = vneg;
        out[j + 1] = bt_add(vpos, ex);
        if (j == 0) out[0] = bt_add(vz, e2);
      }
    }
  }
}

// the band kernel for a support half-width 1 <= Nx <= 16 (compile-time row strides and
// register arrays)
static decltype(&band_tcc_kernel<1>) band_kernel_for(int Nx) {
  switch (Nx) {
    case 1: return band_tcc_kernel<1>;
    case 2: return band_tcc_kernel<2>;
    case 3: return band_tcc_kernel<3>;
    case 4: return band_tcc_kernel<4>;
    case 5: return band_tcc_kernel<5>;
    case 6: return band_tcc_kernel<6>;
    case 7: return band_tcc_kernel<7>;
    case 8: return band_tcc_kernel<8>;
    case 9: return band_tcc_kernel<9>;
    case 10: return band_tcc_kernel<10>;
    case 11: return band_tcc_kernel<11>;
    case 12: return band_tcc_kernel<12>;
    case 13: return band_tcc_kernel<13>;
    case 14: return band_tcc_kernel<14>;
    case 15: return band_tcc_kernel<15>;
    default: return band_tcc_kernel<16>;
  }
}

bool use_band_tcc(const litho_ctx* ctx, const litho_kernel_set* ks, int batch) {
  if (!band_tcc_available(ctx, ks)) return false;
  if (ctx->band_method == LITHO_BAND_TCC) return true;
  const int convN = default_conv_n(ks->Nx, ks->Ny);
  return band_tcc_cost_us(ks->Nx, ks->Ny, ks->band_nc, batch) <= band_fft_cost_us(convN, ks->nk, batch);
}

// Build the T table of a kernel set (krn/scales on the device) on `stream`.
int build_band_table(litho_ctx* ctx, litho_kernel_set* ks, cudaStream_t stream) {
  ks->band_nc = 0;
  const int nc = band_tcc_chunks(ks->Nx, ks->Ny);
  if (nc == 0) return LITHO_OK;  // the FFT form serves this support
  const size_t n = band_tcc_entries(ks->Nx, ks->Ny, nc);
  if (cudaMalloc(&ks->band_tab, n * sizeof(float2)) != cudaSuccess) {
    set_error(ctx, LITHO_ERR_NOMEM, "band table allocation failed");
    return LITHO_ERR_NOMEM;
  }
  band_tab_kernel<<<(ks->Ny + 1) * nc, 256, 0, stream>>>(ks->krn, ks->scales, ks->nk, ks->Nx, ks->Ny, nc,
                                                         ks->band_tab);
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  ks->band_nc = nc;
  return LITHO_OK;
}

size_t band_wsum_bytes(const ImgGeom& g, int batch) {
  const int KD = (2 * g.Nx + 1) * (2 * g.Ny + 1);
  return (size_t)batch * ((KD + 1) & ~1) * sizeof(float2);
}

// The band of every image of the plan into band_part[img][ks->band_nc][2Ny+1][4Nx+1]
// (p.ngroups must be ks->band_nc); wsum: band_wsum_bytes of workspace.
int run_band_tcc(litho_ctx* ctx, const ImgPlan& p, const WindowSrc& w, const litho_kernel_set* ks,
                 float2* wsum, float2* band_part) {
  const ImgGeom& g = p.g;
  const int nc = ks->band_nc;
  if (nc == 0 || p.ngroups != nc || g.Nx != ks->Nx || g.Ny != ks->Ny) {
    set_error(ctx, LITHO_ERR_ARG, "band table missing or plan groups %d != %d", p.ngroups, nc);
    return LITHO_ERR_ARG;
  }
  const int KD = (2 * g.Nx + 1) * (2 * g.Ny + 1), KDP = (KD + 1) & ~1;
  {
    StageScope sc(ctx, LITHO_STAGE_SOCS, 2);
    const int bx = (KDP + 127) / 128;
    // up to four images per thread (their partial loads in flight together), fewer where
    // that would leave fewer than ~4 blocks per SM
    const int sms = std::max(1, p.sms > 0 ? p.sms : ctx->sm_count);
    const int ipt = std::max(1, std::min(4, (p.batch * bx) / (4 * sms)));
    const int by = std::max(1, std::min(65535, (p.batch + ipt - 1) / ipt));
    win_sum_kernel<<<dim3(bx, by), 128, 0, ctx->stream>>>(
        w.part, w.nparts, w.mskf_r, w.mskf_i, g.Fx, g.Fy, g.Nx, g.Ny, KDP, p.batch, wsum);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
    int most = 0;
    const int ntc = (g.Ny + 1) * nc;
    for (int b = 0; b < ntc; ++b) most = std::max(most, bt_task_shape(b, g.Nx, g.Ny, nc).size);
    const int IPW = 32 / (2 * g.Nx);
    decltype(&band_tcc_kernel<1>) k = band_kernel_for(g.Nx);
    auto smem_for = [&](int nw) { return ((size_t)most + (size_t)nw * IPW * KDP) * sizeof(float2); };
    LITHO_CUDA_TRY(ctx, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_for(BT_WARPS)));
    // warps per CTA: the largest that still gives every SM a CTA (small batches take
    // smaller CTAs, so that the tasks spread over the whole GPU)
    int nw = 2;
    for (int w = BT_WARPS; w >= 2; w /= 2)
      if ((long long)ntc * ((p.batch + w * IPW - 1) / (w * IPW)) >= sms) {
        nw = w;
        break;
      }
    int per_sm = 0;
    LITHO_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 32 * nw, smem_for(nw)));
    per_sm = std::max(1, per_sm);
    const int per_pass = nw * IPW;
    const int groups = std::max(1, std::min((p.batch + per_pass - 1) / per_pass, (per_sm * sms + ntc - 1) / ntc));
    k<<<dim3(ntc, groups), 32 * nw, smem_for(nw), ctx->stream>>>(ks->band_tab, wsum, KDP, g.Ny, nc, p.batch,
                                                                 band_part);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
  }
  return LITHO_OK;
}

}  // namespace litho
