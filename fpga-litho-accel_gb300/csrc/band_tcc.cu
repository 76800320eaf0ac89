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
// Work layout.  For a row f = (fy, fx) of the band, the pairs are, for each window
// row py in [fy, 2Ny] (q row py - fy), the diagonal px - qx = fx of the 2Nx+1
// columns: 2Nx+1 - |fx| terms.  The 4Nx+1 diagonals of one row pair split into 2Nx
// lanes of 2Nx+2 or 2Nx+3 terms each: lane j >= 1 takes fx = j then fx = j - 2Nx
// (lengths 2Nx+1-j and j+1) and one idle step; lane 0 takes fx = 2Nx, fx = -2Nx
// (one term each) and fx = 0 (2Nx+1 terms).  So every lane runs the same 2Nx+3
// column steps, each over all rows py of its fy, and its accumulator is saved and
// cleared at two lane-specific steps.  Rows fy and 2Ny - fy pair into one task of
// 2Ny+2 rows (fy = Ny alone has Ny+1); a task's rows may be cut into chunks, whose
// partial bands go to separate groups (summed by the interpolation in order).
// T is stored per task-chunk in exactly the order a lane consumes it
// ([fy of the task][column step][row][lane]), so that a CTA holds its chunk in
// shared memory and every warp streams it while imaging its own images: 2Nx lanes
// per image, 32 / (2Nx) images per warp.
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
// the kernels in order and rounded once.
__global__ void band_tab_kernel(const float2* __restrict__ krn, const float* __restrict__ scales, int nk, int Nx,
                                int Ny, int nc, float2* __restrict__ tab) {
  const BandTask d = bt_task(blockIdx.x, Nx, Ny, nc);
  const int KX = 2 * Nx + 1, KD = KX * (2 * Ny + 1), NL = 2 * Nx;
  for (int e = threadIdx.x; e < d.size; e += blockDim.x) {
    const int j = e % NL;
    int rest = e / NL;
    const int l = rest >= d.nst * d.npy[0] ? 1 : 0;
    if (l == 1) rest -= d.nst * d.npy[0];
    const int npy = l ? d.npy[1] : d.npy[0], py0 = l ? d.py0[1] : d.py0[0], fy = l ? d.fy[1] : d.fy[0];
    const int il = rest / npy, r = rest - il * npy, it = d.st0 + il;
    const BtLane s = bt_lane(j, Nx);
    int px, qx, seg;
    bt_step(s, it, &px, &qx, &seg);
    double tr = 0.0, ti = 0.0;
    if (!(seg == 3 && j > 0)) {
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

// Per-lane register staging of a warp's windows (16-byte pieces): up to BT_PF pieces per
// lane are loaded one pass ahead; the rest of a larger window set is loaded when stored.
constexpr int BT_PF = 10;

__device__ __forceinline__ float4 bt_window_piece(const float2* __restrict__ wsum, int ibase, int e, int h,
                                                  int batch) {
  const int si = e / h, img = ibase + si;
  if (img >= batch) return make_float4(0.f, 0.f, 0.f, 0.f);
  return *reinterpret_cast<const float4*>(wsum + (size_t)img * 2 * h + 2 * (e - si * h));
}

// acc += (a conj(b)) t for one row of a column step
__device__ __forceinline__ void bt_term(float2 a, float2 b, float2 t, float2& acc) {
  const float ux = fmaf(a.x, b.x, a.y * b.y), uy = fmaf(a.y, b.x, -a.x * b.y);
  acc.x = fmaf(ux, t.x, fmaf(-uy, t.y, acc.x));
  acc.y = fmaf(ux, t.y, fmaf(uy, t.x, acc.y));
}

// The n rows of one column step (p, q and T rows KXS, KXS and NLS apart; 0: the runtime
// kx, nl), even rows into e and odd rows into o: two independent FMA chains, four rows
// per step of three base pointers so that every load has an immediate offset.
template <int KXS, int NLS>
__device__ __forceinline__ void bt_rows(const float2* p, const float2* q, const float2* t, int n, int kx_rt,
                                        int nl_rt, float2& e, float2& o) {
  const int kx = KXS > 0 ? KXS : kx_rt, nl = NLS > 0 ? NLS : nl_rt;
  for (; n >= 4; n -= 4) {
    bt_term(p[0], q[0], t[0], e);
    bt_term(p[kx], q[kx], t[nl], o);
    bt_term(p[2 * kx], q[2 * kx], t[2 * nl], e);
    bt_term(p[3 * kx], q[3 * kx], t[3 * nl], o);
    p += 4 * kx;
    q += 4 * kx;
    t += 4 * nl;
  }
  if (n >= 2) {
    bt_term(p[0], q[0], t[0], e);
    bt_term(p[kx], q[kx], t[nl], o);
    p += 2 * kx;
    q += 2 * kx;
    t += 2 * nl;
  }
  if (n & 1) bt_term(p[0], q[0], t[0], e);
}

__device__ __forceinline__ float2 bt_sum(float2 e, float2 o) { return make_float2(e.x + o.x, e.y + o.y); }

// One CTA per (task-chunk, image group): its T chunk in shared memory, each warp
// imaging 32 / (2Nx) images at a time (2Nx lanes each) from its own window copies,
// the next images' windows in flight in registers meanwhile.  Every column step of a
// lane runs over all rows of both band rows of the task (two accumulator sets).
// NXC > 0 fixes Nx at compile time (row strides become immediates); 0 reads nx.
template <int NXC>
__global__ void __launch_bounds__(BT_THREADS, 2) band_tcc_kernel(const float2* __restrict__ tab,
                                                              const float2* __restrict__ wsum, int KDP, int nx,
                                                              int Ny, int nc, int batch,
                                                              float2* __restrict__ band_part) {
  extern __shared__ __align__(16) float2 bts[];
  const int Nx = NXC > 0 ? NXC : nx;
  const BandTask d = bt_task(blockIdx.x, Nx, Ny, nc);
  const int KX = 2 * Nx + 1, KY = 2 * Ny + 1, BW = 4 * Nx + 1, NL = 2 * Nx;
  const int IPW = 32 / NL;
  const int tsz = d.size;                              // even: whole 16-byte pairs
  float2* sT = bts;                                   // [tsz]
  float2* sW = bts + tsz;                             // [warps][IPW][KDP]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  {
    const float2* src = tab + d.toff;
    for (int e = tid; e < tsz / 2; e += blockDim.x) cp_async16(sT + 2 * e, src + 2 * e, 16);
    cp_async_commit();
  }
  const bool active = lane < IPW * NL;
  const int sub = active ? lane / NL : 0, j = active ? lane - sub * NL : lane % NL;
  const BtLane s = bt_lane(j, Nx);
  const int sw1 = s.len1, sw2 = s.len1 + s.len2;
  float4* myW = reinterpret_cast<float4*>(sW + (size_t)warp * IPW * KDP);
  const float2* W = sW + (size_t)warp * IPW * KDP + (size_t)sub * KDP;
  const int h = KDP / 2, n4 = IPW * h;
  const int istep = gridDim.y * nw * IPW;
  int ibase = (blockIdx.y * nw + warp) * IPW;
  float4 pf[BT_PF];
#pragma unroll
  for (int k = 0; k < BT_PF; ++k)
    pf[k] = (lane + 32 * k < n4 && ibase < batch) ? bt_window_piece(wsum, ibase, lane + 32 * k, h, batch)
                                                  : make_float4(0.f, 0.f, 0.f, 0.f);
  // task rows: l = 0 always, l = 1 for a pair
  const int fy0 = d.fy[0], np0 = d.npy[0], fy1 = d.fy[1], np1 = d.npy[1];
  const int pyA = d.py0[0], pyB = d.py0[1];
  const int st0 = d.st0, st1 = d.st0 + d.nst;
  const float2* T1 = sT + (size_t)d.nst * np0 * NL;
  cp_async_wait<0>();
  __syncthreads();
  for (; ibase < batch; ibase += istep) {
    __syncwarp();  // the previous images' windows are no longer read
#pragma unroll
    for (int k = 0; k < BT_PF; ++k)
      if (lane + 32 * k < n4) myW[lane + 32 * k] = pf[k];
    for (int e = lane + 32 * BT_PF; e < n4; e += 32) myW[e] = bt_window_piece(wsum, ibase, e, h, batch);
    __syncwarp();
    const int inext = ibase + istep;
#pragma unroll
    for (int k = 0; k < BT_PF; ++k)
      if (lane + 32 * k < n4 && inext < batch) pf[k] = bt_window_piece(wsum, inext, lane + 32 * k, h, batch);
    const int img = ibase + sub;
    const bool live = active && img < batch;
    const float2 z = make_float2(0.f, 0.f);
    float2 a0 = z, b0 = z, a1 = z, b1 = z, s10 = z, s20 = z, s11 = z, s21 = z;  // a/b: even/odd rows
    for (int it = st0; it < st1; ++it) {
      if (it == sw1) {
        s10 = bt_sum(a0, b0);
        s11 = bt_sum(a1, b1);
        a0 = b0 = a1 = b1 = z;
      }
      if (it == sw2) {
        s20 = bt_sum(a0, b0);
        s21 = bt_sum(a1, b1);
        a0 = b0 = a1 = b1 = z;
      }
      int px, qx, seg;
      bt_step(s, it, &px, &qx, &seg);
      {
        const float2* pp = W + pyA * KX + px;
        const float2* qq = W + (pyA - fy0) * KX + qx;
        bt_rows<NXC ? 2 * NXC + 1 : 0, 2 * NXC>(pp, qq, sT + (size_t)(it - st0) * np0 * NL + j, np0, KX, NL, a0, b0);
      }
      {
        const float2* pp = W + pyB * KX + px;
        const float2* qq = W + (pyB - fy1) * KX + qx;
        bt_rows<NXC ? 2 * NXC + 1 : 0, 2 * NXC>(pp, qq, T1 + (size_t)(it - st0) * np1 * NL + j, np1, KX, NL, a1, b1);
      }
    }
    // the running sums belong to the segment of the chunk's last step (segments the chunk
    // does not reach stay zero in its partial band)
    float2 s30 = z, s31 = z;
    {
      const float2 e0 = bt_sum(a0, b0), e1 = bt_sum(a1, b1);
      if (st1 <= sw1) {
        s10 = e0;
        s11 = e1;
      } else if (st1 <= sw2) {
        s20 = e0;
        s21 = e1;
      } else {
        s30 = e0;
        s31 = e1;
      }
    }
    if (live) {
      float2* out = band_part + (((size_t)img * nc + d.group) * KY + fy0) * BW + 2 * Nx;
      out[s.f1] = s10;
      out[s.f2] = s20;
      if (j == 0) out[s.f3] = s30;
      if (d.nfy == 2) {
        out = band_part + (((size_t)img * nc + d.group) * KY + fy1) * BW + 2 * Nx;
        out[s.f1] = s11;
        out[s.f2] = s21;
        if (j == 0) out[s.f3] = s31;
      }
    }
  }
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
    const int by = std::max(1, std::min(65535, (p.batch + 3) / 4));  // about four images per thread
    win_sum_kernel<<<dim3(bx, by), 128, 0, ctx->stream>>>(
        w.part, w.nparts, w.mskf_r, w.mskf_i, g.Fx, g.Fy, g.Nx, g.Ny, KDP, p.batch, wsum);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
    int most = 0;
    const int ntc = (g.Ny + 1) * nc;
    for (int b = 0; b < ntc; ++b) most = std::max(most, bt_task_shape(b, g.Nx, g.Ny, nc).size);
    const int IPW = 32 / (2 * g.Nx);
    decltype(&band_tcc_kernel<0>) k;
    switch (g.Nx) {
      case 2: k = band_tcc_kernel<2>; break;
      case 4: k = band_tcc_kernel<4>; break;
      case 8: k = band_tcc_kernel<8>; break;
      case 16: k = band_tcc_kernel<16>; break;
      default: k = band_tcc_kernel<0>; break;
    }
    auto smem_for = [&](int nw) { return ((size_t)most + (size_t)nw * IPW * KDP) * sizeof(float2); };
    LITHO_CUDA_TRY(ctx, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_for(BT_WARPS)));
    // warps per CTA: the largest that still gives every SM a CTA (small batches take
    // smaller CTAs, so that the tasks spread over the whole GPU)
    const int sms = std::max(1, p.sms > 0 ? p.sms : ctx->sm_count);
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
    k<<<dim3(ntc, groups), 32 * nw, smem_for(nw), ctx->stream>>>(ks->band_tab, wsum, KDP, g.Nx, g.Ny, nc, p.batch,
                                                                 band_part);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
  }
  return LITHO_OK;
}

}  // namespace litho
