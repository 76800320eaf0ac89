// FP32 imaging pipeline: mask -> spectrum window -> SOCS intensity band -> image.
//
// The reference computes (litho.cpp:1318-1451)
//   mskf  = fftshift(FFT2(ifftshift(pad(mask)))) / (Fx*Fy)          FT_r2c_padded
//   tmpImg = sum_k s_k |IFFT_N(embed(K_k * mskf_window))|^2          calcSOCS kernel loop
//   image = crop(roll(C2R_F(zero-pad(R2C_N(tmpImg)/N^2))))           FI + crop
// Only the (2Ny+1)x(2Nx+1) window of mskf around DC reaches the kernels, and the
// intensity is band-limited to |f| <= 2N, so this file computes exactly those
// pieces and nothing else:
//
//   win_dft_kernel : W[v][u] = 1/(FxFy) sum_{y,x} m[y][x] e^{-2 pi i (u x'/Fx + v y'/Fy)}
//                    (x' = x + (Fx-Lx)/2 - Fx/2).  A separable partial DFT: the
//                    column stage is a 128 x Lx x (2Nx+1) FP32 contraction per CTA
//                    with the mask chunks streamed through a cp.async ring in
//                    shared memory, the row stage a small complex contraction in
//                    the epilogue.  HBM: one read of the mask.
//   socs_kernel    : per kernel k, embed K_k*W in an N x N grid, 2-D inverse FFT
//                    (warp-shuffle radix-2, fft_warp.cuh), accumulate s_k|E|^2 in
//                    registers; then a forward FFT of the intensity and the
//                    |f| <= 2N band S[fy][fx] / N^2 is written out.
//   fi_rows_kernel : T[fy][X] = sum_fx S[fy][fx] e^{+2 pi i fx x'/Fx}   (fy >= 0)
//   fi_out_kernel  : image[Y][X] = T0 + 2 sum_{fy>0} Re(e^{2 pi i fy y'/Fy} T[fy][X]),
//                    a rank-(4Ny+1) FP32 contraction whose cos and sin halves give
//                    rows +y' and -y' from one set of sums, written once with
//                    16-byte streaming stores.  HBM: one write of the image.
// With C2R's Hermitian completion and the two rolls of litho.cpp:934 and
// litho.cpp:700, that is exactly FI's zero-padded interpolation followed by
// crop2DCentered (litho.cpp:164-177, 997-1001).
#include "litho_internal.cuh"
#include "fft_warp.cuh"
#include "fft_lane8.cuh"
#include "fi_mirror.hpp"
#include "tc_common.cuh"

#include <algorithm>

namespace litho {

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ int pmod(long long a, int m) {
  long long r = a % m;
  return (int)(r < 0 ? r + m : r);
}

// exp(sign * 2 pi i * m / F) for an exact integer phase m (the argument of
// sincospif is exact because F is a power of two).
__device__ __forceinline__ float2 cis_exact(long long m, int F, float sign) {
  const int r = (int)(m & (long long)(F - 1));  // F (an FFT size) is a power of two
  float s, c;
  sincospif(2.0f * (float)r / (float)F, &s, &c);
  return make_float2(c, sign * s);
}

// ---------------------------------------------------------------------------
// window DFT column twiddles: twx[x][j], j in [0, NJT):
//   j <= Nx          : cos(2 pi j x'/Fx)
//   Nx < j <= 2Nx    : -sin(2 pi (j-Nx) x'/Fx)
//   otherwise 0 (padding to a multiple of 4)
// ---------------------------------------------------------------------------
__global__ void twx_init_kernel(float* __restrict__ twx, int Lx, int Fx, int Nx, int NJT) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= Lx) return;
  const long long xp = (long long)x + (Fx - Lx) / 2 - Fx / 2;
  for (int j = 0; j < NJT; ++j) {
    float v = 0.f;
    if (j <= 2 * Nx) {
      const int u = j <= Nx ? j : j - Nx;
      long long m = ((long long)u * xp) % Fx;
      if (m < 0) m += Fx;
      double s, c;
      sincospi(2.0 * (double)m / (double)Fx, &s, &c);
      v = j <= Nx ? (float)c : (float)(-s);
    }
    twx[(size_t)x * NJT + j] = v;
  }
}

// ---------------------------------------------------------------------------
// window DFT
// ---------------------------------------------------------------------------
constexpr int WD_BM = 128;          // mask rows per CTA
constexpr int WD_BK = 32;           // mask columns per ring stage
constexpr int WD_SA = WD_BK + 4;    // staged row stride (floats): 16-byte rows, conflict-free 16-byte reads
constexpr int WD_THREADS = 256;

// ring stages: enough mask bytes in flight per SM (two CTAs of 4 x 16 KB where the
// accumulators leave room for two, else one CTA of 8)
template <int NJT>
struct WinRing {
  static constexpr int CTAS = NJT <= 20 ? 2 : 1;
  static constexpr int ST = NJT <= 20 ? 4 : 8;
  static constexpr int A_F = WD_BM * WD_SA;  // floats of a stage's mask chunk
  static constexpr int STAGE_F = A_F + WD_BK * NJT;
};

// shared memory of a window DFT launch: the ring, reused by the k-split reduction and
// the row transform at the end
template <int NJT>
static size_t win_dft_smem(int Ny) {
  const size_t ring = (size_t)WinRing<NJT>::ST * WinRing<NJT>::STAGE_F * sizeof(float);
  const size_t tree = (size_t)4 * NJT * WD_BM * sizeof(float);  // the k-split warps' sums
  const size_t rows = (size_t)NJT * (WD_BM + 4) * sizeof(float) + (size_t)(Ny + 1) * (WD_BM + 2) * sizeof(float2);
  return std::max(ring, std::max(tree, rows));
}

__device__ __forceinline__ void wd_cp16(float* dst, const float* src, bool ok) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(ok ? 16 : 0) : "memory");
}
__device__ __forceinline__ void wd_cp4(float* dst, const float* src, bool ok) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(ok ? 4 : 0) : "memory");
}

// One CTA per (row block of WD_BM rows, column split, image): the mask chunks of its
// columns stream through a ring of cp.async stages (row-major, zero-filled past the
// mask) with the chunk's column twiddles beside them; warp w multiplies columns
// 4w..4w+3 of every chunk into its 4 rows x NJT accumulators (rows lane + 32i), in
// packed f32x2 FMAs.  The eight warps' sums are then added in a fixed tree and each
// row block's row transforms summed over its rows with the row twiddles.
template <int NJT, bool VEC>
__global__ void __launch_bounds__(WD_THREADS, WinRing<NJT>::CTAS) win_dft_kernel(
    const float* __restrict__ masks, int Lx, int Ly, int Fx, int Fy, int Nx, int Ny, const float* __restrict__ twx,
    float2* __restrict__ win_part, int part_stride) {
  using RG = WinRing<NJT>;
  constexpr int ST = RG::ST;
  extern __shared__ __align__(16) float sm[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int rb = blockIdx.x, cs = blockIdx.y, img = blockIdx.z;
  const int colSplits = gridDim.y;
  const int nparts = gridDim.x * gridDim.y;
  const int part = rb * colSplits + cs;
  const int y0 = rb * WD_BM;
  const int nch = (Lx + WD_BK - 1) / WD_BK;
  const int ch0 = (int)((long long)nch * cs / colSplits);
  const int ch1 = (int)((long long)nch * (cs + 1) / colSplits);
  const float* M = masks + (size_t)img * Lx * Ly;
  auto sA = [&](int st) { return sm + (size_t)st * RG::STAGE_F; };        // [WD_BM][WD_SA]
  auto sB = [&](int st) { return sm + (size_t)st * RG::STAGE_F + RG::A_F; };  // [WD_BK][NJT]

  // chunk ch into ring slot st: 128 rows x 32 columns (four 16-byte pieces a thread) and
  // the chunk's twiddle rows (NJT / 4 pieces per column)
  auto issue = [&](int ch, int st) {
    const int x0 = ch * WD_BK;
    float* a = sA(st);
#pragma unroll
    for (int i = 0; i < WD_BM * WD_BK / 4 / WD_THREADS; ++i) {
      const int idx = tid + WD_THREADS * i, row = idx >> 3, c4 = (idx & 7) * 4;
      const int y = y0 + row, x = x0 + c4;
      const bool rok = y < Ly;
      const float* src = M + (size_t)(rok ? y : 0) * Lx;
      float* dst = a + row * WD_SA + c4;
      if (VEC) {
        wd_cp16(dst, src + (rok && x < Lx ? x : 0), rok && x < Lx);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) wd_cp4(dst + e, src + (rok && x + e < Lx ? x + e : 0), rok && x + e < Lx);
      }
    }
    constexpr int Q = NJT / 4;
    float* b = sB(st);
    for (int idx = tid; idx < WD_BK * Q; idx += WD_THREADS) {
      const int kr = idx / Q, c = idx - kr * Q, x = x0 + kr;
      wd_cp16(b + 4 * idx, twx + (size_t)(x < Lx ? x : 0) * NJT + 4 * c, x < Lx);
    }
  };

  // accumulators in column pairs: one packed (f32x2) FMA updates two twiddle columns, each
  // lane rounding as fmaf does
  float2 acc2[4][NJT / 2];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < NJT / 2; ++j) acc2[i][j] = make_float2(0.f, 0.f);
  auto acc = [&](int i, int j) -> float& { return (j & 1) ? acc2[i][j >> 1].y : acc2[i][j >> 1].x; };

  // one commit group per ring step (empty past the last chunk), so that waiting for all
  // but the newest ST - 2 groups means the current stage has landed
#pragma unroll
  for (int k = 0; k < ST - 1; ++k) {
    if (ch0 + k < ch1) issue(ch0 + k, k);
    asm volatile("cp.async.commit_group;" ::: "memory");
  }
  for (int ch = ch0; ch < ch1; ++ch) {
    const int it = ch - ch0, st = it % ST;
    asm volatile("cp.async.wait_group %0;" ::"n"(ST - 2) : "memory");
    __syncthreads();  // the stage is visible to all; every warp is done with the previous one
    if (ch + ST - 1 < ch1) issue(ch + ST - 1, (it + ST - 1) % ST);
    asm volatile("cp.async.commit_group;" ::: "memory");
    const float* a = sA(st) + lane * WD_SA + 4 * warp;
    float4 av[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) av[i] = *reinterpret_cast<const float4*>(a + 32 * i * WD_SA);
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const float4* b4 = reinterpret_cast<const float4*>(sB(st) + (4 * warp + kk) * NJT);
      float2 ai[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float v = kk == 0 ? av[i].x : kk == 1 ? av[i].y : kk == 2 ? av[i].z : av[i].w;
        ai[i] = make_float2(v, v);
      }
#pragma unroll
      for (int c = 0; c < NJT / 4; ++c) {
        const float4 b = b4[c];
        const float2 blo = make_float2(b.x, b.y), bhi = make_float2(b.z, b.w);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          acc2[i][2 * c] = __ffma2_rn(ai[i], blo, acc2[i][2 * c]);
          acc2[i][2 * c + 1] = __ffma2_rn(ai[i], bhi, acc2[i][2 * c + 1]);
        }
      }
    }
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  __syncthreads();

  // tree reduction of the 8 k-split warps: red[w][j][r], r fastest (conflict free)
  float* red = sm;
  for (int s = 4; s >= 1; s >>= 1) {
    if (warp >= s && warp < 2 * s) {
      float* dst = red + (size_t)(warp - s) * NJT * WD_BM;
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < NJT; ++j) dst[j * WD_BM + lane + 32 * i] = acc(i, j);
    }
    __syncthreads();
    if (warp < s) {
      const float* src = red + (size_t)warp * NJT * WD_BM;
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < NJT; ++j) acc(i, j) += src[j * WD_BM + lane + 32 * i];
    }
    __syncthreads();
  }
  // row transforms of this block and the row twiddles, rows padded (132 floats, 130 float2)
  // so that the threads of a warp (different u, |v|) read different banks
  constexpr int RS = WD_BM + 4, RT = WD_BM + 2;
  float* sR = red;  // [NJT][RS]
  if (warp == 0) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < NJT; ++j) sR[j * RS + lane + 32 * i] = acc(i, j);
  }
  // row twiddles e^{-2 pi i v y'/Fy}, v = 0..Ny
  float2* sRT = reinterpret_cast<float2*>(sm + (size_t)NJT * RS);  // [Ny+1][RT]
  const int oyc = (Fy - Ly) / 2 - Fy / 2;
  for (int idx = tid; idx < (Ny + 1) * WD_BM; idx += WD_THREADS) {
    const int v = idx / WD_BM, r = idx - v * WD_BM;
    sRT[v * RT + r] = cis_exact((long long)v * (y0 + r + oyc), Fy, -1.f);
  }
  __syncthreads();

  const int KY = 2 * Ny + 1, NU = Nx + 1;
  const float scale = 1.0f / ((float)Fx * (float)Fy);
  // part_stride > 0: images of this launch sit in a larger per-class array with
  // that many parts per image (the unused parts are zero)
  const int nps = part_stride > 0 ? part_stride : nparts;
  float2* out = win_part + ((size_t)img * nps + part) * KY * NU;
  for (int o = tid; o < KY * NU; o += WD_THREADS) {
    const int vi = o / NU, u = o - vi * NU;
    const int v = vi - Ny;
    const int av = v < 0 ? -v : v;
    const float ts = v < 0 ? -1.f : 1.f;
    const float* rc = sR + u * RS;
    const float* rs = sR + (Nx + u) * RS;
    const float2* rt = sRT + av * RT;
    float re = 0.f, im = 0.f;
    if (u == 0) {
#pragma unroll 4
      for (int r = 0; r < WD_BM; ++r) {
        const float2 t = rt[r];
        re = fmaf(rc[r], t.x, re);
        im = fmaf(rc[r], ts * t.y, im);
      }
    } else {
#pragma unroll 4
      for (int r = 0; r < WD_BM; ++r) {
        const float2 t = rt[r];
        const float ty = ts * t.y;
        re = fmaf(rc[r], t.x, fmaf(-rs[r], ty, re));
        im = fmaf(rc[r], ty, fmaf(rs[r], t.x, im));
      }
    }
    out[o] = make_float2(re * scale, im * scale);
  }
}

// ---------------------------------------------------------------------------
// SOCS: K inverse FFTs on the N x N conv grid, intensity accumulation in
// registers, forward FFT of the intensity, band output.  socs_kernel<N> uses the
// warp-shuffle transforms of fft_warp.cuh and serves the 32 x 32 grid; the 64 and
// 128 grids have their own kernels on the lane-group transforms of fft_lane8.cuh.
// ---------------------------------------------------------------------------
constexpr int SOCS_THREADS = 256;

template <int N>
__global__ void __launch_bounds__(SOCS_THREADS) socs_kernel(
    const float2* __restrict__ win_part, int nparts, const float* __restrict__ mskf_r,
    const float* __restrict__ mskf_i, int Fx, int Fy, int Nx, int Ny, const float2* __restrict__ krn,
    const float* __restrict__ scales, int nk, int kpg, float2* __restrict__ band_part,
    float* __restrict__ tmpImgp) {
  constexpr int J = N / 32, SG = N + 1, CPW = N / 8;
  const int KX = 2 * Nx + 1, KY = 2 * Ny + 1, KD = KX * KY;
  extern __shared__ __align__(16) float2 sg[];
  // only the KY embedded rows of the conv grid are ever non-zero, and the forward
  // pass keeps the rows fy <= 2Ny (= KY rows): a compact [KY][SG] grid
  float2* grid = sg;             // [KY][SG]
  float2* tw = grid + KY * SG;   // [N/2]
  float2* win = tw + N / 2;      // [KY][KX]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = blockIdx.x, img = blockIdx.y, ngroups = gridDim.x;

  for (int e = tid; e < N / 2; e += SOCS_THREADS) {
    float s, c;
    sincospif(2.0f * (float)e / (float)N, &s, &c);
    tw[e] = make_float2(c, -s);
  }
  for (int idx = tid; idx < KD; idx += SOCS_THREADS) {
    const int ky = idx / KX, kx = idx - ky * KX;
    const int v = ky - Ny, u = kx - Nx;
    float2 w;
    if (mskf_r != nullptr) {
      const size_t off = (size_t)img * Fx * Fy + (size_t)(Fy / 2 + v) * Fx + (Fx / 2 + u);
      w = make_float2(mskf_r[off], mskf_i[off]);
    } else {
      const bool neg = u < 0;
      const int vv = neg ? -v : v, uu = neg ? -u : u;
      const float2* P = win_part + (size_t)img * nparts * KY * (Nx + 1) + (size_t)(vv + Ny) * (Nx + 1) + uu;
      const float2 t = sum_strided(P, (size_t)KY * (Nx + 1), nparts);
      w = make_float2(t.x, neg ? -t.y : t.y);
    }
    win[idx] = w;
  }
  __syncthreads();

  const int ex = (N - KX) / 2, ey = (N - KY) / 2;
  float acc[CPW][J];
#pragma unroll
  for (int m = 0; m < CPW; ++m)
#pragma unroll
    for (int j = 0; j < J; ++j) acc[m][j] = 0.f;

  const int k0 = g * kpg, k1 = min(nk, k0 + kpg);
  for (int k = k0; k < k1; ++k) {
    const float2* K = krn + (size_t)k * KD;
    const float lam = scales[k];
    for (int ky = warp; ky < KY; ky += 8) {
      float2 x[J];
#pragma unroll
      for (int j = 0; j < J; ++j) {
        const int kx = lane + 32 * j - ex;
        x[j] = (kx >= 0 && kx < KX) ? cmul(K[ky * KX + kx], win[ky * KX + kx]) : make_float2(0.f, 0.f);
      }
      warp_fft_dif<N, true>(x, tw, lane);
#pragma unroll
      for (int j = 0; j < J; ++j) grid[ky * SG + lane + 32 * j] = x[j];
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < CPW; ++m) {
      const int c = warp + 8 * m;
      float2 x[J];
#pragma unroll
      for (int j = 0; j < J; ++j) {
        const int y = lane + 32 * j;  // rows outside the embedded band are zero
        x[j] = (unsigned)(y - ey) < (unsigned)KY ? grid[(y - ey) * SG + c] : make_float2(0.f, 0.f);
      }
      warp_fft_dif<N, true>(x, tw, lane);
#pragma unroll
      for (int j = 0; j < J; ++j) acc[m][j] = fmaf(lam, fmaf(x[j].x, x[j].x, x[j].y * x[j].y), acc[m][j]);
    }
    __syncthreads();
  }

  if (tmpImgp != nullptr) {
    // litho.cpp:934 myShift(tmpImg -> tmpImgp, fftshift); positions are bit-reversed
    float* T = tmpImgp + (size_t)img * N * N;
#pragma unroll
    for (int m = 0; m < CPW; ++m) {
      const int xs = bitrev<N>(warp + 8 * m);
#pragma unroll
      for (int j = 0; j < J; ++j) {
        const int ys = bitrev<N>(lane + 32 * j);
        T[((ys + N / 2) & (N - 1)) * N + ((xs + N / 2) & (N - 1))] = acc[m][j];
      }
    }
  }

  // forward transform of the intensity: columns (DIT, bit-reversed in -> natural out)
#pragma unroll
  for (int m = 0; m < CPW; ++m) {
    const int c = warp + 8 * m;
    float2 x[J];
#pragma unroll
    for (int j = 0; j < J; ++j) x[j] = make_float2(acc[m][j], 0.f);
    warp_fft_dit<N, false>(x, tw, lane);
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const int fy = lane + 32 * j;
      if (fy <= 2 * Ny) grid[fy * SG + c] = x[j];
    }
  }
  __syncthreads();
  const int BW = 4 * Nx + 1;
  const float inv = 1.0f / ((float)N * (float)N);
  float2* band = band_part + ((size_t)img * ngroups + g) * KY * BW;
  for (int fy = warp; fy <= 2 * Ny; fy += 8) {
    float2 x[J];
#pragma unroll
    for (int j = 0; j < J; ++j) x[j] = grid[fy * SG + lane + 32 * j];
    warp_fft_dit<N, false>(x, tw, lane);
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const int fx = lane + 32 * j;
      int d = 1 << 30;
      if (fx <= 2 * Nx) d = fx;
      else if (fx >= N - 2 * Nx) d = fx - N;
      if (d != (1 << 30)) band[fy * BW + d + 2 * Nx] = cscale(x[j], inv);
    }
  }
}

// SOCS on the 64 x 64 conv grid with the eight-lane 64-point FFTs of
// fft_lane8.cuh: four transforms per warp, natural order throughout.  Same
// arguments, grid and output as socs_kernel<64>.
//   rows     : row ky = 8 q + warp of the embedded kernel * window product
//              (q = lane group); 2Ny + 1 <= 31 rows is one round
//   columns  : column c = warp + 8 (q + 4 m), m = 0, 1; only the embedded rows
//              [ey, ey + 2Ny] are read (the others are zero), so the grid is
//              never cleared; |E|^2 accumulates in registers at (t + 8 k2, c)
//   intensity: forward column transforms of the real intensity, rows fy <= 2Ny
//              kept, then forward row transforms of those rows -> band
// |E|^2 does not depend on where the kernel sits in the grid (a shift is a
// unimodular phase on E); the embedding is the centred one of socs_kernel.
// ---------------------------------------------------------------------------
constexpr int S64_SG = 65;  // grid row stride (float2): columns of a warp's groups 16 banks apart

size_t socs64_smem_bytes(int KD) {
  return ((size_t)64 * S64_SG + 32 + (size_t)(SOCS_THREADS / 32) * 4 * L8_SCR + KD) * sizeof(float2);
}

__global__ void __launch_bounds__(SOCS_THREADS) socs64_kernel(
    const float2* __restrict__ win_part, int nparts, const float* __restrict__ mskf_r,
    const float* __restrict__ mskf_i, int Fx, int Fy, int Nx, int Ny, const float2* __restrict__ krn,
    const float* __restrict__ scales, int nk, int kpg, float2* __restrict__ band_part,
    float* __restrict__ tmpImgp) {
  constexpr int N = 64, SG = S64_SG, NW = SOCS_THREADS / 32;
  extern __shared__ __align__(16) float2 sg[];
  float2* grid = sg;                  // [N][SG]
  float2* tw = grid + N * SG;         // [N/2]
  float2* scr = tw + N / 2;           // [NW][4][L8_SCR]
  float2* win = scr + NW * 4 * L8_SCR;  // [KY][KX]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int q = lane >> 3, t = lane & 7;
  float2* my_scr = scr + (warp * 4 + q) * L8_SCR;
  const int g = blockIdx.x, img = blockIdx.y, ngroups = gridDim.x;
  const int KX = 2 * Nx + 1, KY = 2 * Ny + 1, KD = KX * KY;

  for (int e = tid; e < N / 2; e += SOCS_THREADS) {
    float s, c;
    sincospif(2.0f * (float)e / (float)N, &s, &c);
    tw[e] = make_float2(c, -s);
  }
  for (int idx = tid; idx < KD; idx += SOCS_THREADS) {
    const int ky = idx / KX, kx = idx - ky * KX;
    const int v = ky - Ny, u = kx - Nx;
    float2 w;
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
    win[idx] = w;
  }
  __syncthreads();
  float2 w64[8];
  lane8_twiddles(w64, tw, t);

  const int ex = (N - KX) / 2, ey = (N - KY) / 2;
  float acc[2][8];
#pragma unroll
  for (int m = 0; m < 2; ++m)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[m][j] = 0.f;

  const int k0 = g * kpg, k1 = min(nk, k0 + kpg);
  for (int k = k0; k < k1; ++k) {
    const float2* K = krn + (size_t)k * KD;
    const float lam = scales[k];
    {
      const int ky = 8 * q + warp;
      const bool act = ky < KY;
      float2 x[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const int kx = t + 8 * r - ex;
        x[r] = (act && kx >= 0 && kx < KX) ? cmul(K[ky * KX + kx], win[ky * KX + kx]) : make_float2(0.f, 0.f);
      }
      fft64_lane8<true>(x, w64, my_scr, t);
      if (act) {
#pragma unroll
        for (int j = 0; j < 8; ++j) grid[(ey + ky) * SG + t + 8 * j] = x[j];
      }
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      const int c = warp + 8 * (q + 4 * m);
      float2 x[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const int y = t + 8 * r;
        x[r] = (unsigned)(y - ey) < (unsigned)KY ? grid[y * SG + c] : make_float2(0.f, 0.f);
      }
      fft64_lane8<true>(x, w64, my_scr, t);
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[m][j] = fmaf(lam, fmaf(x[j].x, x[j].x, x[j].y * x[j].y), acc[m][j]);
    }
    __syncthreads();
  }

  if (tmpImgp != nullptr) {
    // litho.cpp:934 myShift(tmpImg -> tmpImgp, fftshift)
    float* T = tmpImgp + (size_t)img * N * N;
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      const int c = warp + 8 * (q + 4 * m);
#pragma unroll
      for (int j = 0; j < 8; ++j) T[((t + 8 * j + N / 2) & (N - 1)) * N + ((c + N / 2) & (N - 1))] = acc[m][j];
    }
  }

  // forward transform of the intensity: columns, then the rows fy <= 2Ny
#pragma unroll
  for (int m = 0; m < 2; ++m) {
    const int c = warp + 8 * (q + 4 * m);
    float2 x[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) x[r] = make_float2(acc[m][r], 0.f);
    fft64_lane8<false>(x, w64, my_scr, t);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int fy = t + 8 * j;
      if (fy <= 2 * Ny) grid[fy * SG + c] = x[j];
    }
  }
  __syncthreads();
  const int BW = 4 * Nx + 1;
  const float inv = 1.0f / ((float)N * (float)N);
  float2* band = band_part + ((size_t)img * ngroups + g) * KY * BW;
  {
    const int fy = 8 * q + warp;
    const bool act = fy <= 2 * Ny;
    float2 x[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) x[r] = act ? grid[fy * SG + t + 8 * r] : make_float2(0.f, 0.f);
    fft64_lane8<false>(x, w64, my_scr, t);
    if (act) {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int fx = t + 8 * j;
        int d = 1 << 30;
        if (fx <= 2 * Nx) d = fx;
        else if (fx >= N - 2 * Nx) d = fx - N;
        if (d != (1 << 30)) band[fy * BW + d + 2 * Nx] = cscale(x[j], inv);
      }
    }
  }
}

// SOCS on the 128 x 128 conv grid with the sixteen-lane 128-point FFTs of
// fft_lane8.cuh (two transforms per warp), 512 threads so that each lane keeps
// four columns' intensities in registers.  Same arguments, grid and output as
// socs_kernel<128>.  Lane (t, h, slot): t = lane & 7, h = (lane >> 3) & 1,
// slot = lane >> 4; transform slot sl = 16 slot + warp of a round (32 per round).
//   rows     : row ky = 32 r + sl of the embedded product, read at columns
//              t + 8i + 64h (inverse, DIF) and stored at columns 2t + h + 16i
//   columns  : column c = 32 m + sl, m = 0..3, read at rows t + 8i + 64h of the
//              compact grid (only the 2Ny + 1 embedded rows exist); |E|^2 lands
//              at rows 2t + h + 16i
//   intensity: forward column transforms (DIT) take that layout and give
//              fy = t + 8i + 64h, rows fy <= 2Ny kept; forward row transforms read
//              columns 2t + h + 16i and give fx = t + 8i + 64h -> band
// ---------------------------------------------------------------------------
constexpr int S128_SG = 129;       // compact grid row stride (float2)
constexpr int S128_THREADS = 512;

size_t socs128_smem_bytes(int KY, int KD) {
  return ((size_t)KY * S128_SG + 64 + 32 + (size_t)(S128_THREADS / 32) * 4 * L8_SCR + KD) * sizeof(float2);
}

__global__ void __launch_bounds__(S128_THREADS) socs128_kernel(
    const float2* __restrict__ win_part, int nparts, const float* __restrict__ mskf_r,
    const float* __restrict__ mskf_i, int Fx, int Fy, int Nx, int Ny, const float2* __restrict__ krn,
    const float* __restrict__ scales, int nk, int kpg, float2* __restrict__ band_part,
    float* __restrict__ tmpImgp) {
  constexpr int N = 128, SG = S128_SG, NW = S128_THREADS / 32;
  const int KX = 2 * Nx + 1, KY = 2 * Ny + 1, KD = KX * KY;
  extern __shared__ __align__(16) float2 sg[];
  float2* grid = sg;                     // [KY][SG]
  float2* tw128 = grid + KY * SG;        // [64]
  float2* tw64 = tw128 + 64;             // [32]
  float2* scr = tw64 + 32;               // [NW][4][L8_SCR]
  float2* win = scr + NW * 4 * L8_SCR;   // [KY][KX]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int t = lane & 7, h = (lane >> 3) & 1, sl = 16 * (lane >> 4) + warp;
  float2* my_scr = scr + (warp * 4 + (lane >> 3)) * L8_SCR;
  const int g = blockIdx.x, img = blockIdx.y, ngroups = gridDim.x;

  for (int e = tid; e < 64; e += S128_THREADS) {
    float sn, cs;
    sincospif((float)e / 64.0f, &sn, &cs);  // W128^e = exp(-2 pi i e / 128)
    tw128[e] = make_float2(cs, -sn);
    if (e < 32) {
      sincospif((float)e / 32.0f, &sn, &cs);
      tw64[e] = make_float2(cs, -sn);
    }
  }
  for (int idx = tid; idx < KD; idx += S128_THREADS) {
    const int ky = idx / KX, kx = idx - ky * KX;
    const int v = ky - Ny, u = kx - Nx;
    float2 w;
    if (mskf_r != nullptr) {
      const size_t off = (size_t)img * Fx * Fy + (size_t)(Fy / 2 + v) * Fx + (Fx / 2 + u);
      w = make_float2(mskf_r[off], mskf_i[off]);
    } else {
      const bool neg = u < 0;
      const int vv = neg ? -v : v, uu = neg ? -u : u;
      const float2* P = win_part + (size_t)img * nparts * KY * (Nx + 1) + (size_t)(vv + Ny) * (Nx + 1) + uu;
      const float2 sm = sum_strided(P, (size_t)KY * (Nx + 1), nparts);
      w = make_float2(sm.x, neg ? -sm.y : sm.y);
    }
    win[idx] = w;
  }
  __syncthreads();
  float2 w64[8];
  lane8_twiddles(w64, tw64, t);

  const int ex = (N - KX) / 2, ey = (N - KY) / 2;
  float acc[4][8];
#pragma unroll
  for (int m = 0; m < 4; ++m)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[m][j] = 0.f;

  const int k0 = g * kpg, k1 = min(nk, k0 + kpg);
  for (int k = k0; k < k1; ++k) {
    const float2* K = krn + (size_t)k * KD;
    const float lam = scales[k];
    for (int r0 = 0; r0 < KY; r0 += 32) {  // uniform bound: every lane takes every round
      const int ky = r0 + sl;
      const bool act = ky < KY;
      float2 x[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int kx = t + 8 * i + 64 * h - ex;
        x[i] = (act && kx >= 0 && kx < KX) ? cmul(K[ky * KX + kx], win[ky * KX + kx]) : make_float2(0.f, 0.f);
      }
      fft128_inv_dif(x, w64, tw128, my_scr, t, h);
      if (act) {
#pragma unroll
        for (int i = 0; i < 8; ++i) grid[ky * SG + 2 * t + h + 16 * i] = x[i];
      }
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int c = 32 * m + sl;
      float2 x[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int y = t + 8 * i + 64 * h;
        x[i] = (unsigned)(y - ey) < (unsigned)KY ? grid[(y - ey) * SG + c] : make_float2(0.f, 0.f);
      }
      fft128_inv_dif(x, w64, tw128, my_scr, t, h);
#pragma unroll
      for (int i = 0; i < 8; ++i) acc[m][i] = fmaf(lam, fmaf(x[i].x, x[i].x, x[i].y * x[i].y), acc[m][i]);
    }
    __syncthreads();
  }

  if (tmpImgp != nullptr) {
    // litho.cpp:934 myShift(tmpImg -> tmpImgp, fftshift)
    float* T = tmpImgp + (size_t)img * N * N;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int c = 32 * m + sl;
#pragma unroll
      for (int i = 0; i < 8; ++i)
        T[((2 * t + h + 16 * i + N / 2) & (N - 1)) * N + ((c + N / 2) & (N - 1))] = acc[m][i];
    }
  }

  // forward transform of the intensity: columns, then the rows fy <= 2Ny
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const int c = 32 * m + sl;
    float2 x[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = make_float2(acc[m][i], 0.f);
    fft128_fwd_dit(x, w64, tw128, my_scr, t, h);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int fy = t + 8 * i + 64 * h;
      if (fy <= 2 * Ny) grid[fy * SG + c] = x[i];
    }
  }
  __syncthreads();
  const int BW = 4 * Nx + 1;
  const float inv = 1.0f / ((float)N * (float)N);
  float2* band = band_part + ((size_t)img * ngroups + g) * KY * BW;
  for (int r0 = 0; r0 < KY; r0 += 32) {
    const int fy = r0 + sl;
    const bool act = fy <= 2 * Ny;
    float2 x[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = act ? grid[fy * SG + 2 * t + h + 16 * i] : make_float2(0.f, 0.f);
    fft128_fwd_dit(x, w64, tw128, my_scr, t, h);
    if (act) {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int fx = t + 8 * i + 64 * h;
        int d = 1 << 30;
        if (fx <= 2 * Nx) d = fx;
        else if (fx >= N - 2 * Nx) d = fx - N;
        if (d != (1 << 30)) band[fy * BW + d + 2 * Nx] = cscale(x[i], inv);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// FI, step 1: T[fy][X] = sum_fx S[fy][fx] e^{+2 pi i fx x'/Fx} for fy = 0..2Ny
// (T[-fy] = conj(T[fy]) because the intensity is real), x' = X + (Fx-Lx)/2 - Fx/2.
// The band, summed over its kernel-group partials in a fixed order, sits in shared
// memory pre-combined as C[fy][d] = (Re(p+q), -Im(p-q), Im(p+q), Re(p-q)) for
// p = S[fy][d], q = S[fy][-d].  With t = e^{+2 pi i d x'/Fx},
//   T(x') = S0 + U + V,  T(-x') = S0 + U - V,
//   U = sum_{d>0} (p+q) Re t,  V = sum_{d>0} i (p-q) Im t,
// so one thread serves a column with x' < 0 and its mirror -x': its packed
// (f32x2) FMAs keep the cos and sin halves apart, and one broadcast shared load
// and two packed FMAs per (fy, d) give both columns.  The columns with x' < 0
// are X in [0, nb), nb = Fx/2 - (Fx-Lx)/2; the mirror of X is 2nb - X when that
// lies inside the image; the column x' = 0 (X = nb) is S0 + sum_{d>0} (p+q) and
// is summed by one warp of the first column block.  A CTA keeps its columns'
// twiddles in registers and walks the images blockIdx.y, blockIdx.y + gridDim.y, ...
// Two output layouts:
//   plain  tm[img][r][X]: r = 0 Re T0, 1..2Ny Re T, 2Ny+1..4Ny Im T (fi_out_kernel)
//   K-major (tensor-core FI) t0[img][X] = Re T0 and hi/lo TF32 splits of
//          tm[img][X][KP]: r = fy-1 Re T, 2Ny+fy-1 Im T, zero to KP
// ---------------------------------------------------------------------------
constexpr int FR_THREADS = 256, FR_COLS = 128, FR_ROWS = 2 * FR_COLS + 1;  // column, mirror, x' = 0

template <int MAXD, bool KMAJ, int KPC>
__global__ void __launch_bounds__(FR_THREADS) fi_rows_kernel(const float2* __restrict__ band_part, int ngroups,
                                                             const float2* __restrict__ twF, int Lx, int Fx,
                                                             int Nx, int Ny, int kp_rt, int batch, int raw_n,
                                                             float* __restrict__ tm, float* __restrict__ tmh,
                                                             float* __restrict__ tml, float* __restrict__ t0) {
  extern __shared__ __align__(16) float4 frs[];
  const int KP = KPC > 0 ? KPC : kp_rt;  // K-major row width (compile time where known)
  const int BH = 2 * Ny + 1, BW = 4 * Nx + 1, ND = 2 * Nx + 1;
  float4* sC = frs;                                       // [BH][MAXD]
  float* sO = reinterpret_cast<float*>(sC + BH * MAXD);  // K-major: [FR_ROWS][KP + 1]
  const int tid = threadIdx.x, xl = tid & (FR_COLS - 1), grp = tid / FR_COLS;
  const int nb = Fx / 2 - (Fx - Lx) / 2, M = 2 * nb;
  const int X0 = blockIdx.x * FR_COLS, X = X0 + xl, Xm = M - X;
  const bool live = X < nb, mlive = live && Xm < Lx;
  const bool xtra = blockIdx.x == 0 && nb < Lx;  // this block adds the column x' = 0
  float2 tw[MAXD];
#pragma unroll
  for (int d = 1; d < MAXD; ++d)
    tw[d] = (d < ND && live) ? (twF != nullptr ? twF[(size_t)d * Lx + X] : cis_exact((long long)d * (X - nb), Fx, 1.f))
                             : make_float2(0.f, 0.f);
  if (KMAJ)  // the K padding columns stay zero for every image
    for (int idx = tid; idx < FR_ROWS * (KP - 4 * Ny); idx += FR_THREADS) {
      const int c = idx / (KP - 4 * Ny), r = 4 * Ny + idx % (KP - 4 * Ny);
      sO[c * (KP + 1) + r] = 0.f;
    }
  const int fy0 = grp == 0 ? 0 : Ny + 1, fy1 = grp == 0 ? Ny + 1 : BH;
  const size_t pst = (size_t)BH * BW;
  // rows of this block in the K-major store: its columns X0.., their mirrors (ascending
  // X = Mlo + j for slots FR_COLS + nbase - 1 - j) and, in the first block, x' = 0
  const int nbase = max(0, min(FR_COLS, nb - X0));
  const int imin = max(0, M - X0 - Lx + 1);
  const int nmir = max(0, nbase - imin), Mlo = M - X0 - nbase + 1;
  const int nrows = nbase + nmir + (xtra ? 1 : 0);
  // the next image's band partials stream into shared memory (8-byte cp.async) while
  // this image is computed, when the two buffers fit (raw_n > 0)
  const int RAWN = ngroups * BH * BW;
  float2* raw = raw_n > 0 ? reinterpret_cast<float2*>(
                                (reinterpret_cast<uintptr_t>(sO + (KMAJ ? FR_ROWS * (KP + 1) : 0)) + 15) & ~uintptr_t(15))
                          : nullptr;
  auto fetch = [&](int im, float2* dst) {
    const float2* src = band_part + (size_t)im * RAWN;
    for (int e = tid; e < RAWN; e += FR_THREADS) {
      const unsigned da = (unsigned)__cvta_generic_to_shared(dst + e);
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(da), "l"(src + e) : "memory");
    }
  };
  if (raw != nullptr) {
    if ((int)blockIdx.y < batch) fetch(blockIdx.y, raw);
    asm volatile("cp.async.commit_group;" ::: "memory");
  }
  for (int img = blockIdx.y, k = 0; img < batch; img += gridDim.y, ++k) {
    if (raw != nullptr) {
      if (img + (int)gridDim.y < batch) fetch(img + gridDim.y, raw + (size_t)((k + 1) & 1) * RAWN);
      asm volatile("cp.async.commit_group;" ::: "memory");
      asm volatile("cp.async.wait_group 1;" ::: "memory");  // this image's partials have landed
    }
    __syncthreads();  // the previous image is out of sC and sO (and this one's partials are visible)
    const float2* B = raw != nullptr ? raw + (size_t)(k & 1) * RAWN : band_part + (size_t)img * RAWN;
    for (int idx = tid; idx < BH * MAXD; idx += FR_THREADS) {
      const int fy = idx / MAXD, d = idx - fy * MAXD;  // MAXD: a compile-time divisor
      if (d >= ND) continue;
      const float2* S = B + fy * BW + 2 * Nx;
      float2 pv = S[d], qv = S[-d];
      for (int gi = 1; gi < ngroups; ++gi) {  // the kernel groups' partials, in order
        const float2 a = S[gi * pst + d], b = S[gi * pst - d];
        pv.x += a.x;
        pv.y += a.y;
        qv.x += b.x;
        qv.y += b.y;
      }
      if (d == 0) {
        sC[fy * MAXD] = make_float4(pv.x, pv.y, 0.f, 0.f);
      } else {
        sC[fy * MAXD + d] = make_float4(pv.x + qv.x, -(pv.y - qv.y), pv.y + qv.y, pv.x - qv.x);
      }
    }
    __syncthreads();
    float* out = KMAJ ? nullptr : tm + (size_t)img * (4 * Ny + 1) * Lx;
    for (int fy = fy0; fy < fy1; ++fy) {
      const float4* C = sC + fy * MAXD;
      // four independent FMA chains as two packed pairs: (ra, rb) += (c0, c1) * t and
      // (ia, ib) += (c2, c3) * t with t = (cos, sin) of the column, one f32x2 FMA each
      // (per component the same fmaf); without the term guard when 2Nx+1 is the table width
      float2 r = make_float2(C[0].x, 0.f), i2 = make_float2(C[0].y, 0.f);
      if (ND == MAXD) {
#pragma unroll
        for (int d = 1; d < MAXD; ++d) {
          const float4 a = C[d];
          r = __ffma2_rn(make_float2(a.x, a.y), tw[d], r);
          i2 = __ffma2_rn(make_float2(a.z, a.w), tw[d], i2);
        }
      } else {
#pragma unroll
        for (int d = 1; d < MAXD; ++d) {
          if (d < ND) {
            const float4 a = C[d];
            r = __ffma2_rn(make_float2(a.x, a.y), tw[d], r);
            i2 = __ffma2_rn(make_float2(a.z, a.w), tw[d], i2);
          }
        }
      }
      if (!live) continue;
      const float re = r.x + r.y, im = i2.x + i2.y, rem = r.x - r.y, imm = i2.x - i2.y;
      if (KMAJ) {
        if (fy == 0) {
          t0[(size_t)img * Lx + X] = re;
          if (mlive) t0[(size_t)img * Lx + Xm] = rem;
        } else {
          sO[xl * (KP + 1) + fy - 1] = re;
          sO[xl * (KP + 1) + 2 * Ny + fy - 1] = im;
          sO[(FR_COLS + xl) * (KP + 1) + fy - 1] = rem;  // unused when the mirror is outside
          sO[(FR_COLS + xl) * (KP + 1) + 2 * Ny + fy - 1] = imm;
        }
      } else if (fy == 0) {
        out[X] = re;
        if (mlive) out[Xm] = rem;
      } else {
        out[(size_t)fy * Lx + X] = re;
        out[(size_t)(2 * Ny + fy) * Lx + X] = im;
        if (mlive) {
          out[(size_t)fy * Lx + Xm] = rem;
          out[(size_t)(2 * Ny + fy) * Lx + Xm] = imm;
        }
      }
    }
    if (xtra && tid < 32) {  // the column x' = 0: S0 + sum_{d>0} (p + q), d in order
      for (int fy = tid; fy < BH; fy += 32) {
        const float4* C = sC + fy * MAXD;
        float re = C[0].x, im = C[0].y;
        for (int d = 1; d < ND; ++d) {
          re += C[d].x;
          im += C[d].z;
        }
        if (KMAJ) {
          if (fy == 0) {
            t0[(size_t)img * Lx + nb] = re;
          } else {
            sO[2 * FR_COLS * (KP + 1) + fy - 1] = re;
            sO[2 * FR_COLS * (KP + 1) + 2 * Ny + fy - 1] = im;
          }
        } else if (fy == 0) {
          out[nb] = re;
        } else {
          out[(size_t)fy * Lx + nb] = re;
          out[(size_t)(2 * Ny + fy) * Lx + nb] = im;
        }
      }
    }
    if (KMAJ) {
      __syncthreads();
      // each row is KP floats of [X][KP]: float4 stores, rows of one run contiguous
      const int q4 = KP / 4;
      for (int e = tid; e < nrows * q4; e += FR_THREADS) {
        const int s = e / q4, c = 4 * (e - s * q4);
        int srow, Xg;
        if (s < nbase) {
          srow = s;
          Xg = X0 + s;
        } else if (s < nbase + nmir) {
          const int j = s - nbase;
          srow = FR_COLS + nbase - 1 - j;
          Xg = Mlo + j;
        } else {
          srow = 2 * FR_COLS;
          Xg = nb;
        }
        const float* v = sO + srow * (KP + 1) + c;
        const float h0 = tc::tf32_round(v[0]), h1 = tc::tf32_round(v[1]), h2 = tc::tf32_round(v[2]),
                    h3 = tc::tf32_round(v[3]);
        const size_t o = ((size_t)img * Lx + Xg) * KP + c;
        *reinterpret_cast<float4*>(tmh + o) = make_float4(h0, h1, h2, h3);
        *reinterpret_cast<float4*>(tml + o) = make_float4(v[0] - h0, v[1] - h1, v[2] - h2, v[3] - h3);
      }
    }
  }
}

template <int MAXD, bool KMAJ, int KPC = 0>
static cudaError_t launch_fi_rows_t(cudaStream_t s, const ImgPlan& p, const float2* band_part, const float2* twF,
                                    int KP, float* tm, float* tmh, float* tml, float* t0) {
  const ImgGeom& g = p.g;
  // two shared buffers for the band partials of the next image when they fit in 32 KB
  const int rawn = p.ngroups * (2 * g.Ny + 1) * (4 * g.Nx + 1);
  const bool pre = (size_t)2 * rawn * sizeof(float2) <= 32 * 1024;
  const size_t smem = (size_t)(2 * g.Ny + 1) * MAXD * sizeof(float4) +
                      (KMAJ ? (size_t)FR_ROWS * (KP + 1) * sizeof(float) : 0) +
                      (pre ? 2 * (size_t)rawn * sizeof(float2) + 16 : 0);
  auto k = fi_rows_kernel<MAXD, KMAJ, KPC>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  // column blocks over the x' < 0 half; as many image groups as keep every CTA resident
  // at once (a second partial wave would double the time of the CTAs in it), each CTA
  // walking its group's images with its twiddles kept in registers
  const int nb = g.Fx / 2 - (g.Fx - g.Lx) / 2;
  const int ncb = std::max(1, (nb + FR_COLS - 1) / FR_COLS);
  const int sms = p.sms > 0 ? p.sms : 148;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, FR_THREADS, smem);
  if (e != cudaSuccess) return e;
  const int groups = std::max(1, std::min(p.batch, std::max(1, per_sm) * sms / ncb));
  k<<<dim3(ncb, groups), FR_THREADS, smem, s>>>(band_part, p.ngroups, twF, g.Lx, g.Fx, g.Nx, g.Ny, KP, p.batch,
                                                pre ? rawn : 0, tm, tmh, tml, t0);
  return cudaGetLastError();
}

cudaError_t launch_fi_rows(cudaStream_t s, const ImgPlan& p, const float2* band_part, const float2* twF, int KP,
                           float* tm, float* tmh, float* tml, float* t0) {
  const int ND = 2 * p.g.Nx + 1;
  const bool km = tmh != nullptr;
  if (km && KP == 32) {  // the K-major width of Ny <= 8 at compile time
    if (ND <= 5) return launch_fi_rows_t<5, true, 32>(s, p, band_part, twF, KP, tm, tmh, tml, t0);
    if (ND <= 9) return launch_fi_rows_t<9, true, 32>(s, p, band_part, twF, KP, tm, tmh, tml, t0);
    if (ND <= 17) return launch_fi_rows_t<17, true, 32>(s, p, band_part, twF, KP, tm, tmh, tml, t0);
    return launch_fi_rows_t<33, true, 32>(s, p, band_part, twF, KP, tm, tmh, tml, t0);
  }
  if (ND <= 5) return km ? launch_fi_rows_t<5, true>(s, p, band_part, twF, KP, tm, tmh, tml, t0)
                         : launch_fi_rows_t<5, false>(s, p, band_part, twF, KP, tm, tmh, tml, t0);
  if (ND <= 9) return km ? launch_fi_rows_t<9, true>(s, p, band_part, twF, KP, tm, tmh, tml, t0)
                         : launch_fi_rows_t<9, false>(s, p, band_part, twF, KP, tm, tmh, tml, t0);
  if (ND <= 17) return km ? launch_fi_rows_t<17, true>(s, p, band_part, twF, KP, tm, tmh, tml, t0)
                          : launch_fi_rows_t<17, false>(s, p, band_part, twF, KP, tm, tmh, tml, t0);
  return km ? launch_fi_rows_t<33, true>(s, p, band_part, twF, KP, tm, tmh, tml, t0)
            : launch_fi_rows_t<33, false>(s, p, band_part, twF, KP, tm, tmh, tml, t0);
}

// twF[d][X] = e^{+2 pi i d x'/Fx}, d = 0..2Nx: the FI column twiddles
__global__ void twF_init_kernel(float2* __restrict__ tw, int Lx, int Fx, int ND) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, d = blockIdx.y;
  if (x >= Lx || d >= ND) return;
  const long long xp = (long long)x + (Fx - Lx) / 2 - Fx / 2;
  tw[(size_t)d * Lx + x] = cis_exact((long long)d * xp, Fx, 1.f);
}

// cached per (Lx, Fx, Nx) on the context
int fi_twiddles(litho_ctx* ctx, const ImgGeom& g, const float2** out) {
  auto key = std::make_tuple(g.Lx, g.Fx, g.Nx, -4000);
  auto it = ctx->twx_tables.find(key);
  if (it == ctx->twx_tables.end()) {
    const int ND = 2 * g.Nx + 1;
    DevBuf b;
    LITHO_RET(b.ensure(ctx, (size_t)ND * g.Lx * sizeof(float2)));
    StageScope sc(ctx, LITHO_STAGE_UPLOAD);
    twF_init_kernel<<<dim3((g.Lx + 127) / 128, ND), 128, 0, ctx->stream>>>(b.as<float2>(), g.Lx, g.Fx, ND);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
    it = ctx->twx_tables.emplace(key, b).first;
  }
  *out = it->second.as<float2>();
  return LITHO_OK;
}

// ---------------------------------------------------------------------------
// FI, step 2: image = Cy (Ly x KB) * Tm (KB x Lx), KB = 4Ny+1.
// ---------------------------------------------------------------------------
constexpr int FO_BM = 32, FO_BN = 128, FO_THREADS = 256;

// The rows pair up around the centre: with y' = Y + oy (oy = (Fy-Ly)/2 - Fy/2) the image is
//   image(+b) = A(b) + B(b),  image(-b) = A(b) - B(b),
//   A(b) = T0 + sum_{r=1..2Ny} 2cos(2 pi r b/Fy) Re T_r,  B(b) = sum_r -2sin(2 pi r b/Fy) Im T_r,
// so one set of sums over the 4Ny+1 rows of Tm serves rows +b and -b.  Cm[r][b] holds the
// coefficients of base row b (r = 0: 1; 1..2Ny: 2cos; 2Ny+1..4Ny: -2sin), b < nbp (the
// base rows |y'| rounded up to FO_BM).  The FI kernel evaluates the same values when it
// has no table (the allocation-free entry point).
__device__ __forceinline__ float fo_cm(int r, int b, int Fy, int Ny) {
  if (r == 0) return 1.f;
  const int dy = r <= 2 * Ny ? r : r - 2 * Ny;
  const float2 e = cis_exact((long long)dy * b, Fy, 1.f);
  return r <= 2 * Ny ? 2.f * e.x : -2.f * e.y;
}

__global__ void fo_cm_init_kernel(float* __restrict__ cm, int nbp, int Fy, int Ny) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y;
  if (b < nbp) cm[(size_t)r * nbp + b] = fo_cm(r, b, Fy, Ny);
}

// the Cm table of a geometry, cached per (Ly, Fy, Ny) on the context
static int fo_cm_table(litho_ctx* ctx, const ImgGeom& g, const float** out, int* nbp) {
  *nbp = (fo_nbase(g.Ly, g.Fy) + FO_BM - 1) / FO_BM * FO_BM;
  auto key = std::make_tuple(g.Ly, g.Fy, g.Ny, -5001);
  auto it = ctx->twx_tables.find(key);
  if (it == ctx->twx_tables.end()) {
    const int KB = 4 * g.Ny + 1;
    DevBuf b;
    LITHO_RET(b.ensure(ctx, (size_t)KB * *nbp * sizeof(float)));
    StageScope sc(ctx, LITHO_STAGE_UPLOAD);
    fo_cm_init_kernel<<<dim3(*nbp / FO_BM, KB), FO_BM, 0, ctx->stream>>>(b.as<float>(), *nbp, g.Fy, g.Ny);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
    it = ctx->twx_tables.emplace(key, b).first;
  }
  *out = it->second.as<float>();
  return LITHO_OK;
}

// One CTA per (FO_BM base rows, FO_BN columns, image): thread (warp w, lane l) sums base
// rows 4w..4w+3 over columns 4l..4l+3, the cos rows of Tm into A and the sin rows into B
// (packed f32x2 FMAs), and writes A + B to row +b and A - B to row -b where they lie in
// the image.
template <bool VEC>
__global__ void __launch_bounds__(FO_THREADS) fi_out_kernel(const float* __restrict__ tm, int Lx, int Ly, int Fy,
                                                            int Ny, const float* __restrict__ cmt, int nbp,
                                                            float* __restrict__ images) {
  extern __shared__ __align__(16) float fo[];
  const int KB = 4 * Ny + 1;
  float* sC = fo;                // [KB][FO_BM]
  float* sT = fo + KB * FO_BM;   // [KB][FO_BN]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int X0 = blockIdx.x * FO_BN, B0 = blockIdx.y * FO_BM, img = blockIdx.z;
  const float* T = tm + (size_t)img * KB * Lx;
  if (VEC) {
    for (int idx = tid; idx < KB * (FO_BN / 4); idx += FO_THREADS) {
      const int r = idx / (FO_BN / 4), c4 = 4 * (idx - r * (FO_BN / 4));
      const int X = X0 + c4;
      reinterpret_cast<float4*>(sT)[idx] =
          X < Lx ? __ldg(reinterpret_cast<const float4*>(T + (size_t)r * Lx + X)) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  } else {
    for (int idx = tid; idx < KB * FO_BN; idx += FO_THREADS) {
      const int r = idx / FO_BN, c = idx - r * FO_BN;
      const int X = X0 + c;
      sT[idx] = X < Lx ? T[(size_t)r * Lx + X] : 0.f;
    }
  }
  if (cmt != nullptr) {  // the cached table: whole 16-byte pieces of the tile's base rows
    for (int idx = tid; idx < KB * (FO_BM / 4); idx += FO_THREADS) {
      const int r = idx / (FO_BM / 4), q = idx - r * (FO_BM / 4);
      reinterpret_cast<float4*>(sC)[idx] = __ldg(reinterpret_cast<const float4*>(cmt + (size_t)r * nbp + B0) + q);
    }
  } else {
    for (int idx = tid; idx < KB * FO_BM; idx += FO_THREADS) {
      const int r = idx / FO_BM, bb = idx - r * FO_BM;
      sC[idx] = fo_cm(r, B0 + bb, Fy, Ny);
    }
  }
  __syncthreads();
  // A and B of 4 base rows x 4 columns, in column pairs
  float2 A[4][2], Bs[4][2];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) A[i][j] = Bs[i][j] = make_float2(0.f, 0.f);
  auto step = [&](int r, float2(&acc)[4][2]) {
    const float4 c = *reinterpret_cast<const float4*>(sC + r * FO_BM + 4 * warp);  // one address per warp
    const float4 t = *reinterpret_cast<const float4*>(sT + r * FO_BN + 4 * lane);
    const float cc[4] = {c.x, c.y, c.z, c.w};
    const float2 tlo = make_float2(t.x, t.y), thi = make_float2(t.z, t.w);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float2 ci = make_float2(cc[i], cc[i]);
      acc[i][0] = __ffma2_rn(ci, tlo, acc[i][0]);
      acc[i][1] = __ffma2_rn(ci, thi, acc[i][1]);
    }
  };
#pragma unroll 4
  for (int r = 0; r <= 2 * Ny; ++r) step(r, A);
#pragma unroll 4
  for (int r = 2 * Ny + 1; r < KB; ++r) step(r, Bs);
  const int nbase = fo_nbase(Ly, Fy);
  float* O = images + (size_t)img * Lx * Ly;
  const int X = X0 + 4 * lane;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int b = B0 + 4 * warp + i;
    if (b >= nbase) continue;
#pragma unroll
    for (int sgn = 0; sgn < 2; ++sgn) {
      const int Y = fo_row(b, sgn, Ly, Fy);  // y' = +b, -b (y' = 0 once)
      if (Y < 0) continue;
      const float o[4] = {sgn == 0 ? A[i][0].x + Bs[i][0].x : A[i][0].x - Bs[i][0].x,
                          sgn == 0 ? A[i][0].y + Bs[i][0].y : A[i][0].y - Bs[i][0].y,
                          sgn == 0 ? A[i][1].x + Bs[i][1].x : A[i][1].x - Bs[i][1].x,
                          sgn == 0 ? A[i][1].y + Bs[i][1].y : A[i][1].y - Bs[i][1].y};
      float* row = O + (size_t)Y * Lx;
      if (VEC && X + 3 < Lx) {
        __stcs(reinterpret_cast<float4*>(row + X), make_float4(o[0], o[1], o[2], o[3]));
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if (X + e < Lx) row[X + e] = o[e];
      }
    }
  }
}

// launch geometry of the FI output kernel
static inline dim3 fo_grid(const ImgGeom& g, int batch) {
  const int nb = fo_nbase(g.Ly, g.Fy);
  return dim3((g.Lx + FO_BN - 1) / FO_BN, (nb + FO_BM - 1) / FO_BM, batch);
}

// ---------------------------------------------------------------------------
// Full centred mask spectrum (litho_fft_mask): two passes of a block FFT over
// shared-memory rows, each pass writing its result transposed.
//   C[X] = sum_p a[p] e^{-2 pi i (X - F/2)(p - F/2)/F}
//        = (-1)^(X + F/2) * DFT((-1)^p a[p])[X]
// ---------------------------------------------------------------------------
constexpr int FM_THREADS = 256;

// rows: `nrows` input rows of length `len` (real if in_i == nullptr), padded
// centred into F; output written transposed: out[X][row] (row stride ldo).
__global__ void __launch_bounds__(FM_THREADS) fft_rows_centred_kernel(
    const float* __restrict__ in_r, const float* __restrict__ in_i, const float2* __restrict__ in_c,
    int nrows, int len, int F, int TR, float scale, float2* __restrict__ out_c, float* __restrict__ out_r,
    float* __restrict__ out_i, int ldo) {
  extern __shared__ __align__(16) float2 fr[];
  const int SF = F + 1;
  float2* s = fr;                 // [TR][SF]
  float2* tw = fr + TR * SF;      // [F/2]
  const int tid = threadIdx.x;
  const int r0 = blockIdx.x * TR;
  const int logF = 31 - __clz(F);
  const int off = (F - len) / 2;
  for (int e = tid; e < F / 2; e += FM_THREADS) {
    float sn, cs;
    sincospif(2.0f * (float)e / (float)F, &sn, &cs);
    tw[e] = make_float2(cs, -sn);
  }
  // load with bit-reversed placement, pre-multiplied by (-1)^p
  for (int idx = tid; idx < TR * F; idx += FM_THREADS) {
    const int r = idx / F, p = idx - r * F;
    const int row = r0 + r;
    float2 v = make_float2(0.f, 0.f);
    const int q = p - off;
    if (row < nrows && q >= 0 && q < len) {
      const size_t o = (size_t)row * len + q;
      if (in_c) v = in_c[o];
      else v = make_float2(in_r[o], in_i ? in_i[o] : 0.f);
      if (p & 1) v = make_float2(-v.x, -v.y);
    }
    const int br = (int)(__brev((unsigned)p) >> (32 - logF));
    s[r * SF + br] = v;
  }
  __syncthreads();
  for (int h = 1; h < F; h <<= 1) {
    for (int idx = tid; idx < TR * (F / 2); idx += FM_THREADS) {
      const int r = idx / (F / 2), b = idx - r * (F / 2);
      const int grp = b / h, pos = b - grp * h;
      const int i0 = grp * 2 * h + pos, i1 = i0 + h;
      const float2 w = tw[pos * (F / (2 * h))];
      float2* rowp = s + r * SF;
      const float2 t = cmul(w, rowp[i1]);
      const float2 a = rowp[i0];
      rowp[i0] = cadd(a, t);
      rowp[i1] = csub(a, t);
    }
    __syncthreads();
  }
  // transposed write with (-1)^(X + F/2) and scale
  const float sgnF = ((F / 2) & 1) ? -1.f : 1.f;
  for (int idx = tid; idx < TR * F; idx += FM_THREADS) {
    const int X = idx / TR, r = idx - X * TR;
    const int row = r0 + r;
    if (row >= nrows) continue;
    float2 v = s[r * SF + X];
    const float sg = ((X & 1) ? -sgnF : sgnF) * scale;
    v = make_float2(v.x * sg, v.y * sg);
    const size_t o = (size_t)X * ldo + row;
    if (out_c) out_c[o] = v;
    else {
      out_r[o] = v.x;
      out_i[o] = v.y;
    }
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int njt_for(int Nx) {
  const int nj = 2 * Nx + 1;
  if (nj <= 8) return 8;
  if (nj <= 12) return 12;
  if (nj <= 20) return 20;
  if (nj <= 36) return 36;
  return -1;
}

ImgPlan make_plan(const ImgGeom& g, int batch, int sm_count) {
  ImgPlan p;
  p.g = g;
  p.batch = batch;
  p.rowBlocks = (g.Ly + WD_BM - 1) / WD_BM;
  const int nch = (g.Lx + WD_BK - 1) / WD_BK;
  const int want = 2 * sm_count;
  int cs = (want + p.rowBlocks * batch - 1) / (p.rowBlocks * batch);
  cs = std::max(1, std::min(cs, std::max(1, nch / 2)));
  p.colSplits = cs;
  // SOCS is latency-bound (warp-shuffle FFT chains), but every kernel group also
  // transforms its own partial intensity: ~2.5 CTAs (20 warps) per SM measured best
  // at 1024^2, K=24, 64 masks (4 kernels per CTA: 36.9 us; 3: 38.9; 8: 45.0)
  int ng = (5 * sm_count + 2 * batch - 1) / (2 * batch);
  ng = std::max(1, std::min(ng, g.nk));
  p.kpg = (g.nk + ng - 1) / ng;
  p.ngroups = (g.nk + p.kpg - 1) / p.kpg;
  p.sms = sm_count;
  return p;
}

static int twx_table(litho_ctx* ctx, int Lx, int Fx, int Nx, int NJT, const float** out) {
  auto key = std::make_tuple(Lx, Fx, Nx, NJT);
  auto it = ctx->twx_tables.find(key);
  if (it == ctx->twx_tables.end()) {
    DevBuf b;
    LITHO_RET(b.ensure(ctx, (size_t)Lx * NJT * sizeof(float)));
    StageScope sc(ctx, LITHO_STAGE_UPLOAD);
    twx_init_kernel<<<(Lx + 127) / 128, 128, 0, ctx->stream>>>(b.as<float>(), Lx, Fx, Nx, NJT);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
    it = ctx->twx_tables.emplace(key, b).first;
  }
  *out = it->second.as<float>();
  return LITHO_OK;
}

template <int NJT>
static int launch_win_dft_t(litho_ctx* ctx, const ImgPlan& p, const float* masks, const float* twx,
                            float2* win_part) {
  const ImgGeom& g = p.g;
  const size_t smem = win_dft_smem<NJT>(g.Ny);
  dim3 grid(p.rowBlocks, p.colSplits, p.batch);
  StageScope sc(ctx, LITHO_STAGE_WIN_DFT);
  if ((g.Lx & 3) == 0) {
    auto k = win_dft_kernel<NJT, true>;
    LITHO_CUDA_TRY(ctx, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k<<<grid, WD_THREADS, smem, ctx->stream>>>(masks, g.Lx, g.Ly, g.Fx, g.Fy, g.Nx, g.Ny, twx, win_part, p.part_stride);
  } else {
    auto k = win_dft_kernel<NJT, false>;
    LITHO_CUDA_TRY(ctx, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k<<<grid, WD_THREADS, smem, ctx->stream>>>(masks, g.Lx, g.Ly, g.Fx, g.Fy, g.Nx, g.Ny, twx, win_part, p.part_stride);
  }
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  return LITHO_OK;
}

// Build the cached column-twiddle table a plain window DFT of this geometry reads, on the
// context's stream (so that launches on other streams find it ready).
int prepare_win_dft(litho_ctx* ctx, const ImgPlan& p) {
  const int NJT = njt_for(p.g.Nx);
  if (NJT < 0) return LITHO_OK;  // the launch reports the unsupported size
  const float* twx = nullptr;
  return twx_table(ctx, p.g.Lx, p.g.Fx, p.g.Nx, NJT, &twx);
}

int run_win_dft(litho_ctx* ctx, const ImgPlan& p, const float* masks, float2* win_part) {
  const int NJT = njt_for(p.g.Nx);
  if (NJT < 0) {
    set_error(ctx, LITHO_ERR_UNSUPPORTED, "window DFT supports Nx <= 16 (got %d)", p.g.Nx);
    return LITHO_ERR_UNSUPPORTED;
  }
  const float* twx = nullptr;
  LITHO_RET(twx_table(ctx, p.g.Lx, p.g.Fx, p.g.Nx, NJT, &twx));
  switch (NJT) {
    case 8: return launch_win_dft_t<8>(ctx, p, masks, twx, win_part);
    case 12: return launch_win_dft_t<12>(ctx, p, masks, twx, win_part);
    case 20: return launch_win_dft_t<20>(ctx, p, masks, twx, win_part);
    default: return launch_win_dft_t<36>(ctx, p, masks, twx, win_part);
  }
}

template <int N>
static int launch_socs_t(litho_ctx* ctx, const ImgPlan& p, const WindowSrc& w, const float2* krn,
                         const float* scales, float2* band_part, float* tmpImgp) {
  const ImgGeom& g = p.g;
  const int KD = (2 * g.Nx + 1) * (2 * g.Ny + 1);
  size_t smem;
  decltype(&socs64_kernel) k;
  if constexpr (N == 64) {
    smem = socs64_smem_bytes(KD);
    k = socs64_kernel;
  } else if constexpr (N == 128) {
    smem = socs128_smem_bytes(2 * g.Ny + 1, KD);
    k = socs128_kernel;
  } else {
    smem = ((size_t)(2 * g.Ny + 1) * (N + 1) + N / 2 + KD) * sizeof(float2);
    k = socs_kernel<N>;
  }
  LITHO_CUDA_TRY(ctx, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid(p.ngroups, p.batch);
  StageScope sc(ctx, LITHO_STAGE_SOCS);
  k<<<grid, N == 128 ? S128_THREADS : SOCS_THREADS, smem, ctx->stream>>>(w.part, w.nparts, w.mskf_r, w.mskf_i, g.Fx,
                                                                       g.Fy, g.Nx, g.Ny, krn,
                                                scales, g.nk, p.kpg, band_part, tmpImgp);
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  return LITHO_OK;
}

int run_socs(litho_ctx* ctx, const ImgPlan& p, const WindowSrc& w, const float2* krn, const float* scales,
             float2* band_part, float* tmpImgp) {
  if (tmpImgp != nullptr && p.ngroups != 1) {
    set_error(ctx, LITHO_ERR_ARG, "tmpImgp output needs a single kernel group");
    return LITHO_ERR_ARG;
  }
  switch (p.g.convN) {
    case 32: return launch_socs_t<32>(ctx, p, w, krn, scales, band_part, tmpImgp);
    case 64: return launch_socs_t<64>(ctx, p, w, krn, scales, band_part, tmpImgp);
    case 128: return launch_socs_t<128>(ctx, p, w, krn, scales, band_part, tmpImgp);
    default:
      set_error(ctx, LITHO_ERR_UNSUPPORTED, "conv grid %d not in {32, 64, 128}", p.g.convN);
      return LITHO_ERR_UNSUPPORTED;
  }
}

int run_fi(litho_ctx* ctx, const ImgPlan& p, const float2* band_part, float* tm, float* images) {
  const ImgGeom& g = p.g;
  {
    const float2* twF = nullptr;
    LITHO_RET(fi_twiddles(ctx, g, &twF));
    StageScope sc(ctx, LITHO_STAGE_FI_PREP);
    LITHO_CUDA_TRY(ctx, launch_fi_rows(ctx->stream, p, band_part, twF, 0, tm, nullptr, nullptr, nullptr));
  }
  {
    const int KB = 4 * g.Ny + 1;
    int nbp = 0;
    const float* cmt = nullptr;
    LITHO_RET(fo_cm_table(ctx, g, &cmt, &nbp));
    const size_t smem = (size_t)KB * (FO_BM + FO_BN) * sizeof(float);
    StageScope sc(ctx, LITHO_STAGE_FI_OUT);
    auto k = (g.Lx & 3) == 0 ? fi_out_kernel<true> : fi_out_kernel<false>;
    LITHO_CUDA_TRY(ctx, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k<<<fo_grid(g, p.batch), FO_THREADS, smem, ctx->stream>>>(tm, g.Lx, g.Ly, g.Fy, g.Ny, cmt, nbp, images);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
  }
  return LITHO_OK;
}

static int fm_rows_per_cta(int F) { return std::max(1, 16384 / F) > 16 ? 16 : std::max(1, 16384 / F); }

int run_fft_mask(litho_ctx* ctx, const float* mask, int Lx, int Ly, float* mskf_r, float* mskf_i) {
  const int Fx = next_pow2(Lx), Fy = next_pow2(Ly);
  // pass 1: mask rows -> tmp[X][y] (Fx x Ly complex)
  LITHO_RET(ctx->stage_x.ensure(ctx, (size_t)Fx * Ly * sizeof(float2)));
  float2* tmp = ctx->stage_x.as<float2>();
  StageScope sc(ctx, LITHO_STAGE_FFT_MASK, 2);
  {
    const int TR = fm_rows_per_cta(Fx);
    const size_t smem = ((size_t)TR * (Fx + 1) + Fx / 2) * sizeof(float2);
    LITHO_CUDA_TRY(ctx, cudaFuncSetAttribute(fft_rows_centred_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    fft_rows_centred_kernel<<<(Ly + TR - 1) / TR, FM_THREADS, smem, ctx->stream>>>(
        mask, nullptr, nullptr, Ly, Lx, Fx, TR, 1.0f, tmp, nullptr, nullptr, Ly);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
  }
  // pass 2: tmp rows (one per X, length Ly) -> mskf[Y][X] / (Fx*Fy)
  {
    const int TR = fm_rows_per_cta(Fy);
    const size_t smem = ((size_t)TR * (Fy + 1) + Fy / 2) * sizeof(float2);
    const float scale = 1.0f / ((float)Fx * (float)Fy);
    LITHO_CUDA_TRY(ctx, cudaFuncSetAttribute(fft_rows_centred_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    fft_rows_centred_kernel<<<(Fx + TR - 1) / TR, FM_THREADS, smem, ctx->stream>>>(
        nullptr, nullptr, tmp, Fx, Ly, Fy, TR, scale, nullptr, mskf_r, mskf_i, Fx);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
  }
  return LITHO_OK;
}

// ---------------------------------------------------------------------------
// Context-free launch of the FP32 pipeline for one image into caller-provided
// scratch (used by the allocation-free entry point in noalloc.cu).  Launches
// only; it allocates nothing and records nothing on a context.
// ---------------------------------------------------------------------------
__global__ void pack_planes_kernel(const float* __restrict__ kr, const float* __restrict__ ki, int n,
                                   float2* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_float2(kr[i], ki[i]);
}

size_t noctx_scratch_layout(const ImgPlan& p, size_t off[6]) {
  const ImgGeom& g = p.g;
  const int KD = (2 * g.Nx + 1) * (2 * g.Ny + 1), KY = 2 * g.Ny + 1;
  const size_t sz[6] = {(size_t)g.nk * KD * sizeof(float2),
                        (size_t)g.nk * sizeof(float),
                        (size_t)g.Lx * njt_for(g.Nx) * sizeof(float),
                        (size_t)p.nparts() * KY * (g.Nx + 1) * sizeof(float2),
                        (size_t)p.ngroups * KY * (4 * g.Nx + 1) * sizeof(float2),
                        (size_t)(4 * g.Ny + 1) * g.Lx * sizeof(float)};
  size_t o = 0;
  for (int i = 0; i < 6; ++i) {
    off[i] = o;
    o += (sz[i] + 255) & ~size_t(255);
  }
  return o;
}

template <int NJT>
static cudaError_t noctx_win_dft_t(cudaStream_t s, const ImgPlan& p, const float* masks, const float* twx,
                                   float2* win_part) {
  const ImgGeom& g = p.g;
  const size_t smem = win_dft_smem<NJT>(g.Ny);
  dim3 grid(p.rowBlocks, p.colSplits, p.batch);
  auto k = (g.Lx & 3) == 0 ? win_dft_kernel<NJT, true> : win_dft_kernel<NJT, false>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<grid, WD_THREADS, smem, s>>>(masks, g.Lx, g.Ly, g.Fx, g.Fy, g.Nx, g.Ny, twx, win_part, 0);
  return cudaGetLastError();
}

template <int N>
static cudaError_t noctx_socs_t(cudaStream_t s, const ImgPlan& p, const float2* win_part, const float2* krn,
                                const float* scales, float2* band_part) {
  const ImgGeom& g = p.g;
  const int KD = (2 * g.Nx + 1) * (2 * g.Ny + 1);
  size_t smem;
  decltype(&socs64_kernel) k;
  if constexpr (N == 64) {
    smem = socs64_smem_bytes(KD);
    k = socs64_kernel;
  } else if constexpr (N == 128) {
    smem = socs128_smem_bytes(2 * g.Ny + 1, KD);
    k = socs128_kernel;
  } else {
    smem = ((size_t)(2 * g.Ny + 1) * (N + 1) + N / 2 + KD) * sizeof(float2);
    k = socs_kernel<N>;
  }
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<dim3(p.ngroups, p.batch), N == 128 ? S128_THREADS : SOCS_THREADS, smem, s>>>(win_part, p.nparts(), nullptr,
                                                                                 nullptr, g.Fx, g.Fy, g.Nx,
                                                          g.Ny, krn, scales, g.nk, p.kpg, band_part, nullptr);
  return cudaGetLastError();
}

cudaError_t image_pipeline_noctx(cudaStream_t s, const ImgPlan& p, const float* mask, const float* krn_r,
                                 const float* krn_i, const float* scales, char* scratch, float* image) {
  const ImgGeom& g = p.g;
  size_t off[6];
  noctx_scratch_layout(p, off);
  float2* krn = reinterpret_cast<float2*>(scratch + off[0]);
  float* sc = reinterpret_cast<float*>(scratch + off[1]);
  float* twx = reinterpret_cast<float*>(scratch + off[2]);
  float2* win_part = reinterpret_cast<float2*>(scratch + off[3]);
  float2* band_part = reinterpret_cast<float2*>(scratch + off[4]);
  float* tm = reinterpret_cast<float*>(scratch + off[5]);
  const int KD = (2 * g.Nx + 1) * (2 * g.Ny + 1);
  const int NJT = njt_for(g.Nx);
  cudaError_t e;
  pack_planes_kernel<<<(g.nk * KD + 255) / 256, 256, 0, s>>>(krn_r, krn_i, g.nk * KD, krn);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(sc, scales, g.nk * sizeof(float), cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return e;
  twx_init_kernel<<<(g.Lx + 127) / 128, 128, 0, s>>>(twx, g.Lx, g.Fx, g.Nx, NJT);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  switch (NJT) {
    case 8: e = noctx_win_dft_t<8>(s, p, mask, twx, win_part); break;
    case 12: e = noctx_win_dft_t<12>(s, p, mask, twx, win_part); break;
    case 20: e = noctx_win_dft_t<20>(s, p, mask, twx, win_part); break;
    default: e = noctx_win_dft_t<36>(s, p, mask, twx, win_part); break;
  }
  if (e != cudaSuccess) return e;
  switch (g.convN) {
    case 32: e = noctx_socs_t<32>(s, p, win_part, krn, sc, band_part); break;
    case 64: e = noctx_socs_t<64>(s, p, win_part, krn, sc, band_part); break;
    default: e = noctx_socs_t<128>(s, p, win_part, krn, sc, band_part); break;
  }
  if (e != cudaSuccess) return e;
  // no twiddle table here (nothing may be allocated): the kernel evaluates them
  if ((e = launch_fi_rows(s, p, band_part, nullptr, 0, tm, nullptr, nullptr, nullptr)) != cudaSuccess) return e;
  {
    const int KB = 4 * g.Ny + 1;
    const size_t smem = (size_t)KB * (FO_BM + FO_BN) * sizeof(float);
    const dim3 grid = fo_grid(g, 1);
    auto k = (g.Lx & 3) == 0 ? fi_out_kernel<true> : fi_out_kernel<false>;
    if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
      return e;
    k<<<grid, FO_THREADS, smem, s>>>(tm, g.Lx, g.Ly, g.Fy, g.Ny, nullptr, 0, image);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// plan of one launch of the mixed form: the persistent tensor-core window kernel splits
// the 64-column chunks of a row block into tiles until there are ~6 tiles per SM, so the
// last round of tiles is short (each split adds an epilogue and a partial)
static ImgPlan mixed_plan(const ImgGeom& g, int batch, int sm_count) {
  ImgPlan p = make_plan(g, batch, sm_count);
  const int nch = (g.Lx + 63) / 64;
  const int units = p.rowBlocks * batch;
  const int want = 6 * sm_count;
  const int cs = units < want ? (want + units - 1) / units : 1;
  p.colSplits = std::max(1, std::min(cs, std::min(4, nch / 2)));
  return p;
}

int image_pipeline(litho_ctx* ctx, const ImgGeom& g, int batch, const float* masks, const litho_kernel_set* ks,
                   float* images, int precision) {
  const int KY = 2 * g.Ny + 1;
  const bool tc = precision == LITHO_PREC_MIXED && tc_supported(g);
  const bool band = use_band_tcc(ctx, ks, batch);
  ImgPlan p = tc ? mixed_plan(g, batch, ctx->sm_count) : make_plan(g, batch, ctx->sm_count);
  if (band) {
    p.ngroups = ks->band_nc;
    p.kpg = g.nk;
  }
  LITHO_RET(ctx->win_part.ensure(ctx, (size_t)batch * p.nparts() * KY * (g.Nx + 1) * sizeof(float2)));
  LITHO_RET(ctx->band_part.ensure(ctx, (size_t)batch * p.ngroups * KY * (4 * g.Nx + 1) * sizeof(float2)));
  if (band) LITHO_RET(ctx->band_w.ensure(ctx, band_wsum_bytes(g, batch)));
  if (tc) {
    LITHO_RET(run_win_dft_tc(ctx, p, masks, ctx->win_part.as<float2>()));
  } else {
    LITHO_RET(ctx->tm.ensure(ctx, (size_t)batch * (4 * g.Ny + 1) * g.Lx * sizeof(float)));
    LITHO_RET(run_win_dft(ctx, p, masks, ctx->win_part.as<float2>()));
  }
  WindowSrc w;
  w.part = ctx->win_part.as<float2>();
  w.nparts = p.nparts();
  if (band) LITHO_RET(run_band_tcc(ctx, p, w, ks, ctx->band_w.as<float2>(), ctx->band_part.as<float2>()));
  else LITHO_RET(run_socs(ctx, p, w, ks->krn, ks->scales, ctx->band_part.as<float2>(), nullptr));
  if (tc) return run_fi_tc(ctx, p, ctx->band_part.as<float2>(), nullptr, images);
  return run_fi(ctx, p, ctx->band_part.as<float2>(), ctx->tm.as<float>(), images);
}

}  // namespace litho
