// Fourier-neural-operator surrogate of the SOCS imaging map: forward, backward
// and Adam kernels, and the litho_surrogate_* C ABI.
//
// The reference has no surrogate (it images every mask with calcSOCS,
// litho.cpp:795-880); the network is the published FNO-2d (Li et al., ICLR
// 2021) with one input channel (the mask), width 32, 16 retained modes per
// axis, four Fourier layers and a 32->128->1 projection.
//
// Data layout (all per batch of B masks, L x L, channels-last):
//   z_l      bf16 [B][L][L][32]   pre-activation of Fourier layer l (v_{l+1} = GELU(z_l))
//   Xf / Xg  f32x2 [B][L][16][32] x-DFT of one row at kx = 0..15 (activations / gradients)
//   Gy / Gg  f32x2 [B][L][16][32] inverse y-DFT of the mixed modes, per row and kx
//   Vs_l     f32x2 [B][32][16][32] retained modes of v_l (kept for dR)
// A Fourier layer is two launches:
//   column kernel  (one CTA per kx and mask): y-DFT of Xf at the 32 kept ky,
//                  mode mixing by R (FP32 master weights), inverse y-DFT -> Gy
//   row kernel     (persistent over rows): z = W v + b + Re sum_kx Gy e^{i kx x}
//                  as two BF16 tensor-core GEMMs (K = 32 each), GELU, and the
//                  x-DFT of the result for the next layer as a third GEMM.
// The 1/L^2 and the factor 2 of the half spectrum are folded into the mixing
// (s_kx = c_kx / L^2), so the inverse evaluation E(U)(p) = sum Re(U phi_p) is
// the same sum in both directions; its adjoint is the forward partial DFT.
// Backward reuses the same pieces in reverse: the gradient of a layer input is
// W^T g_z + E(s conj(R)^T DFT(g_z)) and dR = s DFT(g_z) conj(V).
//
// GEMMs run on the tensor cores with mma.sync m16n8k16 BF16 (FP32 accumulate);
// weights stay in FP32 master copies and are rounded to BF16 in shared memory
// by every CTA.  The spectral intermediates stay FP32.

#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "litho_internal.cuh"

using bf16 = __nv_bfloat16;

namespace litho {
namespace fno {

constexpr int C = LITHO_FNO_WIDTH;    // 32 channels
constexpr int M = LITHO_FNO_MODES;    // 16 retained kx (and 2 x 16 retained ky)
constexpr int J = 2 * M;              // 32 ky slots: ky = j (j < 16), L - 32 + j (j >= 16)
constexpr int H = LITHO_FNO_HIDDEN;   // 128 projection channels
constexpr int NL = LITHO_FNO_LAYERS;  // 4 Fourier layers
constexpr int THREADS = 256;
constexpr int SP = 40;                // padded bf16 row stride of the 32-wide shared tiles

// flat FP32 parameter vector (the oracle's layout)
struct Off {
  static constexpr size_t Pw = 0, Pb = C;
  static constexpr size_t W = 2 * C;                   // [NL][C o][C c]
  static constexpr size_t Wb = W + (size_t)NL * C * C; // [NL][C]
  static constexpr size_t R = Wb + (size_t)NL * C;     // [NL][J][M][C c][C o][2]
  static constexpr size_t RL = (size_t)J * M * C * C * 2;
  static constexpr size_t Q1 = R + NL * RL;            // [H][C]
  static constexpr size_t q1b = Q1 + (size_t)H * C;
  static constexpr size_t Q2 = q1b + H;
  static constexpr size_t q2b = Q2 + H;
  static constexpr size_t N = q2b + 1;
};

// dense (non-spectral) gradient slots written per CTA by the row kernels
struct Dn {
  static constexpr int Pw = 0, Pb = C, W = 2 * C, Wb = W + NL * C * C, Q1 = Wb + NL * C, q1b = Q1 + H * C,
                       Q2 = q1b + H, q2b = Q2 + H, N = q2b + 1;
};

__host__ __device__ inline size_t dense_to_param(int i) {
  if (i < Dn::Wb) return (size_t)i;  // Pw, Pb, W share their offsets
  if (i < Dn::Q1) return Off::Wb + (i - Dn::Wb);
  return Off::Q1 + (size_t)(i - Dn::Q1);  // Q1, q1b, Q2, q2b are contiguous in both
}

// ---------------------------------------------------------------------------
// small device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float2 unpack2(uint32_t u) {
  __nv_bfloat162 v = *reinterpret_cast<__nv_bfloat162*>(&u);
  return __bfloat1622float2(v);
}
__device__ __forceinline__ uint32_t lds32(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }
__device__ __forceinline__ uint32_t ldg32(const bf16* p) { return __ldg(reinterpret_cast<const unsigned int*>(p)); }

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// GELU in its tanh form (Hendrycks & Gimpel 2016): 0.5 x (1 + tanh(k0 (x + k1 x^3)))
constexpr float GK0 = 0.79788456080286536f, GK1 = 0.044715f;
__device__ __forceinline__ float tanh_hw(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float gelu(float x) {
  const float t = tanh_hw(GK0 * fmaf(GK1 * x, x * x, x));
  return 0.5f * x * (1.0f + t);
}
__device__ __forceinline__ float gelu_grad(float x) {
  const float x2 = x * x;
  const float t = tanh_hw(GK0 * fmaf(GK1 * x, x2, x));
  return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * GK0 * fmaf(3.0f * GK1, x2, 1.0f);
}
// GELU and its derivative together
__device__ __forceinline__ void gelu_both(float x, float& g, float& d) {
  const float x2 = x * x;
  const float t = tanh_hw(GK0 * fmaf(GK1 * x, x2, x));
  g = 0.5f * x * (1.0f + t);
  d = 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * GK0 * fmaf(3.0f * GK1, x2, 1.0f);
}

// A fragment (16 x 16, row major) of a C-layout accumulator pair (n tiles 2ks, 2ks+1)
__device__ __forceinline__ void acc_to_a(const float* c0, const float* c1, uint32_t* a) {
  a[0] = pack2(c0[0], c0[1]);
  a[1] = pack2(c0[2], c0[3]);
  a[2] = pack2(c1[0], c1[1]);
  a[3] = pack2(c1[2], c1[3]);
}

// stage one row of Gy/Gg [M][C] complex as bf16 sG[c][2 kx + ri]
__device__ __forceinline__ void stage_g_row(const float2* __restrict__ gr, bf16* sG, int tid) {
  for (int i = tid; i < M * C; i += THREADS) {
    const float2 v = gr[i];
    const int kx = i / C, c = i % C;
    *reinterpret_cast<uint32_t*>(sG + c * SP + 2 * kx) = pack2(v.x, v.y);
  }
}

// ---------------------------------------------------------------------------
// tables: Ttab[px][2kx+ri] = (cos, -sin)(2 pi kx px / L); TT = transpose
// ---------------------------------------------------------------------------
__global__ void tables_kernel(int L, bf16* Ttab, bf16* TT, float2* twL) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < L * M) {
    const int px = i / M, kx = i % M;
    float s, c;
    sincospif(2.0f * (float)((kx * px) % L) / (float)L, &s, &c);
    Ttab[(size_t)px * J + 2 * kx] = __float2bfloat16(c);
    Ttab[(size_t)px * J + 2 * kx + 1] = __float2bfloat16(-s);
    TT[(size_t)(2 * kx) * L + px] = __float2bfloat16(c);
    TT[(size_t)(2 * kx + 1) * L + px] = __float2bfloat16(-s);
  }
  if (i < L) {
    float s, c;
    sincospif(2.0f * (float)i / (float)L, &s, &c);
    twL[i] = make_float2(c, s);  // e^{+2 pi i k / L}
  }
}

// ---------------------------------------------------------------------------
// lift + x-DFT of layer 0: v0 = Pw m + Pb, so X0[kx][c] = Pw[c] DFT(m)[kx] + Pb[c] L d(kx)
// One warp per row.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(THREADS) lift_dft_kernel(int L, int rows, const float* __restrict__ theta,
                                                           const float* __restrict__ masks,
                                                           const float2* __restrict__ twL, float2* __restrict__ Xf,
                                                           float2* __restrict__ Mrow) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row = blockIdx.x * (THREADS / 32) + warp;
  if (row >= rows) return;
  const float* m = masks + (size_t)row * L;
  const int kx = lane & 15, half = lane >> 4;
  float re = 0.f, im = 0.f;
  for (int px = half; px < L; px += 2) {
    const float v = m[px];
    const float2 w = twL[(kx * px) & (L - 1)];
    re = fmaf(v, w.x, re);
    im = fmaf(-v, w.y, im);
  }
  re += __shfl_xor_sync(0xffffffffu, re, 16);
  im += __shfl_xor_sync(0xffffffffu, im, 16);
  if (Mrow && lane < 16) Mrow[(size_t)row * 16 + lane] = make_float2(re, im);  // mask row DFT, kx < 16
  float2* out = Xf + (size_t)row * M * C;
  for (int k = 0; k < M; ++k) {
    const float mr = __shfl_sync(0xffffffffu, re, k), mi = __shfl_sync(0xffffffffu, im, k);
    const float pw = theta[Off::Pw + lane], pb = theta[Off::Pb + lane];
    out[k * C + lane] = make_float2(pw * mr + (k == 0 ? pb * (float)L : 0.f), pw * mi);
  }
}

// ---------------------------------------------------------------------------
// column kernel: per (kx, group of G masks)
//   FWD: V = DFT_y(Xf) at kept ky; U = s R V; Gy = sum_j U e^{+i ky y}
//   BWD: gU = DFT_y(Xg); gV = s conj(R)^T gU; Gg = sum_j gV e^{+i ky y}
// Both y-transforms are real GEMMs on interleaved (re, im) operands, run on the
// tensor cores in TF32 (mma.sync m16n8k8, FP32 accumulate):
//   DFT_y : [2J x 2L] . [2L x C],  rows 2j+ro, K index 2y+ri
//   inverse: [2L x 2J] . [2J x C], rows 2y+ro, K index 2j+ri
// The twiddle operand is generated from a cos/sin table.  The mode weights
// R[.][kx] are read once per CTA for all G masks (FP32 mixing).
// ---------------------------------------------------------------------------
constexpr int COL_G = 4;

__device__ __forceinline__ uint32_t tf32r(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ void mma1688(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

template <bool BWD>
__global__ void __launch_bounds__(THREADS) column_kernel(int L, int B, int G, const float* __restrict__ theta,
                                                         int layer, const float2* __restrict__ Xin,
                                                         float2* __restrict__ Gout, float2* __restrict__ modes_out,
                                                         const float2* __restrict__ twL_g) {
  extern __shared__ __align__(16) unsigned char smraw[];
  float* sX = reinterpret_cast<float*>(smraw);  // [L][C][re,im] tf32; BWD mixing: per-warp transposed R blocks
  float2* sR = reinterpret_cast<float2*>(smraw);
  float2* sTw = reinterpret_cast<float2*>(smraw) + std::max((size_t)L * C, (size_t)(THREADS / 32) * C * (C + 1));
  float2* sV = sTw + L;  // [G][J][C]
  const int kx = blockIdx.x, b0 = blockIdx.y * G, tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5, g = lane >> 2, t = lane & 3;
  const int ng = min(G, B - b0);
  for (int i = tid; i < L; i += THREADS) sTw[i] = twL_g[i];
  // DFT_y tiles: warp -> m-tile (warp >> 1) of 4, n-tiles 2 (warp & 1) .. +1
  const int dmt = warp >> 1, dn0 = 2 * (warp & 1);
  const int jA = 8 * dmt + (g >> 1), roA = g & 1;  // rows g and g + 8 -> j and j + 4
  const int kyA0 = jA < M ? jA : L - J + jA, kyA1 = (jA + 4) < M ? jA + 4 : L - J + jA + 4;
  for (int gi = 0; gi < ng; ++gi) {
    const int b = b0 + gi;
    __syncthreads();
    for (int i = tid; i < L * C; i += THREADS) {
      const int y = i / C, c = i % C;
      const float2 v = Xin[(((size_t)b * L + y) * M + kx) * C + c];
      sX[2 * i] = __uint_as_float(tf32r(v.x));
      sX[2 * i + 1] = __uint_as_float(tf32r(v.y));
    }
    __syncthreads();
    float d[2][4] = {};
    for (int ks = 0; ks < L / 4; ++ks) {  // 8 K entries = 4 y values
      const int y0 = 4 * ks + (t >> 1), y1 = y0 + 2, ri = t & 1;
      // A[m][k]: ro = 0: (cos, sin); ro = 1: (-sin, cos) over ri = 0, 1
      uint32_t a[4];
      {
        const float2 w00 = sTw[(kyA0 * y0) & (L - 1)], w10 = sTw[(kyA1 * y0) & (L - 1)];
        const float2 w01 = sTw[(kyA0 * y1) & (L - 1)], w11 = sTw[(kyA1 * y1) & (L - 1)];
        auto el = [&](float2 w) { return roA == 0 ? (ri == 0 ? w.x : w.y) : (ri == 0 ? -w.y : w.x); };
        a[0] = tf32r(el(w00));
        a[1] = tf32r(el(w10));
        a[2] = tf32r(el(w01));
        a[3] = tf32r(el(w11));
      }
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int c = 8 * (dn0 + q) + g;
        const uint32_t b0r = __float_as_uint(sX[(y0 * C + c) * 2 + ri]);
        const uint32_t b1r = __float_as_uint(sX[(y1 * C + c) * 2 + ri]);
        mma1688(d[q], a, b0r, b1r);
      }
    }
    // D rows m = 16 dmt + g (+8) = 2j + ro, cols c
    float* sVf = reinterpret_cast<float*>(sV + (size_t)gi * J * C);
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int c = 8 * (dn0 + q) + 2 * t;
      sVf[(jA * C + c) * 2 + roA] = d[q][0];
      sVf[(jA * C + c + 1) * 2 + roA] = d[q][1];
      sVf[((jA + 4) * C + c) * 2 + roA] = d[q][2];
      sVf[((jA + 4) * C + c + 1) * 2 + roA] = d[q][3];
    }
  }
  __syncthreads();
  if (modes_out)
    for (int i = tid; i < ng * J * C; i += THREADS) {
      const int gi = i / (J * C), j = (i / C) % J, c = i % C;
      modes_out[(((size_t)(b0 + gi) * J + j) * M + kx) * C + c] = sV[i];
    }
  // mixing: thread (lane = output channel, j = warp + 8 r) for every mask of the group
  const float s = (kx == 0 ? 1.0f : 2.0f) / ((float)L * (float)L);
  const float2* Rl = reinterpret_cast<const float2*>(theta + Off::R + (size_t)layer * Off::RL);
  float2 u[J / 8][COL_G];
#pragma unroll
  for (int r = 0; r < J / 8; ++r)
#pragma unroll
    for (int gg = 0; gg < COL_G; ++gg) u[r][gg] = make_float2(0.f, 0.f);
  float2* sRt = sR + (size_t)warp * C * (C + 1);  // BWD: this warp's block, transposed [o][c] (padded)
#pragma unroll
  for (int r = 0; r < J / 8; ++r) {
    const int j = warp + 8 * r;
    const float2* Rj = Rl + ((size_t)j * M + kx) * C * C;  // [c][o]
    if (!BWD) {  // U[o] = s sum_c R[c][o] V[c]
      for (int c = 0; c < C; ++c) {
        const float2 rr = Rj[c * C + lane];
#pragma unroll
        for (int gg = 0; gg < COL_G; ++gg) {
          if (gg < ng) {
            const float2 v = sV[((size_t)gg * J + j) * C + c];
            u[r][gg].x = fmaf(rr.x, v.x, fmaf(-rr.y, v.y, u[r][gg].x));
            u[r][gg].y = fmaf(rr.x, v.y, fmaf(rr.y, v.x, u[r][gg].y));
          }
        }
      }
    } else {  // gV[c] = s sum_o conj(R[c][o]) gU[o]; lane = c
      __syncwarp();
      for (int c = 0; c < C; ++c) sRt[lane * (C + 1) + c] = Rj[c * C + lane];
      __syncwarp();
      for (int o = 0; o < C; ++o) {
        const float2 rr = sRt[o * (C + 1) + lane];
#pragma unroll
        for (int gg = 0; gg < COL_G; ++gg) {
          if (gg < ng) {
            const float2 v = sV[((size_t)gg * J + j) * C + o];
            u[r][gg].x = fmaf(rr.x, v.x, fmaf(rr.y, v.y, u[r][gg].x));
            u[r][gg].y = fmaf(rr.x, v.y, fmaf(-rr.y, v.x, u[r][gg].y));
          }
        }
      }
    }
  }
  __syncthreads();  // every thread is done reading sV
#pragma unroll
  for (int r = 0; r < J / 8; ++r) {
    const int j = warp + 8 * r;
#pragma unroll
    for (int gg = 0; gg < COL_G; ++gg)
      if (gg < ng)
        sV[((size_t)gg * J + j) * C + lane] = make_float2(__uint_as_float(tf32r(s * u[r][gg].x)),
                                                          __uint_as_float(tf32r(s * u[r][gg].y)));
  }
  __syncthreads();
  // inverse y as [2L x 2J] . [2J x C]: rows m = 2y + ro, K index 2j + ri
  //   ro = 0: (cos, -sin); ro = 1: (sin, cos) over ri = 0, 1
  // warp -> m-tiles warp, warp + 8, ... (2L / 16 = L / 8 of them), all 4 n-tiles
  for (int gi = 0; gi < ng; ++gi) {
    const int b = b0 + gi;
    const float* sUf = reinterpret_cast<const float*>(sV + (size_t)gi * J * C);
    // B fragments of this mask: k-step ks covers j = 4 ks + t/2 (+2), ri = t & 1
    for (int mt = warp; mt < L / 8; mt += THREADS / 32) {
      const int yA = 8 * mt + (g >> 1), ro = g & 1;  // rows g, g + 8 -> y, y + 4
      float d[4][4] = {};
#pragma unroll
      for (int ks = 0; ks < J / 4; ++ks) {
        const int j0 = 4 * ks + (t >> 1), j1 = j0 + 2, ri = t & 1;
        const int ky0 = j0 < M ? j0 : L - J + j0, ky1 = j1 < M ? j1 : L - J + j1;
        const float2 w00 = sTw[(ky0 * yA) & (L - 1)], w10 = sTw[(ky0 * (yA + 4)) & (L - 1)];
        const float2 w01 = sTw[(ky1 * yA) & (L - 1)], w11 = sTw[(ky1 * (yA + 4)) & (L - 1)];
        auto el = [&](float2 w) { return ro == 0 ? (ri == 0 ? w.x : -w.y) : (ri == 0 ? w.y : w.x); };
        uint32_t a[4] = {tf32r(el(w00)), tf32r(el(w10)), tf32r(el(w01)), tf32r(el(w11))};
#pragma unroll
        for (int n = 0; n < 4; ++n) {
          const int c = 8 * n + g;
          mma1688(d[n], a, __float_as_uint(sUf[(j0 * C + c) * 2 + ri]), __float_as_uint(sUf[(j1 * C + c) * 2 + ri]));
        }
      }
      float* go = reinterpret_cast<float*>(Gout);
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        const int c = 8 * n + 2 * t;
        go[((((size_t)b * L + yA) * M + kx) * C + c) * 2 + ro] = d[n][0];
        go[((((size_t)b * L + yA) * M + kx) * C + c + 1) * 2 + ro] = d[n][1];
        go[((((size_t)b * L + yA + 4) * M + kx) * C + c) * 2 + ro] = d[n][2];
        go[((((size_t)b * L + yA + 4) * M + kx) * C + c + 1) * 2 + ro] = d[n][3];
      }
    }
  }
}

size_t column_smem(int L) {
  const size_t x = std::max((size_t)L * C, (size_t)(THREADS / 32) * C * (C + 1));
  return (x + L + (size_t)COL_G * J * C) * sizeof(float2);
}

// ---------------------------------------------------------------------------
// forward row kernel (persistent over rows; the next row's inputs are
// prefetched into registers while the current row is computed)
//   v   = lift(mask) (layer 0) or act_in ? GELU(zin) : zin
//   z_l = W_l v + Wb_l + E(Gy row)
//   zout (optional) = act_out ? GELU(z_l) : z_l
//   !FINAL: Xf = x-DFT(GELU(z_l))        (input of the next column kernel)
//    FINAL: out = Q2 . GELU(Q1 z_3 + q1b) + q2b
// The inverse / forward DFT tables live in shared memory.
// ---------------------------------------------------------------------------
struct RowFwd {
  int L, rows, layer, act_in, act_out;
  const float* theta;
  const float* masks;
  const bf16* zin;
  const float2* Gy;
  bf16* zout;
  float2* Xf;
  float* out;
  const bf16* Ttab;
  const bf16* TT;
};

constexpr int MAXT = 2;  // m-tiles (16 pixels) per warp and row: L <= 256

struct FwdSmem {
  size_t sW, sG, sT, sTT, sVT, sQ1, sQ, total;
  __host__ __device__ static size_t up16(size_t x) { return (x + 15) & ~(size_t)15; }
  __host__ __device__ FwdSmem(int L, bool fin) {
    const size_t LP = (size_t)L + 8;
    size_t o = 0;
    sW = o; o += up16(C * SP * 2);
    sG = o; o += up16(C * SP * 2);
    sT = o; o += up16((size_t)L * SP * 2);
    sTT = sVT = sQ1 = sQ = 0;
    if (!fin) {
      sTT = o; o += up16(J * LP * 2);
      sVT = o; o += up16(C * LP * 2);
    } else {
      sQ1 = o; o += up16(H * SP * 2);
      sQ = o; o += up16(2 * H * sizeof(float));
    }
    total = o;
  }
};

template <bool FINAL>
__global__ void __launch_bounds__(THREADS, 2) row_fwd_kernel(const RowFwd a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int L = a.L, LP = L + 8, l = a.layer, T = L / 16;
  const FwdSmem S(L, FINAL);
  bf16* sW = reinterpret_cast<bf16*>(smraw + S.sW);    // [C o][SP]
  bf16* sG = reinterpret_cast<bf16*>(smraw + S.sG);    // [C c][SP]
  bf16* sT = reinterpret_cast<bf16*>(smraw + S.sT);    // [L px][SP]: inverse table
  bf16* sTT = reinterpret_cast<bf16*>(smraw + S.sTT);  // [J][LP]: forward table
  bf16* sVT = reinterpret_cast<bf16*>(smraw + S.sVT);  // [C][LP]
  bf16* sQ1 = reinterpret_cast<bf16*>(smraw + S.sQ1);  // [H][SP]
  float* sQ = reinterpret_cast<float*>(smraw + S.sQ);  // q1b[H], Q2[H]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  const float* th = a.theta;
  for (int i = tid; i < C * C; i += THREADS) sW[(i / C) * SP + i % C] = __float2bfloat16(th[Off::W + l * C * C + i]);
  for (int i = tid; i < L * J / 2; i += THREADS) {
    const int px = i / (J / 2), k = 2 * (i % (J / 2));
    *reinterpret_cast<uint32_t*>(sT + px * SP + k) = *reinterpret_cast<const uint32_t*>(a.Ttab + (size_t)px * J + k);
  }
  if (!FINAL)
    for (int i = tid; i < J * L / 2; i += THREADS) {
      const int k = i / (L / 2), px = 2 * (i % (L / 2));
      *reinterpret_cast<uint32_t*>(sTT + k * LP + px) = *reinterpret_cast<const uint32_t*>(a.TT + (size_t)k * L + px);
    }
  if (FINAL) {
    for (int i = tid; i < H * C; i += THREADS) sQ1[(i / C) * SP + i % C] = __float2bfloat16(th[Off::Q1 + i]);
    for (int i = tid; i < H; i += THREADS) {
      sQ[i] = th[Off::q1b + i];
      sQ[H + i] = th[Off::Q2 + i];
    }
  }
  float bias[4][2], pw[2][4], pb[2][4];
#pragma unroll
  for (int n = 0; n < 4; ++n) {
    bias[n][0] = th[Off::Wb + l * C + 8 * n + 2 * t];
    bias[n][1] = th[Off::Wb + l * C + 8 * n + 2 * t + 1];
  }
#pragma unroll
  for (int ks = 0; ks < 2; ++ks) {
    const int c0 = 16 * ks + 2 * t;
    pw[ks][0] = th[Off::Pw + c0];     pb[ks][0] = th[Off::Pb + c0];
    pw[ks][1] = th[Off::Pw + c0 + 1]; pb[ks][1] = th[Off::Pb + c0 + 1];
    pw[ks][2] = th[Off::Pw + c0 + 8]; pb[ks][2] = th[Off::Pb + c0 + 8];
    pw[ks][3] = th[Off::Pw + c0 + 9]; pb[ks][3] = th[Off::Pb + c0 + 9];
  }
  const float q2b = th[Off::q2b];

  // register prefetch of one row's inputs
  uint32_t zr[MAXT][8];
  float mr[MAXT][2];
  float2 gr[2];
  auto load_row = [&](int row) {
#pragma unroll
    for (int i = 0; i < MAXT; ++i) {
      const int mt = warp + 8 * i;
      if (mt < T) {
        const int px0 = 16 * mt;
        if (l == 0) {
          mr[i][0] = __ldg(a.masks + (size_t)row * L + px0 + g);
          mr[i][1] = __ldg(a.masks + (size_t)row * L + px0 + g + 8);
        } else {
          const bf16* z0 = a.zin + ((size_t)row * L + px0 + g) * C;
          const bf16* z1 = z0 + 8 * C;
#pragma unroll
          for (int ks = 0; ks < 2; ++ks) {
            const int c0 = 16 * ks + 2 * t;
            zr[i][4 * ks + 0] = ldg32(z0 + c0);
            zr[i][4 * ks + 1] = ldg32(z1 + c0);
            zr[i][4 * ks + 2] = ldg32(z0 + c0 + 8);
            zr[i][4 * ks + 3] = ldg32(z1 + c0 + 8);
          }
        }
      }
    }
    const float2* gp = a.Gy + (size_t)row * M * C;
    gr[0] = __ldg(gp + tid);
    gr[1] = __ldg(gp + tid + THREADS);
  };
  if (blockIdx.x < a.rows) load_row(blockIdx.x);

  for (int row = blockIdx.x; row < a.rows; row += gridDim.x) {
    __syncthreads();  // previous row is done with sG / sVT
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int i = tid + THREADS * q, kx = i / C, c = i % C;
      *reinterpret_cast<uint32_t*>(sG + c * SP + 2 * kx) = pack2(gr[q].x, gr[q].y);
    }
    uint32_t zc[MAXT][8];
    float mc[MAXT][2];
#pragma unroll
    for (int i = 0; i < MAXT; ++i) {
#pragma unroll
      for (int e = 0; e < 8; ++e) zc[i][e] = zr[i][e];
      mc[i][0] = mr[i][0];
      mc[i][1] = mr[i][1];
    }
    if (row + (int)gridDim.x < a.rows) load_row(row + gridDim.x);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < MAXT; ++i) {
      const int mt = warp + 8 * i;
      if (mt >= T) break;
      const int px0 = 16 * mt;
      uint32_t A[2][4];
      if (l == 0) {
        const float m0 = mc[i][0], m1 = mc[i][1];
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
          A[ks][0] = pack2(fmaf(pw[ks][0], m0, pb[ks][0]), fmaf(pw[ks][1], m0, pb[ks][1]));
          A[ks][1] = pack2(fmaf(pw[ks][0], m1, pb[ks][0]), fmaf(pw[ks][1], m1, pb[ks][1]));
          A[ks][2] = pack2(fmaf(pw[ks][2], m0, pb[ks][2]), fmaf(pw[ks][3], m0, pb[ks][3]));
          A[ks][3] = pack2(fmaf(pw[ks][2], m1, pb[ks][2]), fmaf(pw[ks][3], m1, pb[ks][3]));
        }
      } else if (a.act_in) {
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const float2 f = unpack2(zc[i][e]);
          A[e >> 2][e & 3] = pack2(gelu(f.x), gelu(f.y));
        }
      } else {
#pragma unroll
        for (int e = 0; e < 8; ++e) A[e >> 2][e & 3] = zc[i][e];
      }
      float acc[4][4];
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        acc[n][0] = bias[n][0]; acc[n][1] = bias[n][1];
        acc[n][2] = bias[n][0]; acc[n][3] = bias[n][1];
      }
#pragma unroll
      for (int ks = 0; ks < 2; ++ks) {
        uint32_t AT[4];
        const bf16* ta = sT + (px0 + g) * SP + 16 * ks + 2 * t;
        AT[0] = lds32(ta);
        AT[1] = lds32(ta + 8 * SP);
        AT[2] = lds32(ta + 8);
        AT[3] = lds32(ta + 8 * SP + 8);
#pragma unroll
        for (int n = 0; n < 4; ++n) {
          const bf16* bw = sW + (8 * n + g) * SP + 16 * ks + 2 * t;
          mma16816(acc[n], A[ks], lds32(bw), lds32(bw + 8));
          const bf16* bg = sG + (8 * n + g) * SP + 16 * ks + 2 * t;
          mma16816(acc[n], AT, lds32(bg), lds32(bg + 8));
        }
      }
      if (!FINAL) {
        float v[4][4];
#pragma unroll
        for (int n = 0; n < 4; ++n)
#pragma unroll
          for (int e = 0; e < 4; ++e) v[n][e] = gelu(acc[n][e]);
        if (a.zout) {
          bf16* zo0 = a.zout + ((size_t)row * L + px0 + g) * C;
          bf16* zo1 = zo0 + 8 * C;
#pragma unroll
          for (int n = 0; n < 4; ++n) {
            const float* src = a.act_out ? v[n] : acc[n];
            *reinterpret_cast<uint32_t*>(zo0 + 8 * n + 2 * t) = pack2(src[0], src[1]);
            *reinterpret_cast<uint32_t*>(zo1 + 8 * n + 2 * t) = pack2(src[2], src[3]);
          }
        }
#pragma unroll
        for (int n = 0; n < 4; ++n) {
          const int c = 8 * n + 2 * t;
          sVT[c * LP + px0 + g] = __float2bfloat16(v[n][0]);
          sVT[(c + 1) * LP + px0 + g] = __float2bfloat16(v[n][1]);
          sVT[c * LP + px0 + g + 8] = __float2bfloat16(v[n][2]);
          sVT[(c + 1) * LP + px0 + g + 8] = __float2bfloat16(v[n][3]);
        }
      } else {
        if (a.zout) {
          bf16* zo0 = a.zout + ((size_t)row * L + px0 + g) * C;
          bf16* zo1 = zo0 + 8 * C;
#pragma unroll
          for (int n = 0; n < 4; ++n) {
            *reinterpret_cast<uint32_t*>(zo0 + 8 * n + 2 * t) = pack2(acc[n][0], acc[n][1]);
            *reinterpret_cast<uint32_t*>(zo1 + 8 * n + 2 * t) = pack2(acc[n][2], acc[n][3]);
          }
        }
        uint32_t Az[2][4];
        acc_to_a(acc[0], acc[1], Az[0]);
        acc_to_a(acc[2], acc[3], Az[1]);
        float p0 = 0.f, p1 = 0.f;
#pragma unroll 4
        for (int nh = 0; nh < H / 8; ++nh) {
          const int h0 = 8 * nh + 2 * t;
          float hc[4] = {sQ[h0], sQ[h0 + 1], sQ[h0], sQ[h0 + 1]};
#pragma unroll
          for (int ks = 0; ks < 2; ++ks) {
            const bf16* bq = sQ1 + (8 * nh + g) * SP + 16 * ks + 2 * t;
            mma16816(hc, Az[ks], lds32(bq), lds32(bq + 8));
          }
          const float q0 = sQ[H + h0], q1 = sQ[H + h0 + 1];
          p0 = fmaf(q0, gelu(hc[0]), fmaf(q1, gelu(hc[1]), p0));
          p1 = fmaf(q0, gelu(hc[2]), fmaf(q1, gelu(hc[3]), p1));
        }
        p0 += __shfl_xor_sync(0xffffffffu, p0, 1);
        p0 += __shfl_xor_sync(0xffffffffu, p0, 2);
        p1 += __shfl_xor_sync(0xffffffffu, p1, 1);
        p1 += __shfl_xor_sync(0xffffffffu, p1, 2);
        if (t == 0) {
          a.out[(size_t)row * L + px0 + g] = p0 + q2b;
          a.out[(size_t)row * L + px0 + g + 8] = p1 + q2b;
        }
      }
    }
    if (!FINAL) {
      __syncthreads();
      // x-DFT of the row: X[kxri][c] = sum_px TT[kxri][px] v[px][c]; warp -> one 16 x 8 tile
      const int mt2 = warp >> 2, nt = warp & 3;
      float d[4] = {0.f, 0.f, 0.f, 0.f};
      const bf16* ta = sTT + (16 * mt2 + g) * LP + 2 * t;
      const bf16* tb = sVT + (8 * nt + g) * LP + 2 * t;
#pragma unroll 4
      for (int ks = 0; ks < T; ++ks) {
        uint32_t AF[4];
        AF[0] = lds32(ta + 16 * ks);
        AF[1] = lds32(ta + 8 * LP + 16 * ks);
        AF[2] = lds32(ta + 16 * ks + 8);
        AF[3] = lds32(ta + 8 * LP + 16 * ks + 8);
        mma16816(d, AF, lds32(tb + 16 * ks), lds32(tb + 16 * ks + 8));
      }
      float* xf = reinterpret_cast<float*>(a.Xf + (size_t)row * M * C);
      const int k0 = 16 * mt2 + g, c0 = 8 * nt + 2 * t;  // kxri rows k0, k0 + 8
      xf[((k0 >> 1) * C + c0) * 2 + (k0 & 1)] = d[0];
      xf[((k0 >> 1) * C + c0 + 1) * 2 + (k0 & 1)] = d[1];
      xf[(((k0 + 8) >> 1) * C + c0) * 2 + (k0 & 1)] = d[2];
      xf[(((k0 + 8) >> 1) * C + c0 + 1) * 2 + (k0 & 1)] = d[3];
    }
  }
}

size_t row_fwd_smem(int L, bool final_) { return FwdSmem(L, final_).total; }

// ---------------------------------------------------------------------------
// loss: per mask e = ||out - y||, n = ||y||; loss_b = e / n, coef_b = 1 / (B e n)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) loss_kernel(int L, int B, const float* __restrict__ out,
                                                    const float* __restrict__ tgt, float* __restrict__ loss_b,
                                                    float* __restrict__ coef) {
  const int b = blockIdx.x;
  const size_t n = (size_t)L * L;
  const float* o = out + b * n;
  const float* y = tgt + b * n;
  double se = 0.0, sy = 0.0;
  for (size_t i = threadIdx.x; i < n; i += blockDim.x) {
    const double d = (double)o[i] - (double)y[i];
    se += d * d;
    sy += (double)y[i] * (double)y[i];
  }
  __shared__ double r0[32], r1[32];
  for (int k = 16; k > 0; k >>= 1) {
    se += __shfl_xor_sync(0xffffffffu, se, k);
    sy += __shfl_xor_sync(0xffffffffu, sy, k);
  }
  if ((threadIdx.x & 31) == 0) {
    r0[threadIdx.x >> 5] = se;
    r1[threadIdx.x >> 5] = sy;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, c = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a += r0[w];
      c += r1[w];
    }
    const double e = sqrt(a), nn = sqrt(c);
    loss_b[b] = nn > 0.0 ? (float)(e / nn) : 0.f;
    coef[b] = (e > 0.0 && nn > 0.0) ? (float)(1.0 / ((double)B * e * nn)) : 0.f;
  }
}

// ---------------------------------------------------------------------------
// backward row kernel (persistent over rows; per-CTA weight-gradient partials)
//   HEAD_PROJ (layer 3): g_z3 from the projection (dQ1, dq1b, dQ2, dq2b)
//   HEAD_SPEC (layer l < 3): g_z_l = (gvpw_{l+1} + E(Gg_{l+1} row)) * GELU'(z_l)
//   HEAD_LIFT: g_v0 = gvpw_0 + E(Gg_0 row) -> dPw, dPb (no tail)
//   tail (PROJ, SPEC): dW_l += g_z^T v_l, dWb_l += sum g_z, Xg = x-DFT(g_z),
//                      gvpw_l = g_z W_l (bf16)
// ---------------------------------------------------------------------------
enum { HEAD_PROJ = 0, HEAD_SPEC = 1, HEAD_LIFT = 2 };
constexpr int NRED = 2 * H + 2 * C + 1;  // per-warp slots of the vector gradient partials

struct RowBwd {
  int L, rows, layer;
  const float* theta;
  const float* masks;
  const bf16* zl;     // z_l (PROJ: z_3 = v4; SPEC: z_l for GELU')
  const bf16* zlm1;   // z_{l-1} (v_l = GELU(z_{l-1})), unused for l == 0
  const bf16* gvin;   // gvpw_{l+1} (SPEC) / gvpw_0 (LIFT)
  const float2* Gg;   // Gg_{l+1} (SPEC) / Gg_0 (LIFT)
  const float* out;   // PROJ
  const float* tgt;   // PROJ
  const float* coef;  // PROJ [B]
  bf16* gvout;        // gvpw_l
  float2* Xg;         // x-DFT of g_z_l
  float* gpart;       // [gridDim.x][Dn::N]
  const bf16* Ttab;
  const bf16* TT;
};

struct BwdSmem {
  size_t sWT, sG, sGZT, sVT, sQ1, sQ1T, sGHT, sV4T, sT, sTT, sRed, total;
  __host__ __device__ static size_t up16(size_t x) { return (x + 15) & ~(size_t)15; }
  __host__ __device__ BwdSmem(int L, int head) {
    const size_t LP = (size_t)L + 8;
    size_t o = 0;
    sWT = o; o += up16(C * SP * 2);
    sG = o; o += up16(C * SP * 2);
    sGZT = o; o += up16(C * LP * 2);
    sVT = o; o += up16(C * LP * 2);
    sQ1 = sQ1T = sGHT = sV4T = 0;
    if (head == HEAD_PROJ) {
      sQ1 = o; o += up16(H * SP * 2);
      sQ1T = o; o += up16(C * (H + 8) * 2);
      sGHT = o; o += up16(H * LP * 2);
      sV4T = o; o += up16(C * LP * 2);
    }
    sT = sTT = 0;
    if (head != HEAD_PROJ) { sT = o; o += up16((size_t)L * SP * 2); }
    if (head != HEAD_LIFT) { sTT = o; o += up16(J * LP * 2); }
    sRed = o; o += up16((size_t)(THREADS / 32) * NRED * sizeof(float));
    total = o;
  }
};

template <int HEAD>
__global__ void __launch_bounds__(THREADS, 1) row_bwd_kernel(const RowBwd a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int L = a.L, LP = L + 8, l = a.layer;
  const BwdSmem S(L, HEAD);
  bf16* sWT = reinterpret_cast<bf16*>(smraw + S.sWT);    // [C c][SP]: W_l[o][c] at [c][o]
  bf16* sG = reinterpret_cast<bf16*>(smraw + S.sG);      // [C c][SP]
  bf16* sGZT = reinterpret_cast<bf16*>(smraw + S.sGZT);  // [C o][LP]
  bf16* sVT = reinterpret_cast<bf16*>(smraw + S.sVT);    // [C c][LP]
  bf16* sQ1 = reinterpret_cast<bf16*>(smraw + S.sQ1);    // [H][SP]
  bf16* sQ1T = reinterpret_cast<bf16*>(smraw + S.sQ1T);  // [C][H + 8]
  bf16* sGHT = reinterpret_cast<bf16*>(smraw + S.sGHT);  // [H][LP]
  bf16* sV4T = reinterpret_cast<bf16*>(smraw + S.sV4T);  // [C][LP]
  float* sRed = reinterpret_cast<float*>(smraw + S.sRed);
  bf16* sT = reinterpret_cast<bf16*>(smraw + S.sT);      // [L px][SP]: inverse table
  bf16* sTT = reinterpret_cast<bf16*>(smraw + S.sTT);    // [J][LP]: forward table
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  const float* th = a.theta;
  constexpr int HP = H + 8;
  if (HEAD != HEAD_PROJ)
    for (int i = tid; i < L * J / 2; i += THREADS) {
      const int px = i / (J / 2), k = 2 * (i % (J / 2));
      *reinterpret_cast<uint32_t*>(sT + px * SP + k) = *reinterpret_cast<const uint32_t*>(a.Ttab + (size_t)px * J + k);
    }
  if (HEAD != HEAD_LIFT)
    for (int i = tid; i < J * L / 2; i += THREADS) {
      const int k = i / (L / 2), px = 2 * (i % (L / 2));
      *reinterpret_cast<uint32_t*>(sTT + k * LP + px) = *reinterpret_cast<const uint32_t*>(a.TT + (size_t)k * L + px);
    }

  if (HEAD != HEAD_LIFT)
    for (int i = tid; i < C * C; i += THREADS) {
      const int o = i / C, c = i % C;
      sWT[c * SP + o] = __float2bfloat16(th[Off::W + l * C * C + i]);
    }
  if (HEAD == HEAD_PROJ)
    for (int i = tid; i < H * C; i += THREADS) {
      const int h = i / C, c = i % C;
      const bf16 v = __float2bfloat16(th[Off::Q1 + i]);
      sQ1[h * SP + c] = v;
      sQ1T[c * HP + h] = v;
    }
  for (int i = tid; i < (THREADS / 32) * NRED; i += THREADS) sRed[i] = 0.f;
  float pw[2][4], pb[2][4];
#pragma unroll
  for (int ks = 0; ks < 2; ++ks) {
    const int c0 = 16 * ks + 2 * t;
    pw[ks][0] = th[Off::Pw + c0];     pb[ks][0] = th[Off::Pb + c0];
    pw[ks][1] = th[Off::Pw + c0 + 1]; pb[ks][1] = th[Off::Pb + c0 + 1];
    pw[ks][2] = th[Off::Pw + c0 + 8]; pb[ks][2] = th[Off::Pb + c0 + 8];
    pw[ks][3] = th[Off::Pw + c0 + 9]; pb[ks][3] = th[Off::Pb + c0 + 9];
  }
  // per-thread partial sums over rows g, g+8 (columns 8n + 2t, +1)
  float vb[4][2] = {};       // dWb (tail) or dPb (LIFT)
  float vw[4][2] = {};       // dPw (LIFT)
  float dq1b[16][2] = {}, dq2[16][2] = {};
  float dq2b = 0.f;
  float dW[4] = {0.f, 0.f, 0.f, 0.f};  // warp's 16 x 8 tile of dW_l
  float dQ1[4][4] = {};                // warp's four 16 x 8 tiles of dQ1

  for (int row = blockIdx.x; row < a.rows; row += gridDim.x) {
    const int b = row / L;
    __syncthreads();
    if (HEAD != HEAD_PROJ) stage_g_row(a.Gg + (size_t)row * M * C, sG, tid);
    __syncthreads();
    for (int mt = warp; mt < L / 16; mt += THREADS / 32) {
      const int px0 = 16 * mt;
      const size_t p0 = (size_t)row * L + px0 + g, p1 = p0 + 8;
      float gz[4][4];
      if (HEAD == HEAD_PROJ) {
        // v4 = z_3 as an A fragment, and transposed into sV4T for dQ1
        uint32_t A[2][4];
        const bf16* z0 = a.zl + p0 * C;
        const bf16* z1 = a.zl + p1 * C;
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
          const int c0 = 16 * ks + 2 * t;
          A[ks][0] = ldg32(z0 + c0);
          A[ks][1] = ldg32(z1 + c0);
          A[ks][2] = ldg32(z0 + c0 + 8);
          A[ks][3] = ldg32(z1 + c0 + 8);
          const bf16* e0 = reinterpret_cast<const bf16*>(&A[ks][0]);
          const bf16* e1 = reinterpret_cast<const bf16*>(&A[ks][1]);
          const bf16* e2 = reinterpret_cast<const bf16*>(&A[ks][2]);
          const bf16* e3 = reinterpret_cast<const bf16*>(&A[ks][3]);
          sV4T[c0 * LP + px0 + g] = e0[0];       sV4T[(c0 + 1) * LP + px0 + g] = e0[1];
          sV4T[c0 * LP + px0 + g + 8] = e1[0];   sV4T[(c0 + 1) * LP + px0 + g + 8] = e1[1];
          sV4T[(c0 + 8) * LP + px0 + g] = e2[0]; sV4T[(c0 + 9) * LP + px0 + g] = e2[1];
          sV4T[(c0 + 8) * LP + px0 + g + 8] = e3[0];
          sV4T[(c0 + 9) * LP + px0 + g + 8] = e3[1];
        }
        const float go0 = (a.out[p0] - a.tgt[p0]) * a.coef[b];
        const float go1 = (a.out[p1] - a.tgt[p1]) * a.coef[b];
        if (t == 0) dq2b += go0 + go1;
#pragma unroll
        for (int n = 0; n < 4; ++n) gz[n][0] = gz[n][1] = gz[n][2] = gz[n][3] = 0.f;
#pragma unroll
        for (int kh = 0; kh < H / 16; ++kh) {  // hidden channels 16 kh .. 16 kh + 15
          float hc[2][4];
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            const int nh = 2 * kh + u, h0 = 8 * nh + 2 * t;
            const float b0 = th[Off::q1b + h0], b1 = th[Off::q1b + h0 + 1];
            hc[u][0] = b0; hc[u][1] = b1; hc[u][2] = b0; hc[u][3] = b1;
#pragma unroll
            for (int ks = 0; ks < 2; ++ks) {
              const bf16* bq = sQ1 + (8 * nh + g) * SP + 16 * ks + 2 * t;
              mma16816(hc[u], A[ks], lds32(bq), lds32(bq + 8));
            }
            const float q0 = th[Off::Q2 + h0], q1 = th[Off::Q2 + h0 + 1];
            // gh = go * Q2; ghp = gh * GELU'(hpre)
            float ga[4], gd[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) gelu_both(hc[u][e], ga[e], gd[e]);
            const float g00 = go0 * q0 * gd[0], g01 = go0 * q1 * gd[1];
            const float g10 = go1 * q0 * gd[2], g11 = go1 * q1 * gd[3];
            dq2[nh][0] += go0 * ga[0] + go1 * ga[2];
            dq2[nh][1] += go0 * ga[1] + go1 * ga[3];
            dq1b[nh][0] += g00 + g10;
            dq1b[nh][1] += g01 + g11;
            hc[u][0] = g00; hc[u][1] = g01; hc[u][2] = g10; hc[u][3] = g11;
            sGHT[h0 * LP + px0 + g] = __float2bfloat16(g00);
            sGHT[(h0 + 1) * LP + px0 + g] = __float2bfloat16(g01);
            sGHT[h0 * LP + px0 + g + 8] = __float2bfloat16(g10);
            sGHT[(h0 + 1) * LP + px0 + g + 8] = __float2bfloat16(g11);
          }
          uint32_t AG[4];
          acc_to_a(hc[0], hc[1], AG);
#pragma unroll
          for (int n = 0; n < 4; ++n) {  // g_v4 += ghp Q1: B[k = h][n = c] = Q1T[c][h]
            const bf16* bq = sQ1T + (8 * n + g) * HP + 16 * kh + 2 * t;
            mma16816(gz[n], AG, lds32(bq), lds32(bq + 8));
          }
        }
      } else {
        // g_v = gvin + E(G row)
        const bf16* v0 = a.gvin + p0 * C;
        const bf16* v1 = a.gvin + p1 * C;
#pragma unroll
        for (int n = 0; n < 4; ++n) {
          const float2 f0 = unpack2(ldg32(v0 + 8 * n + 2 * t)), f1 = unpack2(ldg32(v1 + 8 * n + 2 * t));
          gz[n][0] = f0.x; gz[n][1] = f0.y; gz[n][2] = f1.x; gz[n][3] = f1.y;
        }
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
          uint32_t AT[4];
          const bf16* ta = sT + (px0 + g) * SP + 16 * ks + 2 * t;
          AT[0] = lds32(ta);
          AT[1] = lds32(ta + 8 * SP);
          AT[2] = lds32(ta + 8);
          AT[3] = lds32(ta + 8 * SP + 8);
#pragma unroll
          for (int n = 0; n < 4; ++n) {
            const bf16* bg = sG + (8 * n + g) * SP + 16 * ks + 2 * t;
            mma16816(gz[n], AT, lds32(bg), lds32(bg + 8));
          }
        }
        if (HEAD == HEAD_LIFT) {
          const float m0 = a.masks[p0], m1 = a.masks[p1];
#pragma unroll
          for (int n = 0; n < 4; ++n) {
            vb[n][0] += gz[n][0] + gz[n][2];
            vb[n][1] += gz[n][1] + gz[n][3];
            vw[n][0] += gz[n][0] * m0 + gz[n][2] * m1;
            vw[n][1] += gz[n][1] * m0 + gz[n][3] * m1;
          }
          continue;
        }
        // g_z_l = g_v * GELU'(z_l)
        const bf16* z0 = a.zl + p0 * C;
        const bf16* z1 = a.zl + p1 * C;
#pragma unroll
        for (int n = 0; n < 4; ++n) {
          const float2 f0 = unpack2(ldg32(z0 + 8 * n + 2 * t)), f1 = unpack2(ldg32(z1 + 8 * n + 2 * t));
          gz[n][0] *= gelu_grad(f0.x); gz[n][1] *= gelu_grad(f0.y);
          gz[n][2] *= gelu_grad(f1.x); gz[n][3] *= gelu_grad(f1.y);
        }
      }
      // ---- tail: g_z_l in gz (C layout) ----
      // v_l for dW_l (transposed into sVT)
      if (l == 0) {
        const float m0 = a.masks[p0], m1 = a.masks[p1];
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
          const int c0 = 16 * ks + 2 * t;
          const int cs[4] = {c0, c0 + 1, c0 + 8, c0 + 9};
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            sVT[cs[q] * LP + px0 + g] = __float2bfloat16(fmaf(pw[ks][q], m0, pb[ks][q]));
            sVT[cs[q] * LP + px0 + g + 8] = __float2bfloat16(fmaf(pw[ks][q], m1, pb[ks][q]));
          }
        }
      } else {
        const bf16* z0 = a.zlm1 + p0 * C;
        const bf16* z1 = a.zlm1 + p1 * C;
#pragma unroll
        for (int n = 0; n < 4; ++n) {
          const int c = 8 * n + 2 * t;
          const float2 f0 = unpack2(ldg32(z0 + c)), f1 = unpack2(ldg32(z1 + c));
          sVT[c * LP + px0 + g] = __float2bfloat16(gelu(f0.x));
          sVT[(c + 1) * LP + px0 + g] = __float2bfloat16(gelu(f0.y));
          sVT[c * LP + px0 + g + 8] = __float2bfloat16(gelu(f1.x));
          sVT[(c + 1) * LP + px0 + g + 8] = __float2bfloat16(gelu(f1.y));
        }
      }
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        const int o = 8 * n + 2 * t;
        vb[n][0] += gz[n][0] + gz[n][2];
        vb[n][1] += gz[n][1] + gz[n][3];
        sGZT[o * LP + px0 + g] = __float2bfloat16(gz[n][0]);
        sGZT[(o + 1) * LP + px0 + g] = __float2bfloat16(gz[n][1]);
        sGZT[o * LP + px0 + g + 8] = __float2bfloat16(gz[n][2]);
        sGZT[(o + 1) * LP + px0 + g + 8] = __float2bfloat16(gz[n][3]);
      }
      // gvpw_l = g_z W_l: B[k = o][n = c] = W[o][c] = sWT[c][o]
      {
        uint32_t AZ[2][4];
        acc_to_a(gz[0], gz[1], AZ[0]);
        acc_to_a(gz[2], gz[3], AZ[1]);
        bf16* w0 = a.gvout + p0 * C;
        bf16* w1 = a.gvout + p1 * C;
#pragma unroll
        for (int n = 0; n < 4; ++n) {
          float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
          for (int ks = 0; ks < 2; ++ks) {
            const bf16* bw = sWT + (8 * n + g) * SP + 16 * ks + 2 * t;
            mma16816(d, AZ[ks], lds32(bw), lds32(bw + 8));
          }
          *reinterpret_cast<uint32_t*>(w0 + 8 * n + 2 * t) = pack2(d[0], d[1]);
          *reinterpret_cast<uint32_t*>(w1 + 8 * n + 2 * t) = pack2(d[2], d[3]);
        }
      }
    }
    if (HEAD == HEAD_LIFT) continue;
    __syncthreads();
    {
      const int mt2 = warp >> 2, nt = warp & 3;
      // dW_l tile (o rows 16 mt2.., c cols 8 nt..) += sum_px gz^T v
      const bf16* pa = sGZT + (16 * mt2 + g) * LP + 2 * t;
      const bf16* pbv = sVT + (8 * nt + g) * LP + 2 * t;
      // Xg tile (kxri rows 16 mt2.., o cols 8 nt..) = sum_px TT gz
      const bf16* ta = sTT + (16 * mt2 + g) * LP + 2 * t;
      const bf16* pbz = sGZT + (8 * nt + g) * LP + 2 * t;
      float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
      for (int ks = 0; ks < L / 16; ++ks) {
        const int k = 16 * ks;
        uint32_t AF[4];
        AF[0] = lds32(pa + k);
        AF[1] = lds32(pa + 8 * LP + k);
        AF[2] = lds32(pa + k + 8);
        AF[3] = lds32(pa + 8 * LP + k + 8);
        mma16816(dW, AF, lds32(pbv + k), lds32(pbv + k + 8));
        AF[0] = lds32(ta + k);
        AF[1] = lds32(ta + 8 * LP + k);
        AF[2] = lds32(ta + k + 8);
        AF[3] = lds32(ta + 8 * LP + k + 8);
        mma16816(d, AF, lds32(pbz + k), lds32(pbz + k + 8));
      }
      float* xg = reinterpret_cast<float*>(a.Xg + (size_t)row * M * C);
      const int k0 = 16 * mt2 + g, c0 = 8 * nt + 2 * t;
      xg[((k0 >> 1) * C + c0) * 2 + (k0 & 1)] = d[0];
      xg[((k0 >> 1) * C + c0 + 1) * 2 + (k0 & 1)] = d[1];
      xg[(((k0 + 8) >> 1) * C + c0) * 2 + (k0 & 1)] = d[2];
      xg[(((k0 + 8) >> 1) * C + c0 + 1) * 2 + (k0 & 1)] = d[3];
    }
    if (HEAD == HEAD_PROJ) {
      // dQ1 tiles (h rows, c cols) += sum_px ghp^T v4; warp -> tiles 4 warp .. 4 warp + 3
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int tile = 4 * warp + q, mh = tile >> 2, nt = tile & 3;
        const bf16* pa = sGHT + (16 * mh + g) * LP + 2 * t;
        const bf16* pbv = sV4T + (8 * nt + g) * LP + 2 * t;
        for (int ks = 0; ks < L / 16; ++ks) {
          const int k = 16 * ks;
          uint32_t AF[4];
          AF[0] = lds32(pa + k);
          AF[1] = lds32(pa + 8 * LP + k);
          AF[2] = lds32(pa + k + 8);
          AF[3] = lds32(pa + 8 * LP + k + 8);
          mma16816(dQ1[q], AF, lds32(pbv + k), lds32(pbv + k + 8));
        }
      }
    }
  }

  // ---- per-CTA partials ----
  float* gp = a.gpart + (size_t)blockIdx.x * Dn::N;
  // vector partials: reduce over g (lanes xor 4, 8, 16), then over warps in a fixed
  // order (per-warp slots), so that the gradient is bitwise reproducible
  auto red_g = [&](float v) {
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 8);
    v += __shfl_xor_sync(0xffffffffu, v, 16);
    return v;
  };
  float* myRed = sRed + warp * NRED;
  __syncthreads();
#pragma unroll
  for (int n = 0; n < 4; ++n)
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const float s0 = red_g(vb[n][e]);
      const float s1 = red_g(vw[n][e]);
      if (g == 0) {
        myRed[8 * n + 2 * t + e] = s0;
        myRed[C + 8 * n + 2 * t + e] = s1;
      }
    }
  if (HEAD == HEAD_PROJ) {
#pragma unroll
    for (int nh = 0; nh < 16; ++nh)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const float s0 = red_g(dq1b[nh][e]);
        const float s1 = red_g(dq2[nh][e]);
        if (g == 0) {
          myRed[2 * C + 8 * nh + 2 * t + e] = s0;
          myRed[2 * C + H + 8 * nh + 2 * t + e] = s1;
        }
      }
    float s = dq2b;
    for (int k = 16; k > 0; k >>= 1) s += __shfl_xor_sync(0xffffffffu, s, k);
    if (lane == 0) myRed[2 * C + 2 * H] = s;
  }
  __syncthreads();
  for (int i = tid; i < NRED; i += THREADS) {
    float s = 0.f;
    for (int w = 0; w < THREADS / 32; ++w) s += sRed[w * NRED + i];
    sRed[i] = s;  // slot 0 of warp 0 is read only by this thread
  }
  __syncthreads();
  if constexpr (HEAD == HEAD_LIFT) {
    for (int i = tid; i < C; i += THREADS) {
      gp[Dn::Pb + i] = sRed[i];
      gp[Dn::Pw + i] = sRed[C + i];
    }
    return;
  } else {
    for (int i = tid; i < C; i += THREADS) gp[Dn::Wb + l * C + i] = sRed[i];
    {
      const int mt2 = warp >> 2, nt = warp & 3;
      const int o = 16 * mt2 + g, c = 8 * nt + 2 * t;
      float* w = gp + Dn::W + l * C * C;
      w[o * C + c] = dW[0];
      w[o * C + c + 1] = dW[1];
      w[(o + 8) * C + c] = dW[2];
      w[(o + 8) * C + c + 1] = dW[3];
    }
    if (HEAD == HEAD_PROJ) {
      for (int i = tid; i < H; i += THREADS) {
        gp[Dn::q1b + i] = sRed[2 * C + i];
        gp[Dn::Q2 + i] = sRed[2 * C + H + i];
      }
      if (tid == 0) gp[Dn::q2b] = sRed[2 * C + 2 * H];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int tile = 4 * warp + q, mh = tile >> 2, nt = tile & 3;
        const int h = 16 * mh + g, c = 8 * nt + 2 * t;
        float* w = gp + Dn::Q1;
        w[h * C + c] = dQ1[q][0];
        w[h * C + c + 1] = dQ1[q][1];
        w[(h + 8) * C + c] = dQ1[q][2];
        w[(h + 8) * C + c + 1] = dQ1[q][3];
      }
    }
  }  // HEAD != HEAD_LIFT
}

// dense partials -> gradient vector
__global__ void reduce_dense_kernel(const float* __restrict__ gpart, int nparts, float* __restrict__ grad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Dn::N) return;
  float s = 0.f;
  for (int p = 0; p < nparts; ++p) s += gpart[(size_t)p * Dn::N + i];
  grad[dense_to_param(i)] = s;
}

// dR[j][kx][c][o] = s_kx sum_b gU_b[j][kx][o] conj(V_b[j][kx][c]); one CTA per (j, kx)
__global__ void __launch_bounds__(THREADS) dR_kernel(int L, int B, int layer, const float2* __restrict__ gU,
                                                     const float2* __restrict__ V, float* __restrict__ grad) {
  const int jk = blockIdx.x, tid = threadIdx.x;  // jk = j * M + kx
  const int kx = jk % M;
  __shared__ float2 su[C], sv[C];
  float2 acc[4] = {};
  for (int b = 0; b < B; ++b) {
    __syncthreads();
    if (tid < C) su[tid] = gU[((size_t)b * J * M + jk) * C + tid];
    else if (tid < 2 * C) sv[tid - C] = V[((size_t)b * J * M + jk) * C + tid - C];
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int idx = tid + THREADS * r, c = idx / C, o = idx % C;
      const float2 u = su[o], v = sv[c];
      acc[r].x += u.x * v.x + u.y * v.y;
      acc[r].y += u.y * v.x - u.x * v.y;
    }
  }
  const float s = (kx == 0 ? 1.0f : 2.0f) / ((float)L * (float)L);
  float2* out = reinterpret_cast<float2*>(grad + Off::R + (size_t)layer * Off::RL) + (size_t)jk * C * C;
#pragma unroll
  for (int r = 0; r < 4; ++r) out[tid + THREADS * r] = make_float2(s * acc[r].x, s * acc[r].y);
}

// Adam (torch semantics: L2 weight decay added to the gradient)
__global__ void adam_kernel(size_t n, float* __restrict__ p, const float* __restrict__ gr, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float eps, float wd, float bc1,
                            float bc2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float g = gr[i] + wd * p[i];
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  }
}

// ---------------------------------------------------------------------------
// seeded rectangle masks (SplitMix64 counters); one CTA per mask
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t splitmix(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void rect_masks_kernel(uint64_t seed, long long first, int L, int nmin, int nmax, int wmin, int wmax,
                                  float* __restrict__ out) {
  __shared__ int4 rc[256];
  __shared__ int nr;
  const uint64_t i = (uint64_t)(first + blockIdx.x);
  const uint64_t base = seed * 0xD1B54A32D192ED03ull + i * 0x9E3779B97F4A7C15ull;
  if (threadIdx.x == 0) nr = nmin + (int)(splitmix(base) % (uint64_t)(nmax - nmin + 1));
  __syncthreads();
  const uint64_t span = (uint64_t)(wmax - wmin + 1);
  for (int r = threadIdx.x; r < nr; r += blockDim.x) {
    const int w = wmin + (int)(splitmix(base + 1 + 4 * r) % span);
    const int h = wmin + (int)(splitmix(base + 2 + 4 * r) % span);
    const int x0 = (int)(splitmix(base + 3 + 4 * r) % (uint64_t)(L - w + 1));
    const int y0 = (int)(splitmix(base + 4 + 4 * r) % (uint64_t)(L - h + 1));
    rc[r] = make_int4(x0, y0, x0 + w, y0 + h);
  }
  __syncthreads();
  float* m = out + (size_t)blockIdx.x * L * L;
  for (int p = threadIdx.x; p < L * L; p += blockDim.x) {
    const int y = p / L, x = p % L;
    float v = 0.f;
    for (int r = 0; r < nr; ++r) {
      const int4 q = rc[r];
      if (x >= q.x && x < q.z && y >= q.y && y < q.w) {
        v = 1.f;
        break;
      }
    }
    m[p] = v;
  }
}

// ---------------------------------------------------------------------------
// band projection of an image onto |kx| <= KB, |ky| <= KBy (the support of any
// SOCS image with kernels of half-width Nx = KB/2, Ny = KBy/2) and its
// out-of-band residual, the surrogate's error estimate.
// ---------------------------------------------------------------------------
// x-DFT of each row at kx = 0..KB (KB <= 15); one warp per row
__global__ void __launch_bounds__(THREADS) band_rows_kernel(int L, int rows, int KB, const float* __restrict__ img,
                                                            const float2* __restrict__ twL, float2* __restrict__ Xb) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row = blockIdx.x * (THREADS / 32) + warp;
  if (row >= rows) return;
  const float* m = img + (size_t)row * L;
  const int kx = lane & 15, half = lane >> 4;
  float re = 0.f, im = 0.f;
  for (int px = half; px < L; px += 2) {
    const float v = m[px];
    const float2 w = twL[(kx * px) & (L - 1)];
    re = fmaf(v, w.x, re);
    im = fmaf(-v, w.y, im);
  }
  re += __shfl_xor_sync(0xffffffffu, re, 16);
  im += __shfl_xor_sync(0xffffffffu, im, 16);
  if (half == 0 && kx <= KB) Xb[(size_t)row * 16 + kx] = make_float2(re, im);
}

// per mask: C[ky + KBy][kx] = sum_y X[y][kx] e^{-i ky y} for kx <= KB, |ky| <= KBy (plain 2-D DFT)
__global__ void __launch_bounds__(THREADS) band_coef_kernel(int L, int KB, int KBy, const float2* __restrict__ Xb,
                                                            const float2* __restrict__ twL, float2* __restrict__ Cb) {
  const int b = blockIdx.x;
  const int nky = 2 * KBy + 1, ncoef = nky * (KB + 1);
  for (int q = threadIdx.x; q < ncoef; q += blockDim.x) {
    const int kyi = q / (KB + 1), kx = q % (KB + 1), ky = kyi - KBy;
    float re = 0.f, im = 0.f;
    for (int y = 0; y < L; ++y) {
      const float2 x = Xb[((size_t)b * L + y) * 16 + kx];
      const float2 w = twL[((ky + L) * y) & (L - 1)];  // e^{+i ky y}; use conj
      re = fmaf(x.x, w.x, fmaf(x.y, w.y, re));
      im = fmaf(x.y, w.x, fmaf(-x.x, w.y, im));
    }
    Cb[(size_t)b * nky * 16 + kyi * 16 + kx] = make_float2(re, im);
  }
}

// in-place synthesis of the band: img[y][x] = 1/L^2 sum_kx w_kx Re(G_y[kx] e^{i kx x}),
// G_y[kx] = sum_ky Cb[ky][kx] e^{i ky y}; per-row energies of the removed part and of the result.
// One CTA per row.
__global__ void __launch_bounds__(THREADS) band_synth_kernel(int L, int KB, int KBy, const float2* __restrict__ Cb,
                                                             const float2* __restrict__ twL, float* __restrict__ img,
                                                             float* __restrict__ Eres, float* __restrict__ Enew) {
  const int row = blockIdx.x, b = row / L, y = row % L, tid = threadIdx.x;
  const int nky = 2 * KBy + 1;
  __shared__ float2 G[16];
  __shared__ float r0[THREADS / 32], r1[THREADS / 32];
  if (tid <= KB) {
    float re = 0.f, im = 0.f;
    for (int kyi = 0; kyi < nky; ++kyi) {
      const int ky = kyi - KBy;
      const float2 c = Cb[(size_t)b * nky * 16 + kyi * 16 + tid];
      const float2 w = twL[((ky + L) * y) & (L - 1)];
      re = fmaf(c.x, w.x, fmaf(-c.y, w.y, re));
      im = fmaf(c.x, w.y, fmaf(c.y, w.x, im));
    }
    const float sc = (tid == 0 ? 1.f : 2.f) / ((float)L * (float)L);
    G[tid] = make_float2(sc * re, sc * im);
  }
  __syncthreads();
  float er = 0.f, en = 0.f;
  for (int x = tid; x < L; x += THREADS) {
    float v = 0.f;
    for (int kx = 0; kx <= KB; ++kx) {
      const float2 w = twL[(kx * x) & (L - 1)];
      v = fmaf(G[kx].x, w.x, fmaf(-G[kx].y, w.y, v));
    }
    const size_t i = (size_t)row * L + x;
    const float d = img[i] - v;
    er = fmaf(d, d, er);
    en = fmaf(v, v, en);
    img[i] = v;
  }
  for (int k = 16; k > 0; k >>= 1) {
    er += __shfl_xor_sync(0xffffffffu, er, k);
    en += __shfl_xor_sync(0xffffffffu, en, k);
  }
  if ((tid & 31) == 0) {
    r0[tid >> 5] = er;
    r1[tid >> 5] = en;
  }
  __syncthreads();
  if (tid == 0) {
    float a = 0.f, c = 0.f;
    for (int w = 0; w < THREADS / 32; ++w) {
      a += r0[w];
      c += r1[w];
    }
    Eres[row] = a;
    Enew[row] = c;
  }
}

// est[b] = alpha * sqrt(sum_rows Eres / sum_rows Enew)
__global__ void oob_est_kernel(int L, int B, const float* __restrict__ Eres, const float* __restrict__ Enew,
                               float alpha, float* __restrict__ est) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  double a = 0.0, c = 0.0;
  for (int y = 0; y < L; ++y) {
    a += Eres[(size_t)b * L + y];
    c += Enew[(size_t)b * L + y];
  }
  est[b] = c > 0.0 ? (float)(alpha * sqrt(a / c)) : INFINITY;
}

// Exact image coefficients at the five lowest frequencies q in {(0,0), (1,0), (0,1),
// (1,1), (-1,1)} (with their conjugates the 3 x 3 lowest block):
//   I(q) = 1/L^2 sum_k s_k sum_f B_k(f + q) conj(B_k(f)),  B_k(f) = krn_k(f) M(f),
// M the plain DFT of the mask on the (2Nx+1) x (2Ny+1) window (Cm holds u >= 0).
// est[b] = alpha * sqrt(sum_q w_q |I_net(q) - I(q)|^2 / L^2) / ||image||, w = 1 at DC, 2 else.
// One CTA per mask.
__global__ void __launch_bounds__(128) lowq_est_kernel(int L, int Nx, int Ny, const float2* __restrict__ Cm,
                                                       const float2* __restrict__ Cb, const float2* __restrict__ krn,
                                                       const float* __restrict__ scales, int nk,
                                                       const float* __restrict__ Enew, float alpha,
                                                       float* __restrict__ est) {
  const int b = blockIdx.x, tid = threadIdx.x;
  const int KX = 2 * Nx + 1, KY = 2 * Ny + 1, KD = KX * KY;
  __shared__ float2 sM[33 * 33];
  __shared__ float2 part[5][64];
  __shared__ double en;
  for (int i = tid; i < KD; i += blockDim.x) {
    const int v = i / KX - Ny, u = i % KX - Nx;
    float2 m;
    if (u >= 0) {
      m = Cm[((size_t)b * KY + (v + Ny)) * 16 + u];
    } else {
      const float2 c = Cm[((size_t)b * KY + (-v + Ny)) * 16 + (-u)];
      m = make_float2(c.x, -c.y);
    }
    sM[i] = m;
  }
  if (tid == 0) {
    double a = 0.0;
    for (int y = 0; y < L; ++y) a += Enew[(size_t)b * L + y];
    en = a;
  }
  __syncthreads();
  const int qx[5] = {0, 1, 0, 1, -1}, qy[5] = {0, 0, 1, 1, 1};
  for (int p = tid; p < 5 * 64; p += blockDim.x) {
    const int qi = p / 64, k = p % 64;
    float re = 0.f, im = 0.f;
    if (k < nk) {
      const float2* kk = krn + (size_t)k * KD;
      for (int i = 0; i < KD; ++i) {
        const int v = i / KX - Ny, u = i % KX - Nx;
        const int v2 = v + qy[qi], u2 = u + qx[qi];
        if (v2 < -Ny || v2 > Ny || u2 < -Nx || u2 > Nx) continue;
        const int j = (v2 + Ny) * KX + (u2 + Nx);
        const float2 a = cmulf(kk[j], sM[j]), c = cmulf(kk[i], sM[i]);
        re = fmaf(a.x, c.x, fmaf(a.y, c.y, re));   // a conj(c)
        im = fmaf(a.y, c.x, fmaf(-a.x, c.y, im));
      }
      re *= scales[k];
      im *= scales[k];
    }
    part[qi][k] = make_float2(re, im);
  }
  __syncthreads();
  if (tid < 32) {
    float d2 = 0.f;
    for (int qi = 0; qi < 5; ++qi) {
      float re = part[qi][tid].x + part[qi][tid + 32].x, im = part[qi][tid].y + part[qi][tid + 32].y;
      for (int k = 16; k > 0; k >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, k);
        im += __shfl_xor_sync(0xffffffffu, im, k);
      }
      const float inv = 1.0f / ((float)L * (float)L);
      re *= inv;
      im *= inv;
      float2 net;
      const int KBy = 2 * Ny;
      if (qx[qi] >= 0) {
        net = Cb[((size_t)b * (2 * KBy + 1) + (qy[qi] + KBy)) * 16 + qx[qi]];
      } else {
        const float2 c = Cb[((size_t)b * (2 * KBy + 1) + (-qy[qi] + KBy)) * 16 + (-qx[qi])];
        net = make_float2(c.x, -c.y);
      }
      const float dr = net.x - re, di = net.y - im;
      d2 += (qi == 0 ? 1.f : 2.f) * (dr * dr + di * di);
    }
    if (tid == 0) {
      const double e = sqrt((double)d2) / (double)L;
      est[b] = en > 0.0 ? (float)(alpha * e / sqrt(en)) : INFINITY;
    }
  }
}

}  // namespace fno
}  // namespace litho

// ===========================================================================
// host side
// ===========================================================================
using namespace litho;
using namespace litho::fno;

struct litho_fno {
  litho_ctx* ctx = nullptr;
  int L = 0;
  int cap = 0;  // batch capacity of the workspaces
  long long step = 0;
  DevBuf theta, grad, adam_m, adam_v;
  DevBuf Ttab, TT, twL;
  DevBuf z[NL];      // z_l (training keeps all; inference ping-pongs z[0], z[1])
  DevBuf Xf, Gy;     // per-row spectral intermediates (also Xg, Gg in backward)
  DevBuf Vs[NL], gU;
  DevBuf gv[2];      // gvpw ping-pong
  DevBuf out, lossb, coef, gpart;
  int bwd_grid = 0;
  // error estimate = alpha * ||out-of-band residual|| / ||band part||
  float est_alpha = 1.0f;
  DevBuf Xb, Eres, Enew, Cb, Mrow, Cm, est, stage_m, stage_i;
};

namespace {

int fno_grid(litho_fno* f, int rows) { return std::max(1, std::min(rows, 2 * f->ctx->sm_count)); }

// masks per column-kernel CTA: enough CTAs for two per SM, at most COL_G
int col_group(litho_fno* f, int B) { return std::max(1, std::min(COL_G, B * M / (2 * f->ctx->sm_count))); }

int ensure_batch(litho_fno* f, int B, bool train) {
  litho_ctx* ctx = f->ctx;
  const size_t L = f->L;
  const size_t act = (size_t)B * L * L * C * sizeof(bf16);
  const size_t row = (size_t)B * L * M * C * sizeof(float2);
  for (int l = 0; l < (train ? NL : 2); ++l) LITHO_RET(f->z[l].ensure(ctx, act));
  LITHO_RET(f->Xf.ensure(ctx, row));
  LITHO_RET(f->Gy.ensure(ctx, row));
  LITHO_RET(f->out.ensure(ctx, (size_t)B * L * L * sizeof(float)));
  LITHO_RET(f->lossb.ensure(ctx, (size_t)B * sizeof(float)));
  LITHO_RET(f->coef.ensure(ctx, (size_t)B * sizeof(float)));
  if (train) {
    for (int l = 0; l < NL; ++l) LITHO_RET(f->Vs[l].ensure(ctx, (size_t)B * J * M * C * sizeof(float2)));
    LITHO_RET(f->gU.ensure(ctx, (size_t)B * J * M * C * sizeof(float2)));
    LITHO_RET(f->gv[0].ensure(ctx, act));
    LITHO_RET(f->gv[1].ensure(ctx, act));
    f->bwd_grid = fno_grid(f, (int)(B * L));
    LITHO_RET(f->gpart.ensure(ctx, (size_t)f->bwd_grid * Dn::N * sizeof(float)));
  }
  return LITHO_OK;
}

int set_smem(litho_ctx* ctx, const void* fn, size_t bytes) {
  LITHO_CUDA_TRY(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return LITHO_OK;
}

// forward pass over B masks; train keeps z_l and V_l for the backward pass
int forward(litho_fno* f, const float* masks, int B, bool train, float* images, float2* Mrow = nullptr) {
  litho_ctx* ctx = f->ctx;
  const int L = f->L, rows = B * L;
  const float* th = f->theta.as<float>();
  const size_t csm = column_smem(L);
  LITHO_RET(set_smem(ctx, (const void*)column_kernel<false>, csm));
  LITHO_RET(set_smem(ctx, (const void*)row_fwd_kernel<false>, row_fwd_smem(L, false)));
  LITHO_RET(set_smem(ctx, (const void*)row_fwd_kernel<true>, row_fwd_smem(L, true)));
  StageScope sc(ctx, LITHO_STAGE_SURROGATE, 2 * NL + 1);
  lift_dft_kernel<<<(rows + 7) / 8, THREADS, 0, ctx->stream>>>(L, rows, th, masks, f->twL.as<float2>(),
                                                               f->Xf.as<float2>(), Mrow);
  const int grid = fno_grid(f, rows);
  const int G = col_group(f, B);
  for (int l = 0; l < NL; ++l) {
    column_kernel<false><<<dim3(M, (B + G - 1) / G), THREADS, csm, ctx->stream>>>(
        L, B, G, th, l, f->Xf.as<float2>(), f->Gy.as<float2>(), train ? f->Vs[l].as<float2>() : nullptr,
        f->twL.as<float2>());
    RowFwd a;
    a.L = L; a.rows = rows; a.layer = l; a.theta = th; a.masks = masks;
    a.act_in = train ? 1 : 0;   // training keeps z_l, inference keeps GELU(z_l)
    a.act_out = train ? 0 : 1;
    a.zin = l == 0 ? nullptr : (train ? f->z[l - 1].as<bf16>() : f->z[(l - 1) & 1].as<bf16>());
    a.Gy = f->Gy.as<float2>();
    a.zout = train ? f->z[l].as<bf16>() : (l < NL - 1 ? f->z[l & 1].as<bf16>() : nullptr);
    a.Xf = f->Xf.as<float2>();
    a.out = images;
    a.Ttab = f->Ttab.as<bf16>(); a.TT = f->TT.as<bf16>();
    if (l < NL - 1)
      row_fwd_kernel<false><<<grid, THREADS, row_fwd_smem(L, false), ctx->stream>>>(a);
    else
      row_fwd_kernel<true><<<grid, THREADS, row_fwd_smem(L, true), ctx->stream>>>(a);
  }
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  return LITHO_OK;
}

// loss (device, per mask) + gradient into f->grad
int backward(litho_fno* f, const float* masks, const float* targets, int B) {
  litho_ctx* ctx = f->ctx;
  const int L = f->L, rows = B * L, grid = f->bwd_grid;
  const float* th = f->theta.as<float>();
  const size_t csm = column_smem(L);
  LITHO_RET(set_smem(ctx, (const void*)column_kernel<true>, csm));
  const BwdSmem sp(L, HEAD_PROJ), ss(L, HEAD_SPEC), sl(L, HEAD_LIFT);
  LITHO_RET(set_smem(ctx, (const void*)row_bwd_kernel<HEAD_PROJ>, sp.total));
  LITHO_RET(set_smem(ctx, (const void*)row_bwd_kernel<HEAD_SPEC>, ss.total));
  LITHO_RET(set_smem(ctx, (const void*)row_bwd_kernel<HEAD_LIFT>, sl.total));
  const int G = col_group(f, B);
  StageScope sc(ctx, LITHO_STAGE_SURROGATE, 3 * NL + 3);
  loss_kernel<<<B, 1024, 0, ctx->stream>>>(L, B, f->out.as<float>(), targets, f->lossb.as<float>(),
                                           f->coef.as<float>());
  LITHO_CUDA_TRY(ctx, cudaMemsetAsync(f->gpart.p, 0, (size_t)grid * Dn::N * sizeof(float), ctx->stream));
  float2* Xg = f->Xf.as<float2>();
  float2* Gg = f->Gy.as<float2>();
  RowBwd a{};
  a.L = L; a.rows = rows; a.theta = th; a.masks = masks;
  a.out = f->out.as<float>(); a.tgt = targets; a.coef = f->coef.as<float>();
  a.Xg = Xg; a.Gg = Gg; a.gpart = f->gpart.as<float>();
  a.Ttab = f->Ttab.as<bf16>(); a.TT = f->TT.as<bf16>();
  int cur = 0;
  for (int l = NL - 1; l >= 0; --l) {
    a.layer = l;
    a.zl = f->z[l].as<bf16>();
    a.zlm1 = l > 0 ? f->z[l - 1].as<bf16>() : nullptr;
    a.gvin = f->gv[cur ^ 1].as<bf16>();
    a.gvout = f->gv[cur].as<bf16>();
    if (l == NL - 1)
      row_bwd_kernel<HEAD_PROJ><<<grid, THREADS, sp.total, ctx->stream>>>(a);
    else
      row_bwd_kernel<HEAD_SPEC><<<grid, THREADS, ss.total, ctx->stream>>>(a);
    column_kernel<true><<<dim3(M, (B + G - 1) / G), THREADS, csm, ctx->stream>>>(L, B, G, th, l, Xg, Gg,
                                                                                  f->gU.as<float2>(),
                                                                                  f->twL.as<float2>());
    dR_kernel<<<J * M, THREADS, 0, ctx->stream>>>(L, B, l, f->gU.as<float2>(), f->Vs[l].as<float2>(),
                                                  f->grad.as<float>());
    cur ^= 1;
  }
  a.layer = 0;
  a.gvin = f->gv[cur ^ 1].as<bf16>();
  row_bwd_kernel<HEAD_LIFT><<<grid, THREADS, sl.total, ctx->stream>>>(a);
  reduce_dense_kernel<<<(Dn::N + 255) / 256, 256, 0, ctx->stream>>>(f->gpart.as<float>(), grid,
                                                                    f->grad.as<float>());
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  return LITHO_OK;
}

// band projection of `images` onto |kx| <= 2Nx, |ky| <= 2Ny (in place) -> f->Cb, f->Eres, f->Enew
int project(litho_fno* f, int Nx, int Ny, float* images, int batch) {
  litho_ctx* ctx = f->ctx;
  const int L = f->L, rows = batch * L, KB = 2 * Nx, KBy = 2 * Ny;
  LITHO_RET(f->Xb.ensure(ctx, (size_t)rows * 16 * sizeof(float2)));
  LITHO_RET(f->Eres.ensure(ctx, (size_t)rows * sizeof(float)));
  LITHO_RET(f->Enew.ensure(ctx, (size_t)rows * sizeof(float)));
  LITHO_RET(f->Cb.ensure(ctx, (size_t)batch * (2 * KBy + 1) * 16 * sizeof(float2)));
  StageScope sc(ctx, LITHO_STAGE_SURROGATE, 3);
  band_rows_kernel<<<(rows + 7) / 8, THREADS, 0, ctx->stream>>>(L, rows, KB, images, f->twL.as<float2>(),
                                                                f->Xb.as<float2>());
  band_coef_kernel<<<batch, THREADS, 0, ctx->stream>>>(L, KB, KBy, f->Xb.as<float2>(), f->twL.as<float2>(),
                                                       f->Cb.as<float2>());
  band_synth_kernel<<<rows, THREADS, 0, ctx->stream>>>(L, KB, KBy, f->Cb.as<float2>(), f->twL.as<float2>(), images,
                                                       f->Eres.as<float>(), f->Enew.as<float>());
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  return LITHO_OK;
}

// network -> band projection -> exact low-frequency check (est on the device)
int predict(litho_fno* f, const litho_kernel_set* ks, const float* masks, int batch, float* images, float* est) {
  litho_ctx* ctx = f->ctx;
  const int L = f->L, rows = batch * L;
  LITHO_RET(ensure_batch(f, batch, false));
  LITHO_RET(f->Mrow.ensure(ctx, (size_t)rows * 16 * sizeof(float2)));
  LITHO_RET(f->Cm.ensure(ctx, (size_t)batch * (2 * ks->Ny + 1) * 16 * sizeof(float2)));
  LITHO_RET(forward(f, masks, batch, false, images, f->Mrow.as<float2>()));
  LITHO_RET(project(f, ks->Nx, ks->Ny, images, batch));
  StageScope sc(ctx, LITHO_STAGE_SURROGATE, 2);
  band_coef_kernel<<<batch, THREADS, 0, ctx->stream>>>(L, ks->Nx, ks->Ny, f->Mrow.as<float2>(), f->twL.as<float2>(),
                                                       f->Cm.as<float2>());
  lowq_est_kernel<<<batch, 128, 0, ctx->stream>>>(L, ks->Nx, ks->Ny, f->Cm.as<float2>(), f->Cb.as<float2>(), ks->krn,
                                                  ks->scales, ks->nk, f->Enew.as<float>(), f->est_alpha, est);
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  return LITHO_OK;
}

// Kaiming-uniform linear layers and FNO spectral weights (scale/(in*out) * U[0,1))
void init_params(std::vector<float>& p, unsigned long long seed) {
  std::mt19937_64 rng(seed);
  auto uni = [&](float lo, float hi) {
    return lo + (hi - lo) * (float)((rng() >> 11) * (1.0 / 9007199254740992.0));
  };
  p.assign(Off::N, 0.f);
  for (int i = 0; i < C; ++i) p[Off::Pw + i] = uni(-1.f, 1.f);
  for (int i = 0; i < C; ++i) p[Off::Pb + i] = uni(-1.f, 1.f);
  const float bw = 1.0f / std::sqrt((float)C);
  for (int l = 0; l < NL; ++l) {
    for (int i = 0; i < C * C; ++i) p[Off::W + (size_t)l * C * C + i] = uni(-bw, bw);
    for (int i = 0; i < C; ++i) p[Off::Wb + (size_t)l * C + i] = uni(-bw, bw);
  }
  const float sc = 1.0f / (float)(C * C);
  for (size_t i = 0; i < NL * Off::RL; ++i) p[Off::R + i] = sc * uni(0.f, 1.f);
  for (int i = 0; i < H * C; ++i) p[Off::Q1 + i] = uni(-bw, bw);
  for (int i = 0; i < H; ++i) p[Off::q1b + i] = uni(-bw, bw);
  const float bh = 1.0f / std::sqrt((float)H);
  for (int i = 0; i < H; ++i) p[Off::Q2 + i] = uni(-bh, bh);
  p[Off::q2b] = uni(-bh, bh);
}

}  // namespace

extern "C" {

long long litho_surrogate_num_params(void) { return (long long)Off::N; }

int litho_surrogate_create(litho_ctx* ctx, int L, unsigned long long seed, litho_fno** out) {
  if (ctx == nullptr || out == nullptr) return LITHO_ERR_ARG;
  *out = nullptr;
  LITHO_ARG_CHECK(ctx, L == 64 || L == 128 || L == 256, "surrogate grid L=%d must be 64, 128 or 256", L);
  LITHO_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  litho_fno* f = new litho_fno;
  f->ctx = ctx;
  f->L = L;
  int rc = LITHO_OK;
  do {
    const size_t pb = Off::N * sizeof(float);
    if ((rc = f->theta.ensure(ctx, pb)) || (rc = f->grad.ensure(ctx, pb)) || (rc = f->adam_m.ensure(ctx, pb)) ||
        (rc = f->adam_v.ensure(ctx, pb)))
      break;
    if ((rc = f->Ttab.ensure(ctx, (size_t)L * J * sizeof(bf16))) || (rc = f->TT.ensure(ctx, (size_t)L * J * sizeof(bf16))) ||
        (rc = f->twL.ensure(ctx, (size_t)L * sizeof(float2))))
      break;
    std::vector<float> p;
    init_params(p, seed);
    if (cudaMemcpyAsync(f->theta.p, p.data(), pb, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        cudaMemsetAsync(f->adam_m.p, 0, pb, ctx->stream) != cudaSuccess ||
        cudaMemsetAsync(f->adam_v.p, 0, pb, ctx->stream) != cudaSuccess ||
        cudaMemsetAsync(f->grad.p, 0, pb, ctx->stream) != cudaSuccess) {
      set_error(ctx, LITHO_ERR_CUDA, "surrogate parameter upload failed");
      rc = LITHO_ERR_CUDA;
      break;
    }
    tables_kernel<<<(L * M + 255) / 256, 256, 0, ctx->stream>>>(L, f->Ttab.as<bf16>(), f->TT.as<bf16>(),
                                                               f->twL.as<float2>());
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
      set_error(ctx, LITHO_ERR_CUDA, "surrogate table setup failed");
      rc = LITHO_ERR_CUDA;
    }
  } while (0);
  if (rc != LITHO_OK) {
    litho_surrogate_destroy(f);
    return rc;
  }
  *out = f;
  return LITHO_OK;
}

void litho_surrogate_destroy(litho_fno* f) {
  if (!f) return;
  DevBuf* bufs[] = {&f->theta, &f->grad, &f->adam_m, &f->adam_v, &f->Ttab, &f->TT, &f->twL, &f->Xf, &f->Gy,
                    &f->gU, &f->gv[0], &f->gv[1], &f->out, &f->lossb, &f->coef, &f->gpart, &f->Xb, &f->Eres,
                    &f->Enew, &f->Cb, &f->Mrow, &f->Cm, &f->est, &f->stage_m, &f->stage_i};
  for (DevBuf* b : bufs) b->release();
  for (int l = 0; l < NL; ++l) {
    f->z[l].release();
    f->Vs[l].release();
  }
  delete f;
}

int litho_surrogate_get_params(litho_fno* f, float* host, long long n) {
  if (!f || !host) return LITHO_ERR_ARG;
  litho_ctx* ctx = f->ctx;
  LITHO_ARG_CHECK(ctx, n == (long long)Off::N, "expected %lld parameters", (long long)Off::N);
  LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(host, f->theta.p, Off::N * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  LITHO_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return LITHO_OK;
}

int litho_surrogate_set_params(litho_fno* f, const float* host, long long n) {
  if (!f || !host) return LITHO_ERR_ARG;
  litho_ctx* ctx = f->ctx;
  LITHO_ARG_CHECK(ctx, n == (long long)Off::N, "expected %lld parameters", (long long)Off::N);
  const size_t pb = Off::N * sizeof(float);
  LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(f->theta.p, host, pb, cudaMemcpyHostToDevice, ctx->stream));
  LITHO_CUDA_TRY(ctx, cudaMemsetAsync(f->adam_m.p, 0, pb, ctx->stream));
  LITHO_CUDA_TRY(ctx, cudaMemsetAsync(f->adam_v.p, 0, pb, ctx->stream));
  LITHO_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  f->step = 0;
  return LITHO_OK;
}

int litho_surrogate_forward(litho_fno* f, const float* masks, int batch, float* images) {
  if (!f) return LITHO_ERR_ARG;
  litho_ctx* ctx = f->ctx;
  LITHO_ARG_CHECK(ctx, masks && images && batch >= 1, "bad argument");
  LITHO_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  LITHO_RET(ensure_batch(f, batch, false));
  return forward(f, masks, batch, false, images);
}

int litho_surrogate_loss_grad(litho_fno* f, const float* masks, const float* targets, int batch, float* loss,
                              float* grad_host) {
  if (!f || !masks || !targets || batch < 1) return LITHO_ERR_ARG;
  litho_ctx* ctx = f->ctx;
  LITHO_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  LITHO_RET(ensure_batch(f, batch, true));
  LITHO_RET(forward(f, masks, batch, true, f->out.as<float>()));
  LITHO_RET(backward(f, masks, targets, batch));
  if (loss) {
    std::vector<float> lb(batch);
    LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(lb.data(), f->lossb.p, batch * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    LITHO_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    double s = 0.0;
    for (float v : lb) s += v;
    *loss = (float)(s / batch);
  }
  if (grad_host) {
    LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(grad_host, f->grad.p, Off::N * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    LITHO_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return LITHO_OK;
}

int litho_surrogate_train_step(litho_fno* f, const float* masks, const float* targets, int batch, float lr,
                               float weight_decay, float* loss) {
  if (!f || !masks || !targets || batch < 1) return LITHO_ERR_ARG;
  litho_ctx* ctx = f->ctx;
  LITHO_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  LITHO_RET(ensure_batch(f, batch, true));
  LITHO_RET(forward(f, masks, batch, true, f->out.as<float>()));
  LITHO_RET(backward(f, masks, targets, batch));
  f->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.f - (float)std::pow((double)b1, (double)f->step);
  const float bc2 = 1.f - (float)std::pow((double)b2, (double)f->step);
  {
    StageScope sc(ctx, LITHO_STAGE_SURROGATE);
    adam_kernel<<<4 * ctx->sm_count, 256, 0, ctx->stream>>>(Off::N, f->theta.as<float>(), f->grad.as<float>(),
                                                            f->adam_m.as<float>(), f->adam_v.as<float>(), lr, b1, b2,
                                                            1e-8f, weight_decay, bc1, bc2);
  }
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  if (loss) {
    std::vector<float> lb(batch);
    LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(lb.data(), f->lossb.p, batch * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    LITHO_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    double s = 0.0;
    for (float v : lb) s += v;
    *loss = (float)(s / batch);
  }
  return LITHO_OK;
}

int litho_rect_masks(litho_ctx* ctx, unsigned long long seed, long long first, int count, int L, int nmin, int nmax,
                     int wmin, int wmax, float* masks) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  LITHO_ARG_CHECK(ctx, masks && count >= 1 && L >= 1, "bad argument");
  LITHO_ARG_CHECK(ctx, nmin >= 0 && nmax >= nmin && nmax <= 256, "rectangle count range [%d, %d] (max 256)", nmin, nmax);
  LITHO_ARG_CHECK(ctx, wmin >= 1 && wmax >= wmin && wmax <= L, "rectangle side range [%d, %d] for L=%d", wmin, wmax, L);
  LITHO_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  rect_masks_kernel<<<count, 256, 0, ctx->stream>>>((uint64_t)seed, first, L, nmin, nmax, wmin, wmax, masks);
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  return LITHO_OK;
}

int litho_surrogate_set_alpha(litho_fno* f, float alpha) {
  if (!f) return LITHO_ERR_ARG;
  LITHO_ARG_CHECK(f->ctx, alpha > 0.f && std::isfinite(alpha), "alpha must be positive");
  f->est_alpha = alpha;
  return LITHO_OK;
}

float litho_surrogate_get_alpha(const litho_fno* f) { return f ? f->est_alpha : 0.f; }

int litho_surrogate_project(litho_fno* f, int Nx, int Ny, float* images, int batch, float* est) {
  if (!f) return LITHO_ERR_ARG;
  litho_ctx* ctx = f->ctx;
  const int L = f->L;
  LITHO_ARG_CHECK(ctx, images && est && batch >= 1, "bad argument");
  LITHO_ARG_CHECK(ctx, Nx >= 0 && Ny >= 0 && 2 * Nx <= 15 && 2 * Ny <= 15, "band half-widths Nx=%d Ny=%d unsupported (2 N <= 15)", Nx, Ny);
  LITHO_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  LITHO_RET(project(f, Nx, Ny, images, batch));
  StageScope sc(ctx, LITHO_STAGE_SURROGATE);
  oob_est_kernel<<<(batch + 127) / 128, 128, 0, ctx->stream>>>(L, batch, f->Eres.as<float>(), f->Enew.as<float>(),
                                                               f->est_alpha, est);
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  return LITHO_OK;
}

int litho_surrogate_predict(litho_fno* f, const litho_kernel_set* ks, const float* masks, int batch, float* images,
                            float* est) {
  if (!f) return LITHO_ERR_ARG;
  litho_ctx* ctx = f->ctx;
  LITHO_ARG_CHECK(ctx, ks && masks && images && est && batch >= 1, "bad argument");
  LITHO_ARG_CHECK(ctx, ks->ctx == ctx, "kernel set belongs to another context");
  LITHO_ARG_CHECK(ctx, 2 * ks->Nx <= 15 && 2 * ks->Ny <= 15 && ks->nk <= 64,
                  "estimator needs 2 Nx, 2 Ny <= 15 and nk <= 64 (Nx=%d Ny=%d nk=%d)", ks->Nx, ks->Ny, ks->nk);
  LITHO_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  return predict(f, ks, masks, batch, images, est);
}

int litho_surrogate_image(litho_fno* f, const litho_kernel_set* ks, const float* masks, int batch, float threshold,
                          float* images, float* est_host, int* used_socs) {
  if (!f) return LITHO_ERR_ARG;
  litho_ctx* ctx = f->ctx;
  const int L = f->L;
  LITHO_ARG_CHECK(ctx, ks && masks && images && batch >= 1, "bad argument");
  LITHO_ARG_CHECK(ctx, ks->ctx == ctx, "kernel set belongs to another context");
  LITHO_ARG_CHECK(ctx, 2 * ks->Nx <= 15 && 2 * ks->Ny <= 15 && ks->nk <= 64,
                  "estimator needs 2 Nx, 2 Ny <= 15 and nk <= 64 (Nx=%d Ny=%d nk=%d)", ks->Nx, ks->Ny, ks->nk);
  LITHO_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  LITHO_RET(f->est.ensure(ctx, (size_t)batch * sizeof(float)));
  LITHO_RET(predict(f, ks, masks, batch, images, f->est.as<float>()));
  std::vector<float> est(batch);
  LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(est.data(), f->est.p, batch * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  LITHO_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  std::vector<int> rej;
  for (int b = 0; b < batch; ++b) {
    const bool r = !(est[b] <= threshold);  // NaN rejects
    if (r) rej.push_back(b);
    if (used_socs) used_socs[b] = r ? 1 : 0;
    if (est_host) est_host[b] = est[b];
  }
  if (!rej.empty()) {
    const int n = (int)rej.size();
    const size_t img = (size_t)L * L * sizeof(float);
    LITHO_RET(f->stage_m.ensure(ctx, n * img));
    LITHO_RET(f->stage_i.ensure(ctx, n * img));
    for (int i = 0; i < n; ++i)
      LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(f->stage_m.as<char>() + i * img, reinterpret_cast<const char*>(masks) + rej[i] * img,
                                          img, cudaMemcpyDeviceToDevice, ctx->stream));
    const ImgGeom g{L, L, L, L, ks->Nx, ks->Ny, ks->nk, default_conv_n(ks->Nx, ks->Ny)};
    LITHO_RET(image_pipeline(ctx, g, n, f->stage_m.as<float>(), ks, f->stage_i.as<float>(),
                             LITHO_PREC_FP32));
    for (int i = 0; i < n; ++i)
      LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(reinterpret_cast<char*>(images) + rej[i] * img, f->stage_i.as<char>() + i * img,
                                          img, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  return LITHO_OK;
}

}  // extern "C"
