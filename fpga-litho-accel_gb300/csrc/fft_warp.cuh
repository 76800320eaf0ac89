// Warp-level radix-2 FFTs held in registers and exchanged with warp shuffles.
//
// A length-N vector (N = 32*J, J = 1, 2, 4) is spread over one warp: the element
// at position i = lane + 32*j lives in register x[j] of lane `lane`.  Stages whose
// butterfly span is >= 32 are register butterflies inside a lane; spans < 32 are
// done with __shfl_xor_sync.
//
//   warp_fft_dif : natural-order input  -> bit-reversed-order output
//   warp_fft_dit : bit-reversed input   -> natural-order output
//
// Chaining DIF (inverse) with DIT (forward) needs no reordering pass at all: the
// SOCS stage transforms the kernel*mask product with DIF, accumulates |E|^2 in
// bit-reversed order (a pointwise operation), and transforms the intensity back
// with DIT, which lands in natural frequency order.
//
// tw[e] = exp(-2*pi*i*e/N) for e in [0, N/2) (forward convention); INV selects
// the conjugate (exp(+2*pi*i*e/N), FFTW_BACKWARD, unnormalised).
#pragma once
#include <cuda_runtime.h>

namespace litho {

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 shfl_xor2(float2 v, int m) {
  return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

template <bool INV>
__device__ __forceinline__ float2 twid(const float2* tw, int e) {
  float2 t = tw[e];
  if (INV) t.y = -t.y;
  return t;
}

template <int N, bool INV>
__device__ __forceinline__ void warp_fft_dif(float2 (&x)[N / 32], const float2* __restrict__ tw, int lane) {
  constexpr int J = N / 32;
#pragma unroll
  for (int hj = J / 2; hj >= 1; hj >>= 1) {
    const int h = 32 * hj;
#pragma unroll
    for (int j = 0; j < J; ++j) {
      if ((j & hj) == 0) {
        const int i = lane + 32 * j;
        const int e = (i & (2 * h - 1)) * (N / (2 * h));
        const float2 a = x[j], b = x[j + hj];
        x[j] = cadd(a, b);
        x[j + hj] = cmul(csub(a, b), twid<INV>(tw, e));
      }
    }
  }
  // shuffle stages, branch-free: with s = +1 (top) / -1 (bottom) and w' = 1 (top) /
  // w (bottom), both halves are (s x + p) w': two FMAs and a complex product per
  // element instead of both butterfly halves and a select
#pragma unroll
  for (int h = 16; h >= 1; h >>= 1) {
    const bool bottom = (lane & h) != 0;
    const float s = bottom ? -1.f : 1.f;
    const float2 w = bottom ? twid<INV>(tw, (lane & (h - 1)) * (N / (2 * h))) : make_float2(1.f, 0.f);
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const float2 p = shfl_xor2(x[j], h);
      x[j] = cmul(make_float2(fmaf(s, x[j].x, p.x), fmaf(s, x[j].y, p.y)), w);
    }
  }
}

template <int N, bool INV>
__device__ __forceinline__ void warp_fft_dit(float2 (&x)[N / 32], const float2* __restrict__ tw, int lane) {
  constexpr int J = N / 32;
  // shuffle stages, branch-free: the bottom lane pre-multiplies its element by w
  // (the top lane by 1) before the exchange; then both halves are s z + p_z with
  // s = +1 (top) / -1 (bottom)
#pragma unroll
  for (int h = 1; h <= 16; h <<= 1) {
    const bool bottom = (lane & h) != 0;
    const float s = bottom ? -1.f : 1.f;
    const float2 w = bottom ? twid<INV>(tw, (lane & (h - 1)) * (N / (2 * h))) : make_float2(1.f, 0.f);
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const float2 z = cmul(w, x[j]);
      const float2 p = shfl_xor2(z, h);
      x[j] = make_float2(fmaf(s, z.x, p.x), fmaf(s, z.y, p.y));
    }
  }
#pragma unroll
  for (int hj = 1; hj <= J / 2; hj <<= 1) {
    const int h = 32 * hj;
#pragma unroll
    for (int j = 0; j < J; ++j) {
      if ((j & hj) == 0) {
        const int i = lane + 32 * j;
        const int e = (i & (2 * h - 1)) * (N / (2 * h));
        const float2 t = cmul(twid<INV>(tw, e), x[j + hj]);
        x[j + hj] = csub(x[j], t);
        x[j] = cadd(x[j], t);
      }
    }
  }
}

constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n >> 1); }

// bit reversal of an index in [0, N), N a power of two
template <int N>
__device__ __forceinline__ int bitrev(int i) {
  return (int)(__brev((unsigned)i) >> (32 - ilog2(N)));
}

}  // namespace litho
