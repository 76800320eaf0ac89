// 64-point FFTs on groups of eight lanes (four transforms per warp, natural order
// in and out) and 128-point FFTs on groups of sixteen lanes built from them.
//
// Lane t (t = lane & 7) of a group holds x[r] = v[t + 8r], r = 0..7.  The
// transform is the 8 x 8 Cooley-Tukey split of 64 = 8 * 8:
//   1. an 8-point DFT over r in registers:  Y_t[k1] = sum_r v[t + 8r] W8^(r k1)
//   2. the twiddle W64^(t k1) on Y_t[k1]
//   3. an 8 x 8 transpose inside the group through shared memory: lane k1 gets
//      Y_s[k1] W64^(s k1) for s = 0..7
//   4. an 8-point DFT over s:  V[k1 + 8 k2] = sum_s Y_s[k1] W64^(s k1) W8^(s k2)
// so lane t ends holding V[t + 8 k2] in register k2.  Against a radix-2 warp
// transform (five shuffle stages of two shuffles, a twiddle product and two FMAs
// per element) this is one store and one load per element plus two 8-point DFTs
// whose only non-trivial factors are (+-1 +- i)/sqrt(2).
//
// Transpose scratch: 72 float2 per group, rows of 9.  A store (fixed k1, lanes t)
// covers 16 consecutive banks and the two groups of a half-warp sit 16 banks
// apart (72 float2 = 144 words = 16 mod 32); a load (fixed s, lanes t, stride 9
// float2 = 18 words) hits banks 18t mod 32, again disjoint between the two
// groups: every access is conflict-free.
//
// W64^e = exp(-2 pi i e / 64) (forward); INV selects the conjugate (backward,
// unnormalised, the FFTW_BACKWARD convention).
#pragma once
#include <cuda_runtime.h>

#include "fft_warp.cuh"

namespace litho {

constexpr int L8_SCR = 72;  // transpose scratch per group of eight lanes (float2)

// complex add / subtract as one packed f32x2 add (per component the same as the
// scalar adds; a - b is a + (-b), exact)
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }

// a * conj(w)
__device__ __forceinline__ float2 cmul_conj(float2 a, float2 w) {
  return make_float2(fmaf(a.x, w.x, a.y * w.y), fmaf(a.y, w.x, -a.x * w.y));
}

// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 mul_mi(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// 8-point DFT in place, natural order in and out (radix-2 decimation in frequency
// with the output permutation done by register naming)
template <bool INV>
__device__ __forceinline__ void dft8(float2 (&x)[8]) {
  constexpr float R = 0.70710678118654752f;  // 1 / sqrt(2)
  const float2 a0 = padd(x[0], x[4]), b0 = psub(x[0], x[4]);
  const float2 a1 = padd(x[1], x[5]), d1 = psub(x[1], x[5]);
  const float2 a2 = padd(x[2], x[6]), d2 = psub(x[2], x[6]);
  const float2 a3 = padd(x[3], x[7]), d3 = psub(x[3], x[7]);
  // b_n = (x_n - x_{n+4}) W8^n: W8 = (1 - i)/sqrt2, W8^2 = -i, W8^3 = (-1 - i)/sqrt2 (forward)
  const float2 b1 = INV ? make_float2((d1.x - d1.y) * R, (d1.x + d1.y) * R)
                        : make_float2((d1.x + d1.y) * R, (d1.y - d1.x) * R);
  const float2 b2 = mul_mi<INV>(d2);
  const float2 b3 = INV ? make_float2(-(d3.x + d3.y) * R, (d3.x - d3.y) * R)
                        : make_float2((d3.y - d3.x) * R, -(d3.x + d3.y) * R);
  // even outputs: 4-point DFT of a; odd outputs: 4-point DFT of b
  const float2 c0 = padd(a0, a2), e0 = psub(a0, a2);
  const float2 c1 = padd(a1, a3), e1 = mul_mi<INV>(psub(a1, a3));
  const float2 f0 = padd(b0, b2), g0 = psub(b0, b2);
  const float2 f1 = padd(b1, b3), g1 = mul_mi<INV>(psub(b1, b3));
  x[0] = padd(c0, c1);
  x[4] = psub(c0, c1);
  x[2] = padd(e0, e1);
  x[6] = psub(e0, e1);
  x[1] = padd(f0, f1);
  x[5] = psub(f0, f1);
  x[3] = padd(g0, g1);
  x[7] = psub(g0, g1);
}

// per-lane twiddles w[k] = W64^(t k), k = 0..7, from tw[e] = W64^e (e < 32)
__device__ __forceinline__ void lane8_twiddles(float2 (&w)[8], const float2* tw, int t) {
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int e = t * k;  // < 50
    const float2 v = tw[e & 31];
    w[k] = e < 32 ? v : make_float2(-v.x, -v.y);
  }
}

// 64-point transform of the group's vector (see the header); scr: the group's
// L8_SCR float2 of shared memory.  Every lane of the warp must call it.
template <bool INV>
__device__ __forceinline__ void fft64_lane8(float2 (&x)[8], const float2 (&w)[8], float2* scr, int t) {
  dft8<INV>(x);
#pragma unroll
  for (int k = 1; k < 8; ++k) x[k] = INV ? cmul_conj(x[k], w[k]) : cmul(x[k], w[k]);
#pragma unroll
  for (int k = 0; k < 8; ++k) scr[k * 9 + t] = x[k];
  __syncwarp();
#pragma unroll
  for (int s = 0; s < 8; ++s) x[s] = scr[t * 9 + s];
  __syncwarp();  // the scratch may be rewritten by the next transform
  dft8<INV>(x);
}

// 128-point transforms on groups of sixteen lanes (two transforms per warp): one
// radix-2 stage across the two eight-lane halves of the group (lane bit 3, h) and
// a 64-point transform (fft64_lane8) in each half.  t = lane & 7.
//
// Inverse, decimation in frequency: lane (t, h) holds v[t + 8i + 64h] in x[i];
//   u = v[n], w = v[n + 64] (n = t + 8i): half 0 forms u + w, half 1 forms
//   (u - w) conj(W128^n); then each half runs the inverse 64-point transform, so
//   lane (t, h) ends holding V[2(t + 8i) + h] = V[2t + h + 16i].
// Forward, decimation in time: lane (t, h) holds v[2t + h + 16i] (half 0 the even
//   samples, half 1 the odd ones); each half runs the forward 64-point transform
//   (E, O at k = t + 8i), half 1 multiplies by W128^k, and the halves exchange:
//   lane (t, h) ends holding V[t + 8i + 64h] = E[k] + (-1)^h W128^k O[k].
// So the inverse takes the forward's output layout and gives the forward's input
// layout: an inverse pass followed by a forward pass needs no reordering.
// tw128[e] = W128^e for e < 64; the half-1 factors are read per call (registers).
template <bool INV>
__device__ __forceinline__ float2 l16_twiddle(const float2* tw128, int t, int i, int h) {
  const float2 v = tw128[t + 8 * i];
  return h ? (INV ? make_float2(v.x, -v.y) : v) : make_float2(1.f, 0.f);
}

__device__ __forceinline__ void fft128_inv_dif(float2 (&x)[8], const float2 (&w64)[8], const float2* tw128,
                                               float2* scr, int t, int h) {
  const float s = h ? -1.f : 1.f;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const float2 p = shfl_xor2(x[i], 8);
    const float2 y = make_float2(fmaf(s, x[i].x, p.x), fmaf(s, x[i].y, p.y));
    x[i] = cmul(y, l16_twiddle<true>(tw128, t, i, h));
  }
  fft64_lane8<true>(x, w64, scr, t);
}

__device__ __forceinline__ void fft128_fwd_dit(float2 (&x)[8], const float2 (&w64)[8], const float2* tw128,
                                               float2* scr, int t, int h) {
  fft64_lane8<false>(x, w64, scr, t);
  const float s = h ? -1.f : 1.f;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const float2 z = cmul(x[i], l16_twiddle<false>(tw128, t, i, h));
    const float2 p = shfl_xor2(z, 8);
    x[i] = make_float2(fmaf(s, z.x, p.x), fmaf(s, z.y, p.y));
  }
}

}  // namespace litho
