// SOCS kernel extraction (litho.cpp:579-645 calcKernels): the top-nk eigenpairs
// of the Hermitian TCC in FP64 on the GPU.  The reference calls LAPACK zheevr
// ('V', 'I', 'U'); this file computes the same eigenpairs with
//
//   1. hermitize_kernel     A = upper triangle of TCC mirrored (zheevr reads 'U' only)
//   2. Householder tridiagonalisation, one reflector per column k (the zhetd2
//      recurrence), two launches per column: symv_hh_kernel forms v, tau, beta
//      and x = tau*B*v; her2_kernel B -= v w^H + w v^H with w = x - tau/2 (x^H v) v
//      on the lower-triangle tiles, mirrored.  The off-diagonal comes out real.
//      Column k below the diagonal is read as the conjugate of row k (A stays
//      Hermitian in full), and v_k is packed contiguously for the back-transform.
//      Both kernels are bound by the FP64 pipe (GB300: 2 DFMA/clk/SM), so the
//      arithmetic is written as FMA chains and the update touches each element
//      pair once.
//   3. multisect_kernel     the nk largest eigenvalues of the real tridiagonal T
//                           by Sturm counts, one warp per eigenvalue and one CTA
//                           per SM: each round evaluates 32 points of the
//                           bracketing interval at once (33-way multisection);
//   4. invvec_kernel        eigenvector j of T by inverse iteration on the
//                           pivoted tridiagonal LU of T - shift_j I (the dgttrf
//                           recurrence), one CTA per eigenvector with the LU in
//                           shared memory;
//      cluster_rr_kernel    inside each cluster of close eigenvalues (a symmetric
//                           source gives exact degenerate pairs) the vectors are
//                           orthonormalised (Gram-Schmidt, twice) and rotated by
//                           a Rayleigh-Ritz step on the cluster's subspace
//                           (Jacobi eigendecomposition of Z^T T Z);
//   5. backtransform_kernel y = H_0 H_1 ... H_{n-2} z;
//   6. output_kernel        scales[i] = lambda_i (descending) and
//                           krn[i][j] = y_i[n-1-j] (litho.cpp:626-634 reversal).
// No kernel waits on another; every step is a separate launch on the stream.
#include "litho_internal.cuh"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

namespace litho {

__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zconj(double2 a) { return make_double2(a.x, -a.y); }
// conj by flipping the sign bit on the integer pipe (the FP64 pipe is the scarce one)
__device__ __forceinline__ double2 zconj_bits(double2 a) {
  return make_double2(a.x, __longlong_as_double(__double_as_longlong(a.y) ^ (long long)0x8000000000000000ull));
}
// lower-triangle tile t = I (I + 1) / 2 + J -> (I, J), in FP32 plus integer fix-ups
__device__ __forceinline__ void tri_tile(int t, int& I, int& J) {
  I = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
  while (I * (I + 1) / 2 > t) --I;
  while ((I + 1) * (I + 2) / 2 <= t) ++I;
  J = t - I * (I + 1) / 2;
}

template <int NT>
__device__ double block_sum(double v, double* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < NT / 32) t = red[threadIdx.x];
  if (w == 0) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) red[0] = t;
  }
  __syncthreads();
  const double r = red[0];
  __syncthreads();
  return r;
}

__global__ void hermitize_kernel(const double2* __restrict__ in, double2* __restrict__ A, int n) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (i >= n || j >= n) return;
  double2 v;
  if (i < j) v = in[(size_t)i * n + j];
  else if (i > j) v = zconj(in[(size_t)j * n + i]);
  else v = make_double2(in[(size_t)i * n + i].x, 0.0);
  A[(size_t)i * n + j] = v;
}

// Step k of the reduction, fused: the reflector of column k and x = tau B v with
// B = A[k+1:, k+1:].  Column k below the diagonal is conj(row k right of it), read
// contiguously.  Every CTA derives the reflector's scalars (norm, beta, tau, scale)
// from row k by the same fixed-order reduction, so they agree bitwise, and CTA 0
// publishes v, tau, d[k], e[k] and the packed copy of v kept for the back-transform.
// With v = (1, scl conj(row_k[1:])), B v = B[:,0] + scl B[:,1:] conj(row_k[1:]), so a
// row needs only row k itself; one warp per row, FMA chains (4 per complex element).
// Each CTA also leaves the partial sum of conj(x_i) v_i over its rows: the rank-2
// update adds them up in a fixed order for its correction term.
__device__ __forceinline__ size_t vpack_off(int n, int k) { return (size_t)k * (n - 1) - (size_t)k * (k - 1) / 2; }

__global__ void __launch_bounds__(256) symv_hh_kernel(const double2* __restrict__ A, int n, int k,
                                                      double2* __restrict__ vbuf, double2* __restrict__ vpack,
                                                      double2* __restrict__ tau, double* __restrict__ d,
                                                      double* __restrict__ e, double2* __restrict__ xbuf,
                                                      double2* __restrict__ part) {
  __shared__ double red[32];
  __shared__ double2 sp[8];
  const int m = n - k - 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const double2* rowk = A + (size_t)k * n + (k + 1);
  double s = 0.0;
  for (int i = 1 + threadIdx.x; i < m; i += 256) {
    const double2 x = rowk[i];
    s = fma(x.x, x.x, s);
    s = fma(x.y, x.y, s);
  }
  const double xnorm2 = block_sum<256>(s, red);
  __shared__ double2 s_t, s_scl;
  __shared__ double s_beta;
  if (threadIdx.x == 0) {  // the reflector's scalars (FP64 is scarce: one thread)
    const double2 alpha = zconj(rowk[0]);
    double2 tt = make_double2(0.0, 0.0);
    double beta = alpha.x;
    double2 sc = make_double2(0.0, 0.0);
    if (!(xnorm2 == 0.0 && alpha.y == 0.0)) {
      const double nrm = sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm2);
      beta = alpha.x >= 0.0 ? -nrm : nrm;
      tt = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
      // scl = 1 / (alpha - beta)
      const double2 den = make_double2(alpha.x - beta, alpha.y);
      const double dd = den.x * den.x + den.y * den.y;
      sc = make_double2(den.x / dd, -den.y / dd);
    }
    s_t = tt;
    s_scl = sc;
    s_beta = beta;
  }
  __syncthreads();
  const double2 t = s_t, scl = s_scl;
  const double beta = s_beta;
  if (blockIdx.x == 0) {
    double2* vp = vpack + vpack_off(n, k);
    for (int i = threadIdx.x; i < m; i += 256) {
      const double2 v = i == 0 ? make_double2(1.0, 0.0) : zmul(zconj(rowk[i]), scl);
      vbuf[i] = v;
      vp[i] = v;
    }
    if (threadIdx.x == 0) {
      tau[k] = t;
      e[k] = beta;
      d[k] = A[(size_t)k * n + k].x;
    }
  }
  const int row = blockIdx.x * 8 + warp;
  double2 contrib = make_double2(0.0, 0.0);
  if (row < m) {
    const double2* Ar = A + (size_t)(k + 1 + row) * n + (k + 1);
    double re = 0.0, im = 0.0;
    for (int j = 1 + lane; j < m; j += 32) {
      const double2 a = Ar[j], r = rowk[j];  // a * conj(r)
      re = fma(a.x, r.x, re);
      re = fma(a.y, r.y, re);
      im = fma(a.y, r.x, im);
      im = fma(-a.x, r.y, im);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      re += __shfl_xor_sync(0xffffffffu, re, o);
      im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    const double2 a0 = Ar[0];
    const double2 bv = make_double2(a0.x + (scl.x * re - scl.y * im), a0.y + (scl.x * im + scl.y * re));
    const double2 xr = zmul(t, bv);
    const double2 vr = row == 0 ? make_double2(1.0, 0.0) : zmul(zconj(rowk[row]), scl);
    contrib = zmul(zconj(xr), vr);
    if (lane == 0) xbuf[row] = xr;
  }
  if (lane == 0) sp[warp] = contrib;
  __syncthreads();
  if (threadIdx.x == 0) {
    double2 acc = sp[0];
    for (int w = 1; w < 8; ++w) acc = make_double2(acc.x + sp[w].x, acc.y + sp[w].y);
    part[blockIdx.x] = acc;
  }
}

// B -= v w^H + w v^H with w = x - tau/2 (x^H v) v, on the lower-triangle 32 x 32
// tiles (I >= J) only; x^H v is the fixed-order sum of the nparts partials of the
// product kernel, formed by every CTA.  An off-diagonal tile is computed once and
// written twice, as itself and as its conjugate transpose (staged in shared memory
// so both writes are coalesced); a diagonal tile writes its lower half and mirrors
// it into the upper.  That halves the FP64 work, and B stays exactly Hermitian,
// which the product kernel (full rows) relies on.  Each element is 8 FMAs.
// blockIdx.x enumerates the tiles row by row: t = I (I + 1) / 2 + J.
__global__ void __launch_bounds__(256) her2_kernel(double2* __restrict__ A, int n, int k,
                                                   const double2* __restrict__ vbuf, const double2* __restrict__ xbuf,
                                                   const double2* __restrict__ tau, const double2* __restrict__ part,
                                                   int nparts) {
  __shared__ double2 tile[32][33];
  __shared__ double2 s_c;
  __shared__ double2 s_v[2][32], s_w[2][32];  // [0]: the tile's columns, [1]: its rows
  const int m = n - k - 1;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  if (ty == 0) {
    double sr = 0.0, si = 0.0;
    for (int p = tx; p < nparts; p += 32) {
      sr += part[p].x;
      si += part[p].y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, o);
      si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    if (tx == 0) {
      const double2 tk = tau[k];
      s_c = zmul(make_double2(-0.5 * tk.x, -0.5 * tk.y), make_double2(sr, si));
    }
  }
  __syncthreads();
  int I, J;
  tri_tile(blockIdx.x, I, J);
  if (threadIdx.x < 64) {  // w = x + c v for the tile's 32 columns and 32 rows, once
    const int side = threadIdx.x >> 5, q = (side ? I : J) * 32 + tx;
    double2 vq = make_double2(0.0, 0.0), wq = vq;
    if (q < m) {
      const double2 c = s_c;
      vq = vbuf[q];
      const double2 xq = xbuf[q];
      wq = make_double2(xq.x + (c.x * vq.x - c.y * vq.y), xq.y + (c.x * vq.y + c.y * vq.x));
    }
    s_v[side][tx] = vq;
    s_w[side][tx] = wq;
  }
  __syncthreads();
  const int j = J * 32 + tx;
  const double2 vj = s_v[0][tx], wj = s_w[0][tx];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int i = I * 32 + ty + 8 * r;
    if (i < m && j < m) {
      const double2 vi = s_v[1][ty + 8 * r], wi = s_w[1][ty + 8 * r];
      double2* a = A + (size_t)(k + 1 + i) * n + (k + 1 + j);
      const double2 av = *a;
      // a - vi conj(wj) - wi conj(vj)
      double re = fma(-vi.x, wj.x, av.x);
      re = fma(-vi.y, wj.y, re);
      re = fma(-wi.x, vj.x, re);
      re = fma(-wi.y, vj.y, re);
      double im = fma(-vi.y, wj.x, av.y);
      im = fma(vi.x, wj.y, im);
      im = fma(-wi.y, vj.x, im);
      im = fma(wi.x, vj.y, im);
      const double2 nv = make_double2(re, im);
      if (I != J) *a = nv;
      tile[ty + 8 * r][tx] = nv;
    }
  }
  __syncthreads();
  if (I == J) {  // diagonal tile: lower half as computed, upper half mirrored
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int ii = ty + 8 * r, i = I * 32 + ii;
      if (i < m && j < m)
        A[(size_t)(k + 1 + i) * n + (k + 1 + j)] = ii >= tx ? tile[ii][tx] : zconj_bits(tile[tx][ii]);
    }
    return;
  }
  // mirror: A[J-tile row jj][I-tile col ii] = conj(tile[ii][jj])
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int jj = ty + 8 * r, ii = tx;
    const int row = J * 32 + jj, col = I * 32 + ii;
    if (row < m && col < m) A[(size_t)(k + 1 + row) * n + (k + 1 + col)] = zconj_bits(tile[ii][jj]);
  }
}

__global__ void last_diag_kernel(const double2* __restrict__ A, int n, double* __restrict__ d) {
  if (threadIdx.x == 0) d[n - 1] = A[(size_t)(n - 1) * n + (n - 1)].x;
}

__global__ void square_kernel(const double* __restrict__ e, double* __restrict__ e2, int m) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) e2[i] = e[i] * e[i];
}

// Number of eigenvalues of T below x: the sign changes of the leading principal
// minors p_i of T - xI, p_i = (d_i - x) p_{i-1} - e_{i-1}^2 p_{i-2} (p_{-1} = 1),
// i.e. the rows with q_i = p_i / p_{i-1} < 0 of the classical ratio recurrence,
// without its division per row (a division is some ten FP64 operations, and
// GB300 issues two FP64 FMAs per clock per SM).  A minor that comes out zero is
// replaced by -pivmin p_{i-1} (the ratio recurrence's q_i = -pivmin).  p_{i-1},
// p_i are rescaled together by 2^-256 / 2^256 (exact) when p_i leaves
// [2^-256, 2^256), so both stay below 2^512 and a step cannot overflow; the
// test reads the exponent bits on the integer pipe.
__device__ int sturm_count_lt(const double* d, const double* e2, int n, double x, double pivmin) {
  int c = 0;
  double pm = 1.0;       // p_{i-1}
  double p = d[0] - x;   // p_i
  if (p == 0.0) p = -pivmin;
  c += p < 0.0;
  for (int i = 1; i < n; ++i) {
    double pn = fma(d[i] - x, p, -e2[i - 1] * pm);
    if (pn == 0.0) pn = -pivmin * p;
    c += (__double_as_longlong(pn) ^ __double_as_longlong(p)) < 0;  // sign change
    pm = p;
    p = pn;
    const unsigned ex = (unsigned)(__double_as_longlong(p) >> 52) & 0x7FFu;
    if (ex - 767u >= 512u) {  // |p| outside [2^-256, 2^256) (or subnormal)
      const int sh = ex >= 1279u ? -256 : 256;
      p = ldexp(p, sh);
      pm = ldexp(pm, sh);
    }
  }
  return c;
}

// eigenvalue j (0 = largest) of T (diagonal d, off-diagonal e) by multisection:
// one CTA of MS_THREADS per eigenvalue (blockIdx.x); every round evaluates the Sturm
// count at MS_THREADS interior points of the bracket [lo, hi], count(lo) <= m <
// count(hi) with m the ascending index, and keeps the sub-interval holding the
// crossing.  A Sturm count is a sequential FP64 recurrence with a division per row,
// so one count is latency-bound; the points of a round run side by side, and a
// 129-way split needs ~8 rounds where bisection needs ~52.  The rounds stop when the
// bracket no longer shrinks in floating point.
constexpr int MS_THREADS = 128;

__global__ void __launch_bounds__(MS_THREADS) multisect_kernel(const double* __restrict__ d,
                                                               const double* __restrict__ e,
                                                               const double* __restrict__ e2, int n, int nk,
                                                               double* __restrict__ evals) {
  __shared__ double sh[3][MS_THREADS / 32];
  __shared__ unsigned masks[MS_THREADS / 32];
  const int j = blockIdx.x, t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (j >= nk) return;
  double lo = 1e300, hi = -1e300, emax = 0.0;
  for (int i = t; i < n; i += MS_THREADS) {
    const double r = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i < n - 1 ? fabs(e[i]) : 0.0);
    lo = fmin(lo, d[i] - r);
    hi = fmax(hi, d[i] + r);
    if (i < n - 1) emax = fmax(emax, e[i] * e[i]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    emax = fmax(emax, __shfl_xor_sync(0xffffffffu, emax, o));
  }
  if (lane == 0) {
    sh[0][warp] = lo;
    sh[1][warp] = hi;
    sh[2][warp] = emax;
  }
  __syncthreads();
  for (int w = 0; w < MS_THREADS / 32; ++w) {
    lo = fmin(lo, sh[0][w]);
    hi = fmax(hi, sh[1][w]);
    emax = fmax(emax, sh[2][w]);
  }
  const double span = fmax(fabs(lo), fabs(hi));
  lo -= 2.0 * DBL_EPSILON * span + 1e-300;
  hi += 2.0 * DBL_EPSILON * span + 1e-300;
  const double pivmin = 1e-290 * fmax(1.0, emax);
  const int m = n - 1 - j;  // ascending index
  for (int it = 0; it < 64; ++it) {
    // every thread evaluates the same expressions, so lo, hi stay identical in all
    const double w = (hi - lo) / (double)(MS_THREADS + 1);
    const double x = lo + w * (double)(t + 1);
    const bool above = x > lo && x < hi && sturm_count_lt(d, e2, n, x, pivmin) > m;
    const unsigned up = __ballot_sync(0xffffffffu, above);
    __syncthreads();  // the previous round's masks have been read
    if (lane == 0) masks[warp] = up;
    __syncthreads();
    // counts grow with the point index: the first point above m
    int f = MS_THREADS;
    for (int ww = MS_THREADS / 32 - 1; ww >= 0; --ww)
      if (masks[ww]) f = 32 * ww + __ffs(masks[ww]) - 1;
    const double nlo = f == 0 ? lo : lo + w * (double)f;
    const double nhi = f == MS_THREADS ? hi : lo + w * (double)(f + 1);
    if (!(nhi - nlo < hi - lo)) break;  // no progress: the bracket is a few ulps wide
    lo = nlo;
    hi = nhi;
  }
  if (t == 0) evals[j] = 0.5 * (lo + hi);
}

// Eigenvector j of T by inverse iteration, one CTA per eigenvector.  Inside a
// cluster of close eigenvalues the shifts are separated as dstein does, so each
// member starts from a distinct shift; the cluster's vectors are made orthonormal
// and rotated afterwards (cluster_rr_kernel).  Thread 0 runs the pivoted
// tridiagonal LU of T - shift I (the dgttrf recurrence) and the triangular solves,
// which are sequential by nature, on arrays in shared memory (or in this CTA's
// slice of global scratch when n is large); the CTA normalises between iterations.
constexpr int IV_THREADS = 128;
constexpr int IV_ITERS = 4;

__device__ __forceinline__ double iv_ortol(const double* d, const double* e, int n, double* red) {
  double t = 0.0;
  for (int i = threadIdx.x; i < n; i += IV_THREADS)
    t = fmax(t, fabs(d[i]) + (i > 0 ? fabs(e[i - 1]) : 0.0) + (i < n - 1 ? fabs(e[i]) : 0.0));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t = fmax(t, __shfl_xor_sync(0xffffffffu, t, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  double r = 0.0;
  for (int w = 0; w < IV_THREADS / 32; ++w) r = fmax(r, red[w]);
  __syncthreads();
  return r;
}

// Shared-memory path: [dl, dd, du, du2, z] (5n doubles) + n pivot bytes.  Global
// path (large n): this CTA's slice of `scratch`, [dl, dd, du, du2, z, pivot] as 6n
// doubles; vectors j0 .. j0 + gridDim.x - 1.
template <bool SMEM>
__global__ void __launch_bounds__(IV_THREADS) invvec_kernel(const double* __restrict__ d,
                                                            const double* __restrict__ e, int n, int j0,
                                                            const double* __restrict__ evals, double* __restrict__ Z,
                                                            double* __restrict__ scratch) {
  extern __shared__ __align__(16) double ivs[];
  __shared__ double red[32];
  const int j = j0 + blockIdx.x;
  double* base = SMEM ? ivs : scratch + (size_t)blockIdx.x * 6 * n;
  double* dl = base;           // L multipliers
  double* dd = base + n;       // U diagonal (its reciprocal after the factorisation)
  double* du = base + 2 * n;   // U first super-diagonal
  double* du2 = base + 3 * n;  // U second super-diagonal
  double* z = base + 4 * n;
  unsigned char* pivb = reinterpret_cast<unsigned char*>(base + 5 * n);  // SMEM: bytes
  double* pivd = base + 5 * n;                                           // global: doubles
  const double tnorm = iv_ortol(d, e, n, red);
  const double ortol = 1e-3 * tnorm;
  const double eps = DBL_EPSILON;
  const double tiny = eps * fmax(tnorm, 1e-300);
  // the shift of member j: dstein's perturbation applied along its cluster
  double lam = evals[j];
  {
    int c0 = j;
    while (c0 > 0 && fabs(evals[c0 - 1] - evals[c0]) <= ortol) --c0;
    double prev = evals[c0];
    for (int i = c0 + 1; i <= j; ++i) {
      double li = evals[i];
      const double pert = 10.0 * eps * fmax(fabs(li), tnorm * 1e-3);
      if (prev - li < pert) li = prev - pert;
      prev = li;
    }
    lam = prev;
  }
  // deterministic start vector
  for (int i = threadIdx.x; i < n; i += IV_THREADS) {
    unsigned h = (unsigned)(i * 2654435761u) ^ (unsigned)((j + 1) * 40503u);
    h ^= h >> 13;
    h *= 0x5bd1e995u;
    h ^= h >> 15;
    z[i] = ((double)(h & 0xffffff) / 16777216.0) - 0.5;
  }
  if (threadIdx.x == 0) {
    for (int i = 0; i < n; ++i) {
      dd[i] = d[i] - lam;
      du[i] = i < n - 1 ? e[i] : 0.0;
      dl[i] = i < n - 1 ? e[i] : 0.0;
      du2[i] = 0.0;
    }
    for (int i = 0; i < n - 1; ++i) {
      bool sw = false;
      if (fabs(dd[i]) >= fabs(dl[i])) {
        if (dd[i] == 0.0) dd[i] = tiny;
        const double f = dl[i] / dd[i];
        dl[i] = f;
        dd[i + 1] -= f * du[i];
        du2[i] = 0.0;
      } else {
        const double f = dd[i] / dl[i];
        dd[i] = dl[i];
        dl[i] = f;
        const double t = du[i];
        du[i] = dd[i + 1];
        dd[i + 1] = t - f * dd[i + 1];
        if (i < n - 2) {
          du2[i] = du[i + 1];
          du[i + 1] = -f * du[i + 1];
        }
        sw = true;
      }
      if (SMEM) pivb[i] = sw ? 1 : 0;
      else pivd[i] = sw ? 1.0 : 0.0;
    }
    if (dd[n - 1] == 0.0) dd[n - 1] = tiny;
  }
  __syncthreads();
  // U's diagonal, clamped away from zero, is kept as its reciprocal: the serial
  // back substitutions multiply (an FP64 division is a multi-instruction sequence,
  // and GB300 issues two FP64 operations per clock per SM)
  for (int i = threadIdx.x; i < n; i += IV_THREADS) {
    double v = dd[i];
    if (fabs(v) < tiny) v = v < 0.0 ? -tiny : tiny;
    dd[i] = 1.0 / v;
  }
  __syncthreads();
  for (int it = 0; it < IV_ITERS; ++it) {
    if (threadIdx.x == 0) {
      for (int i = 0; i < n - 1; ++i) {
        const bool sw = SMEM ? pivb[i] != 0 : pivd[i] != 0.0;
        if (!sw) {
          z[i + 1] -= dl[i] * z[i];
        } else {
          const double t = z[i];
          z[i] = z[i + 1];
          z[i + 1] = t - dl[i] * z[i];
        }
      }
      z[n - 1] *= dd[n - 1];
      if (n > 1) z[n - 2] = (z[n - 2] - du[n - 2] * z[n - 1]) * dd[n - 2];
      for (int i = n - 3; i >= 0; --i) z[i] = (z[i] - du[i] * z[i + 1] - du2[i] * z[i + 2]) * dd[i];
    }
    __syncthreads();
    double sq = 0.0;
    for (int i = threadIdx.x; i < n; i += IV_THREADS) sq += z[i] * z[i];
    sq = block_sum<IV_THREADS>(sq, red);
    const double inv = sq > 0.0 ? 1.0 / sqrt(sq) : 0.0;
    for (int i = threadIdx.x; i < n; i += IV_THREADS) z[i] *= inv;
    __syncthreads();
  }
  for (int i = threadIdx.x; i < n; i += IV_THREADS) Z[(size_t)j * n + i] = z[i];
}

// Clusters of close eigenvalues (|lambda_{i-1} - lambda_i| <= 1e-3 ||T||, the
// inverse-iteration cluster rule; on a flat spectrum it chains many members): the
// members' vectors Z_c are orthonormalised by Cholesky QR applied twice (Gram matrix
// G = Z_c^T Z_c = L L^T, Z_c <- Z_c L^-T), then rotated by the eigenvectors of the
// Rayleigh quotient H = Z_c^T T Z_c (cyclic Jacobi), ordered by descending Ritz
// value, so each member is the eigenvector of its own eigenvalue, not a mixture.
// The Gram and Rayleigh matrices are formed with one warp per entry pair and every
// row update is one thread per vector component, so the work is parallel.  A cluster
// larger than RR_MAXC (the near-zero tail of a rank-deficient TCC), or one whose
// Gram matrix is not numerically positive definite, is orthonormalised by modified
// Gram-Schmidt (two passes) instead, without the rotation in the first case.
// One CTA per cluster: CTA j works only if a cluster starts at j.
constexpr int RR_THREADS = 256, RR_MAXC = 48;

// y_i = (T z)_i for the symmetric tridiagonal T
__device__ __forceinline__ double tri_mul(const double* d, const double* e, const double* z, int n, int i) {
  double y = d[i] * z[i];
  if (i > 0) y += e[i - 1] * z[i - 1];
  if (i < n - 1) y += e[i] * z[i + 1];
  return y;
}

// S[a][b] = z_a . (T z_b) (withT) or z_a . z_b over the c x c lower triangle, mirrored;
// one warp per pair
__device__ void rr_pairs(const double* d, const double* e, const double* Zc, int n, int c, bool withT,
                         double (*S)[RR_MAXC + 1]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int np = c * (c + 1) / 2;
  for (int p = warp; p < np; p += RR_THREADS / 32) {
    int a, b;
    tri_tile(p, a, b);
    const double* za = Zc + (size_t)a * n;
    const double* zb = Zc + (size_t)b * n;
    // four independent partial sums: four loads of each row in flight per lane
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int i = lane;
    if (withT) {
      for (; i + 96 < n; i += 128) {
        s0 += za[i] * tri_mul(d, e, zb, n, i);
        s1 += za[i + 32] * tri_mul(d, e, zb, n, i + 32);
        s2 += za[i + 64] * tri_mul(d, e, zb, n, i + 64);
        s3 += za[i + 96] * tri_mul(d, e, zb, n, i + 96);
      }
      for (; i < n; i += 32) s0 += za[i] * tri_mul(d, e, zb, n, i);
    } else {
      for (; i + 96 < n; i += 128) {
        s0 += za[i] * zb[i];
        s1 += za[i + 32] * zb[i + 32];
        s2 += za[i + 64] * zb[i + 64];
        s3 += za[i + 96] * zb[i + 96];
      }
      for (; i < n; i += 32) s0 += za[i] * zb[i];
    }
    double sd = (s0 + s1) + (s2 + s3);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sd += __shfl_xor_sync(0xffffffffu, sd, o);
    if (lane == 0) {
      S[a][b] = sd;
      S[b][a] = sd;
    }
  }
}

__global__ void __launch_bounds__(RR_THREADS) cluster_rr_kernel(const double* __restrict__ d,
                                                                const double* __restrict__ e, int n, int nk,
                                                                const double* __restrict__ evals,
                                                                double* __restrict__ Z) {
  __shared__ double red[32];
  __shared__ double H[RR_MAXC][RR_MAXC + 1];
  __shared__ double V[RR_MAXC][RR_MAXC + 1];
  __shared__ int s_order[RR_MAXC];
  __shared__ int s_ok;
  double tn = 0.0;
  for (int i = threadIdx.x; i < n; i += RR_THREADS)
    tn = fmax(tn, fabs(d[i]) + (i > 0 ? fabs(e[i - 1]) : 0.0) + (i < n - 1 ? fabs(e[i]) : 0.0));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) tn = fmax(tn, __shfl_xor_sync(0xffffffffu, tn, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = tn;
  __syncthreads();
  double tnorm = 0.0;
  for (int w = 0; w < RR_THREADS / 32; ++w) tnorm = fmax(tnorm, red[w]);
  __syncthreads();
  const double ortol = 1e-3 * tnorm;
  const int c0 = blockIdx.x;
  if (c0 > 0 && fabs(evals[c0 - 1] - evals[c0]) <= ortol) return;  // not a cluster start
  int c1 = c0 + 1;
  while (c1 < nk && fabs(evals[c1 - 1] - evals[c1]) <= ortol) ++c1;
  const int c = c1 - c0;
  if (c < 2) return;
  double* Zc = Z + (size_t)c0 * n;
  bool ok = c <= RR_MAXC;
  // Cholesky QR, twice
  for (int pass = 0; ok && pass < 2; ++pass) {
    rr_pairs(d, e, Zc, n, c, false, H);
    __syncthreads();
    if (threadIdx.x == 0) {
      s_ok = 1;
      for (int a = 0; a < c && s_ok; ++a) {  // H <- L (lower), in place
        double diag = H[a][a];
        for (int b = 0; b < a; ++b) diag -= H[a][b] * H[a][b];
        if (!(diag > 1e-24)) {
          s_ok = 0;
          break;
        }
        H[a][a] = sqrt(diag);
        for (int r = a + 1; r < c; ++r) {
          double v = H[r][a];
          for (int b = 0; b < a; ++b) v -= H[r][b] * H[a][b];
          H[r][a] = v / H[a][a];
        }
      }
    }
    __syncthreads();
    ok = s_ok != 0;
    if (!ok) break;
    // z_i <- L^-1 z_i for every component i (forward substitution)
    for (int i = threadIdx.x; i < n; i += RR_THREADS) {
      double y[RR_MAXC];
      for (int a = 0; a < c; ++a) {
        double v = Zc[(size_t)a * n + i];
        for (int b = 0; b < a; ++b) v -= H[a][b] * y[b];
        y[a] = v / H[a][a];
      }
      for (int a = 0; a < c; ++a) Zc[(size_t)a * n + i] = y[a];
    }
    __syncthreads();
  }
  if (!ok) {  // modified Gram-Schmidt, two passes
    for (int pass = 0; pass < 2; ++pass)
      for (int a = 0; a < c; ++a) {
        double* za = Zc + (size_t)a * n;
        for (int b = 0; b < a; ++b) {
          const double* zb = Zc + (size_t)b * n;
          double sd = 0.0;
          for (int i = threadIdx.x; i < n; i += RR_THREADS) sd += zb[i] * za[i];
          sd = block_sum<RR_THREADS>(sd, red);
          for (int i = threadIdx.x; i < n; i += RR_THREADS) za[i] -= sd * zb[i];
          __syncthreads();
        }
        double sq = 0.0;
        for (int i = threadIdx.x; i < n; i += RR_THREADS) sq += za[i] * za[i];
        sq = block_sum<RR_THREADS>(sq, red);
        const double inv = sq > 0.0 ? 1.0 / sqrt(sq) : 0.0;
        for (int i = threadIdx.x; i < n; i += RR_THREADS) za[i] *= inv;
        __syncthreads();
      }
    if (c > RR_MAXC) return;
  }
  // Rayleigh-Ritz: H = Z_c^T T Z_c
  rr_pairs(d, e, Zc, n, c, true, H);
  for (int i = threadIdx.x; i < c * c; i += RR_THREADS) V[i / c][i % c] = (i / c == i % c) ? 1.0 : 0.0;
  __syncthreads();
  // cyclic Jacobi on the c x c symmetric H, V accumulating the rotations, in
  // round-robin order: a sweep is cp - 1 rounds (cp = c rounded up to even; index
  // c is a dummy when c is odd), each rotating cp/2 disjoint pairs (p, q) at once.
  // A pair's rotation is computed from the matrix before its round (the 2 x 2
  // block of (p, q) is touched by no other rotation of the round), then all
  // column rotations (H <- H J, V <- V J) and all row rotations (H <- J^T H)
  // are applied by the whole block.  Same rotation formulas as the serial
  // cyclic method; the circle method pairs every (p, q) once per sweep.
  {
    __shared__ double s_cs[RR_MAXC / 2], s_sn[RR_MAXC / 2];
    __shared__ int s_p[RR_MAXC / 2], s_q[RR_MAXC / 2];
    __shared__ int s_done;
    const int cp = c + (c & 1), np = cp / 2;
    for (int sweep = 0; sweep < 30; ++sweep) {
      if (threadIdx.x == 0) {
        double off = 0.0, dia = 0.0;
        for (int a = 0; a < c; ++a) {
          dia += H[a][a] * H[a][a];
          for (int b = a + 1; b < c; ++b) off += H[a][b] * H[a][b];
        }
        s_done = off <= 1e-32 * dia;
      }
      __syncthreads();
      if (s_done) break;
      for (int r = 0; r < cp - 1; ++r) {
        if (threadIdx.x < np) {
          const int i = threadIdx.x, j = cp - 1 - i;
          const int a = i == 0 ? 0 : (i - 1 + r) % (cp - 1) + 1;
          const int b = (j - 1 + r) % (cp - 1) + 1;
          const int pp = min(a, b), qq = max(a, b);
          double cs = 1.0, sn = 0.0;
          if (qq < c) {
            const double apq = H[pp][qq];
            if (apq != 0.0) {
              const double theta = (H[qq][qq] - H[pp][pp]) / (2.0 * apq);
              const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
              cs = 1.0 / sqrt(t * t + 1.0);
              sn = t * cs;
            }
          }
          s_p[i] = pp;
          s_q[i] = qq;
          s_cs[i] = cs;
          s_sn[i] = sn;
        }
        __syncthreads();
        for (int w = threadIdx.x; w < np * c; w += RR_THREADS) {  // columns p, q of H and V
          const int i = w / c, k = w - i * c, pp = s_p[i], qq = s_q[i];
          if (qq < c) {
            const double cs = s_cs[i], sn = s_sn[i];
            const double hkp = H[k][pp], hkq = H[k][qq];
            H[k][pp] = cs * hkp - sn * hkq;
            H[k][qq] = sn * hkp + cs * hkq;
            const double vkp = V[k][pp], vkq = V[k][qq];
            V[k][pp] = cs * vkp - sn * vkq;
            V[k][qq] = sn * vkp + cs * vkq;
          }
        }
        __syncthreads();
        for (int w = threadIdx.x; w < np * c; w += RR_THREADS) {  // rows p, q of H
          const int i = w / c, k = w - i * c, pp = s_p[i], qq = s_q[i];
          if (qq < c) {
            const double cs = s_cs[i], sn = s_sn[i];
            const double hpk = H[pp][k], hqk = H[qq][k];
            H[pp][k] = cs * hpk - sn * hqk;
            H[qq][k] = sn * hpk + cs * hqk;
          }
        }
        __syncthreads();
      }
    }
  }
  if (threadIdx.x == 0) {  // descending Ritz values
    for (int a = 0; a < c; ++a) s_order[a] = a;
    for (int a = 1; a < c; ++a) {
      const int key = s_order[a];
      int b = a - 1;
      while (b >= 0 && H[s_order[b]][s_order[b]] < H[key][key]) {
        s_order[b + 1] = s_order[b];
        --b;
      }
      s_order[b + 1] = key;
    }
  }
  __syncthreads();
  // Z_c <- Z_c V (columns in descending Ritz order), one thread per component
  for (int i = threadIdx.x; i < n; i += RR_THREADS) {
    double x[RR_MAXC];
    for (int b = 0; b < c; ++b) x[b] = Zc[(size_t)b * n + i];
    for (int a = 0; a < c; ++a) {
      const int col = s_order[a];
      double acc = 0.0;
      for (int b = 0; b < c; ++b) acc += x[b] * V[b][col];
      Zc[(size_t)a * n + i] = acc;
    }
  }
}

// y = H_0 H_1 ... H_{n-2} z for eigenvector j = blockIdx.x; H_k = I - tau_k v_k v_k^H
// acting on rows k+1..n-1, v_k packed contiguously in vpack.
// y_j = H_0 H_1 ... H_{n-2} z_j for every eigenvector j, with the reflectors taken
// WY_NB at a time in compact WY form: H_k0 ... H_{k0+nb-1} = I - V T V^H (V the
// block's reflectors as columns, T upper triangular: T_jj = tau_j,
// T[0:j, j] = -tau_j T[0:j, 0:j] (V[:, 0:j]^H v_j)), so a block costs three block
// barriers (w = V^H y reduced over the CTA, u = T w, y -= V u) instead of one per
// reflector, for the same FP64 work.
constexpr int WY_NB = 16;

// T of every block (one CTA per block): the Gram products v_i^H v_j (i < j, over
// v_j's support) one warp per pair, then the triangular recurrence on one thread
__global__ void __launch_bounds__(256) wy_t_kernel(const double2* __restrict__ vpack,
                                                   const double2* __restrict__ tau, int n,
                                                   double2* __restrict__ Tg) {
  __shared__ double2 G[WY_NB][WY_NB];
  __shared__ double2 T[WY_NB][WY_NB];
  const int b = blockIdx.x, k0 = b * WY_NB, nbb = min(WY_NB, n - 1 - k0);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int np = nbb * (nbb - 1) / 2;
  for (int p = warp; p < np; p += 8) {
    int j = 1;
    while ((j + 1) * j / 2 <= p) ++j;  // p = j (j - 1) / 2 + i, i < j
    const int i = p - j * (j - 1) / 2;
    const int ki = k0 + i, kj = k0 + j;
    const double2* vi = vpack + vpack_off(n, ki) - (ki + 1);  // v_i[r], r in [ki+1, n)
    const double2* vj = vpack + vpack_off(n, kj) - (kj + 1);
    double sr = 0.0, si = 0.0;  // conj(v_i) . v_j
    for (int r = kj + 1 + lane; r < n; r += 32) {
      const double2 a = vi[r], c = vj[r];
      sr = fma(a.x, c.x, fma(a.y, c.y, sr));
      si = fma(a.x, c.y, fma(-a.y, c.x, si));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, o);
      si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    if (lane == 0) G[i][j] = make_double2(sr, si);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int jj = 0; jj < WY_NB; ++jj)
      for (int ii = 0; ii < WY_NB; ++ii) T[ii][jj] = make_double2(0.0, 0.0);
    for (int jj = 0; jj < nbb; ++jj) {
      const double2 tj = tau[k0 + jj];
      T[jj][jj] = tj;
      for (int ii = 0; ii < jj; ++ii) {
        double2 acc = make_double2(0.0, 0.0);
        for (int l = ii; l < jj; ++l) {
          const double2 t = T[ii][l], g = G[l][jj];
          acc.x += t.x * g.x - t.y * g.y;
          acc.y += t.x * g.y + t.y * g.x;
        }
        T[ii][jj] = make_double2(-(tj.x * acc.x - tj.y * acc.y), -(tj.x * acc.y + tj.y * acc.x));
      }
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < WY_NB * WY_NB; e += 256) Tg[(size_t)b * WY_NB * WY_NB + e] = T[e / WY_NB][e % WY_NB];
}

// one CTA per vector; thread t owns the elements y[t + 256 s] for the whole loop
__global__ void __launch_bounds__(256) backtransform_kernel(const double2* __restrict__ vpack, int n,
                                                            const double2* __restrict__ Tg,
                                                            const double* __restrict__ Z, double2* __restrict__ Y) {
  __shared__ double2 red[8][WY_NB];
  __shared__ double2 s_w[WY_NB], s_u[WY_NB];
  __shared__ long long s_base[WY_NB];  // v_i[r] = vpack[s_base[i] + r]
  const int j = blockIdx.x, t = threadIdx.x, lane = t & 31, w = t >> 5;
  double2* y = Y + (size_t)j * n;
  for (int i = t; i < n; i += 256) y[i] = make_double2(Z[(size_t)j * n + i], 0.0);
  const int nblk = (n - 1 + WY_NB - 1) / WY_NB;
  for (int b = nblk - 1; b >= 0; --b) {
    const int k0 = b * WY_NB, nbb = min(WY_NB, n - 1 - k0);
    if (t < WY_NB) s_base[t] = t < nbb ? (long long)vpack_off(n, k0 + t) - (k0 + t + 1) : 0;
    __syncthreads();  // s_base; also, every thread is past the previous block's reads of s_u
    int r0 = t;
    if (r0 < k0 + 1) r0 += ((k0 + 1 - r0 + 255) / 256) * 256;
    double ar[WY_NB], ai[WY_NB];
#pragma unroll
    for (int i = 0; i < WY_NB; ++i) ar[i] = ai[i] = 0.0;
    for (int r = r0; r < n; r += 256) {
      const double2 yy = y[r];
#pragma unroll
      for (int i = 0; i < WY_NB; ++i)
        if (i < nbb && r > k0 + i) {
          const double2 vv = vpack[s_base[i] + r];
          ar[i] = fma(vv.x, yy.x, fma(vv.y, yy.y, ar[i]));  // conj(v) * y
          ai[i] = fma(vv.x, yy.y, fma(-vv.y, yy.x, ai[i]));
        }
    }
#pragma unroll
    for (int i = 0; i < WY_NB; ++i) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        ar[i] += __shfl_xor_sync(0xffffffffu, ar[i], o);
        ai[i] += __shfl_xor_sync(0xffffffffu, ai[i], o);
      }
      if (lane == 0) red[w][i] = make_double2(ar[i], ai[i]);
    }
    __syncthreads();
    if (t < WY_NB) {
      double2 sm = red[0][t];
      for (int q = 1; q < 8; ++q) {
        sm.x += red[q][t].x;
        sm.y += red[q][t].y;
      }
      s_w[t] = sm;
    }
    __syncthreads();
    if (t < WY_NB) {  // u = T w (T upper triangular)
      const double2* Tb = Tg + (size_t)b * WY_NB * WY_NB + (size_t)t * WY_NB;
      double2 u = make_double2(0.0, 0.0);
      for (int l = t; l < nbb; ++l) {
        const double2 a = Tb[l], c = s_w[l];
        u.x += a.x * c.x - a.y * c.y;
        u.y += a.x * c.y + a.y * c.x;
      }
      s_u[t] = u;
    }
    __syncthreads();
    for (int r = r0; r < n; r += 256) {  // y -= V u
      double2 yy = y[r];
#pragma unroll
      for (int i = 0; i < WY_NB; ++i)
        if (i < nbb && r > k0 + i) {
          const double2 vv = vpack[s_base[i] + r], u = s_u[i];
          yy.x = fma(-u.x, vv.x, fma(u.y, vv.y, yy.x));
          yy.y = fma(-u.x, vv.y, fma(-u.y, vv.x, yy.y));
        }
      y[r] = yy;
    }
  }
}

__global__ void output_kernel(const double2* __restrict__ Y, const double* __restrict__ evals, int n, int nk,
                              float* __restrict__ kr, float* __restrict__ ki, float* __restrict__ sc,
                              double2* __restrict__ k64, double* __restrict__ s64) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (i >= nk) return;
  if (j < n) {
    const double2 v = Y[(size_t)i * n + (n - 1 - j)];
    kr[(size_t)i * n + j] = (float)v.x;
    ki[(size_t)i * n + j] = (float)v.y;
    if (k64) k64[(size_t)i * n + j] = v;
  }
  if (j == 0) {
    sc[i] = (float)evals[i];
    if (s64) s64[i] = evals[i];
  }
}

}  // namespace litho

using namespace litho;

extern "C" int litho_calc_kernels(litho_ctx* ctx, const double* tcc, int tccSize, int nk, float* krn_r, float* krn_i,
                                  float* scales, double* krn64, double* scales64, int mem) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  LITHO_ARG_CHECK(ctx, tcc && krn_r && krn_i && scales, "null pointer");
  LITHO_ARG_CHECK(ctx, tccSize >= 1 && tccSize <= 8192, "tccSize %d outside [1, 8192]", tccSize);
  LITHO_ARG_CHECK(ctx, nk >= 1 && nk <= tccSize, "nk %d outside [1, tccSize=%d]", nk, tccSize);
  LITHO_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  const int n = tccSize;
  const size_t nn = (size_t)n * n;
  const void* dtcc = nullptr;
  LITHO_RET(stage_in(ctx, ctx->tcc_c, tcc, nn * sizeof(double2), mem, &dtcc));
  LITHO_RET(ctx->eig_v.ensure(ctx, nn * sizeof(double2)));
  // workspace: vbuf, xbuf, tau (n double2 each); packed reflectors (n(n-1)/2
  // double2); per-CTA partial dots ((n+7)/8 double2); d, e (n double); evals (nk);
  // Z (nk*n double); inverse-iteration scratch (large n only: IV_CHUNK * 6n double);
  // Y (nk*n double2)
  const size_t iv_smem = (size_t)5 * n * sizeof(double) + n;
  const bool iv_in_smem = iv_smem <= 200 * 1024;
  constexpr int IV_CHUNK = 64;
  const size_t iv_scratch = iv_in_smem ? 0 : (size_t)IV_CHUNK * 6 * n * sizeof(double);
  const size_t vpack_bytes = (size_t)n * (n - 1) / 2 * sizeof(double2) + sizeof(double2);
  const size_t part_bytes = (size_t)((n + 7) / 8) * sizeof(double2);
  const size_t wbytes = 3 * n * sizeof(double2) + vpack_bytes + part_bytes + 3 * n * sizeof(double) + nk * sizeof(double) +
                        (size_t)nk * n * sizeof(double) + iv_scratch + (size_t)nk * n * sizeof(double2) +
                        (size_t)((n + WY_NB - 1) / WY_NB + 1) * WY_NB * WY_NB * sizeof(double2) + 17 * 64;
  LITHO_RET(ctx->eig_work.ensure(ctx, wbytes));
  char* w = ctx->eig_work.as<char>();
  auto take = [&](size_t b) {
    char* p = w;
    w += (b + 63) & ~size_t(63);
    return p;
  };
  double2* vbuf = reinterpret_cast<double2*>(take(n * sizeof(double2)));
  double2* xbuf = reinterpret_cast<double2*>(take(n * sizeof(double2)));
  double2* tau = reinterpret_cast<double2*>(take(n * sizeof(double2)));
  double2* vpack = reinterpret_cast<double2*>(take(vpack_bytes));
  double2* part = reinterpret_cast<double2*>(take(part_bytes));
  double* d = reinterpret_cast<double*>(take(n * sizeof(double)));
  double* e = reinterpret_cast<double*>(take(n * sizeof(double)));
  double* e2 = reinterpret_cast<double*>(take(n * sizeof(double)));
  double* ev = reinterpret_cast<double*>(take(nk * sizeof(double)));
  double* Z = reinterpret_cast<double*>(take((size_t)nk * n * sizeof(double)));
  double* ivs = iv_in_smem ? nullptr : reinterpret_cast<double*>(take(iv_scratch));
  double2* Y = reinterpret_cast<double2*>(take((size_t)nk * n * sizeof(double2)));
  const int wy_blocks = n > 1 ? (n - 1 + WY_NB - 1) / WY_NB : 0;
  double2* Tg = reinterpret_cast<double2*>(take((size_t)(wy_blocks > 0 ? wy_blocks : 1) * WY_NB * WY_NB * sizeof(double2)));
  double2* A = ctx->eig_v.as<double2>();
  {
    // hermitize, 2 per reflector, last diagonal, e^2, multisection, inverse iteration
    // (one launch, or one per chunk of IV_CHUNK vectors), cluster Rayleigh-Ritz, WY factors, back-transform
    const int iv_launches = iv_in_smem ? 1 : (nk + IV_CHUNK - 1) / IV_CHUNK;
    StageScope sc(ctx, LITHO_STAGE_EIG, 2 * (n > 1 ? n - 1 : 0) + 6 + (wy_blocks > 0 ? 1 : 0) + iv_launches);
    hermitize_kernel<<<dim3((n + 127) / 128, n), 128, 0, ctx->stream>>>(static_cast<const double2*>(dtcc), A, n);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
    LITHO_CUDA_TRY(ctx, cudaMemsetAsync(e, 0, n * sizeof(double), ctx->stream));
    for (int k = 0; k + 1 < n; ++k) {
      const int m = n - k - 1;
      const int nb = (m + 7) / 8;
      symv_hh_kernel<<<nb, 256, 0, ctx->stream>>>(A, n, k, vbuf, vpack, tau, d, e, xbuf, part);
      const int nt = (m + 31) / 32;
      her2_kernel<<<nt * (nt + 1) / 2, 256, 0, ctx->stream>>>(A, n, k, vbuf, xbuf, tau, part, nb);
    }
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
    last_diag_kernel<<<1, 32, 0, ctx->stream>>>(A, n, d);
    square_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(e, e2, n - 1);
    multisect_kernel<<<nk, MS_THREADS, 0, ctx->stream>>>(d, e, e2, n, nk, ev);
    if (iv_in_smem) {
      LITHO_CUDA_TRY(ctx, cudaFuncSetAttribute(invvec_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)iv_smem));
      invvec_kernel<true><<<nk, IV_THREADS, iv_smem, ctx->stream>>>(d, e, n, 0, ev, Z, nullptr);
    } else {
      for (int j0 = 0; j0 < nk; j0 += IV_CHUNK)
        invvec_kernel<false><<<std::min(IV_CHUNK, nk - j0), IV_THREADS, 0, ctx->stream>>>(d, e, n, j0, ev, Z, ivs);
    }
    cluster_rr_kernel<<<nk, RR_THREADS, 0, ctx->stream>>>(d, e, n, nk, ev, Z);
    if (wy_blocks > 0) wy_t_kernel<<<wy_blocks, 256, 0, ctx->stream>>>(vpack, tau, n, Tg);
    backtransform_kernel<<<nk, 256, 0, ctx->stream>>>(vpack, n, Tg, Z, Y);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
  }
  float *okr = krn_r, *oki = krn_i, *osc = scales;
  double *ok64 = krn64, *os64 = scales64;
  if (mem == LITHO_MEM_HOST) {
    LITHO_RET(ctx->eig_info.ensure(ctx, (size_t)nk * n * (2 * sizeof(float) + sizeof(double2)) +
                                            nk * (sizeof(float) + sizeof(double)) + 256));
    char* o = ctx->eig_info.as<char>();
    ok64 = reinterpret_cast<double*>(o);
    o += (size_t)nk * n * sizeof(double2);
    os64 = reinterpret_cast<double*>(o);
    o += nk * sizeof(double);
    okr = reinterpret_cast<float*>(o);
    o += (size_t)nk * n * sizeof(float);
    oki = reinterpret_cast<float*>(o);
    o += (size_t)nk * n * sizeof(float);
    osc = reinterpret_cast<float*>(o);
  }
  {
    StageScope sc(ctx, LITHO_STAGE_UPLOAD);
    output_kernel<<<dim3((n + 127) / 128, nk), 128, 0, ctx->stream>>>(Y, ev, n, nk, okr, oki, osc,
                                                                     reinterpret_cast<double2*>(ok64), os64);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
  }
  if (mem == LITHO_MEM_HOST) {
    LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(krn_r, okr, (size_t)nk * n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(krn_i, oki, (size_t)nk * n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(scales, osc, nk * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    if (krn64)
      LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(krn64, ok64, (size_t)nk * n * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
    if (scales64)
      LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(scales64, os64, nk * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    LITHO_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < nk; ++i)
      if (!std::isfinite(scales[i])) {
        set_error(ctx, LITHO_ERR_NAN, "non-finite eigenvalue %d", i);
        return LITHO_ERR_NAN;
      }
  }
  return LITHO_OK;
}
