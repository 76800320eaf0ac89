// SOCS kernel extraction (litho.cpp:579-645 calcKernels): the top-nk eigenpairs
// of the Hermitian TCC in FP64 on the GPU.  The reference calls LAPACK zheevr
// ('V', 'I', 'U'); this file computes the same eigenpairs with
//
//   1. hermitize_kernel     A = upper triangle of TCC mirrored (zheevr reads 'U' only)
//   2. Householder tridiagonalisation, one reflector per column k (the zhetd2
//      recurrence): hh_kernel forms v, tau, beta; symv_kernel x = tau*B*v;
//      her2_kernel B -= v w^H + w v^H with w = x - tau/2 (x^H v) v.  The
//      off-diagonal comes out real; v_k is kept in column k below the diagonal.
//   3. bisect_kernel        the nk largest eigenvalues of the real tridiagonal T
//                           by Sturm-count bisection (one thread each);
//   4. inviter_kernel       eigenvectors of T by inverse iteration on a pivoted
//                           tridiagonal LU, re-orthogonalised inside clusters of
//                           close eigenvalues (degenerate pairs are common: a
//                           symmetric source gives exact pairs);
//   5. backtransform_kernel y = H_0 H_1 ... H_{n-2} z;
//   6. output_kernel        scales[i] = lambda_i (descending) and
//                           krn[i][j] = y_i[n-1-j] (litho.cpp:626-634 reversal).
// No kernel waits on another; every step is a separate launch on the stream.
#include "litho_internal.cuh"

#include <cfloat>
#include <cmath>
#include <vector>

namespace litho {

__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zconj(double2 a) { return make_double2(a.x, -a.y); }

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

// Reflector for column k: x = A[k+1:n][k], m = n-k-1.
__global__ void __launch_bounds__(256) hh_kernel(double2* __restrict__ A, int n, int k, double2* __restrict__ vbuf,
                                                 double2* __restrict__ tau, double* __restrict__ d,
                                                 double* __restrict__ e) {
  __shared__ double red[32];
  const int m = n - k - 1;
  double s = 0.0;
  for (int i = 1 + threadIdx.x; i < m; i += 256) {
    const double2 x = A[(size_t)(k + 1 + i) * n + k];
    s += x.x * x.x + x.y * x.y;
  }
  const double xnorm2 = block_sum<256>(s, red);
  const double2 alpha = A[(size_t)(k + 1) * n + k];
  double2 t = make_double2(0.0, 0.0);
  double beta = alpha.x;
  double2 scl = make_double2(0.0, 0.0);
  if (!(xnorm2 == 0.0 && alpha.y == 0.0)) {
    const double nrm = sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm2);
    beta = alpha.x >= 0.0 ? -nrm : nrm;
    t = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
    // scl = 1 / (alpha - beta)
    const double2 den = make_double2(alpha.x - beta, alpha.y);
    const double dd = den.x * den.x + den.y * den.y;
    scl = make_double2(den.x / dd, -den.y / dd);
  }
  for (int i = threadIdx.x; i < m; i += 256) {
    double2 v;
    if (i == 0) v = make_double2(1.0, 0.0);
    else v = zmul(A[(size_t)(k + 1 + i) * n + k], scl);
    vbuf[i] = v;
    A[(size_t)(k + 1 + i) * n + k] = v;  // keep v_k for the back-transform
  }
  if (threadIdx.x == 0) {
    tau[k] = t;
    e[k] = beta;
    d[k] = A[(size_t)k * n + k].x;
  }
}

// x_i = tau * sum_j B[i][j] v_j, B = A[k+1:, k+1:]; one warp per row.
__global__ void __launch_bounds__(256) symv_kernel(const double2* __restrict__ A, int n, int k,
                                                   const double2* __restrict__ vbuf, const double2* __restrict__ tau,
                                                   double2* __restrict__ xbuf) {
  const int m = n - k - 1;
  const int row = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (row >= m) return;
  const double2* Ar = A + (size_t)(k + 1 + row) * n + (k + 1);
  double re = 0.0, im = 0.0;
  for (int j = lane; j < m; j += 32) {
    const double2 a = Ar[j], v = vbuf[j];
    re += a.x * v.x - a.y * v.y;
    im += a.x * v.y + a.y * v.x;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_xor_sync(0xffffffffu, re, o);
    im += __shfl_xor_sync(0xffffffffu, im, o);
  }
  if (lane == 0) xbuf[row] = zmul(tau[k], make_double2(re, im));
}

// w = x - tau/2 (x^H v) v (one CTA), written over xbuf.
__global__ void __launch_bounds__(256) wdot_kernel(int n, int k, const double2* __restrict__ vbuf,
                                                   double2* __restrict__ xbuf, const double2* __restrict__ tau) {
  __shared__ double red[32];
  const int m = n - k - 1;
  double sr = 0.0, si = 0.0;
  for (int i = threadIdx.x; i < m; i += 256) {
    const double2 x = xbuf[i], v = vbuf[i];
    sr += x.x * v.x + x.y * v.y;  // conj(x) * v
    si += x.x * v.y - x.y * v.x;
  }
  sr = block_sum<256>(sr, red);
  si = block_sum<256>(si, red);
  const double2 t = tau[k];
  const double2 c = zmul(make_double2(-0.5 * t.x, -0.5 * t.y), make_double2(sr, si));
  for (int i = threadIdx.x; i < m; i += 256) {
    const double2 v = vbuf[i];
    const double2 x = xbuf[i];
    xbuf[i] = make_double2(x.x + c.x * v.x - c.y * v.y, x.y + c.x * v.y + c.y * v.x);
  }
}

// B -= v w^H + w v^H (w in wbuf); 32 x 32 tiles, 8 rows per pass.
__global__ void __launch_bounds__(256) her2_kernel(double2* __restrict__ A, int n, int k,
                                                   const double2* __restrict__ vbuf, const double2* __restrict__ wbuf) {
  const int m = n - k - 1;
  const int j = blockIdx.x * 32 + (threadIdx.x & 31);
  const int i0 = blockIdx.y * 32 + (threadIdx.x >> 5);
  if (j >= m) return;
  const double2 vj = vbuf[j];
  const double2 wj = wbuf[j];
  for (int i = i0; i < min(m, blockIdx.y * 32 + 32); i += 8) {
    const double2 vi = vbuf[i];
    const double2 wi = wbuf[i];
    double2* a = A + (size_t)(k + 1 + i) * n + (k + 1 + j);
    const double2 p = zmul(vi, zconj(wj)), q = zmul(wi, zconj(vj));
    a->x -= p.x + q.x;
    a->y -= p.y + q.y;
  }
}

__global__ void last_diag_kernel(const double2* __restrict__ A, int n, double* __restrict__ d) {
  if (threadIdx.x == 0) d[n - 1] = A[(size_t)(n - 1) * n + (n - 1)].x;
}

__device__ int sturm_count_lt(const double* d, const double* e, int n, double x, double pivmin) {
  int c = 0;
  double q = d[0] - x;
  if (fabs(q) < pivmin) q = -pivmin;
  if (q < 0.0) ++c;
  for (int i = 1; i < n; ++i) {
    q = d[i] - x - e[i - 1] * e[i - 1] / q;
    if (fabs(q) < pivmin) q = -pivmin;
    if (q < 0.0) ++c;
  }
  return c;
}

// eigenvalue j (0 = largest) of T by bisection; T has diagonal d, off-diagonal e.
__global__ void bisect_kernel(const double* __restrict__ d, const double* __restrict__ e, int n, int nk,
                              double* __restrict__ evals) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nk) return;
  double lo = d[0], hi = d[0], emax = 0.0;
  for (int i = 0; i < n; ++i) {
    const double r = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i < n - 1 ? fabs(e[i]) : 0.0);
    lo = fmin(lo, d[i] - r);
    hi = fmax(hi, d[i] + r);
    if (i < n - 1) emax = fmax(emax, e[i] * e[i]);
  }
  const double span = fmax(fabs(lo), fabs(hi));
  lo -= 2.0 * DBL_EPSILON * span + 1e-300;
  hi += 2.0 * DBL_EPSILON * span + 1e-300;
  const double pivmin = 1e-290 * fmax(1.0, emax);
  const int m = n - 1 - j;  // ascending index
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (sturm_count_lt(d, e, n, mid, pivmin) > m) hi = mid;
    else lo = mid;
  }
  evals[j] = 0.5 * (lo + hi);
}

// Inverse iteration for all nk eigenvectors of T, in descending order, one CTA.
// Thread 0 runs the pivoted tridiagonal LU and the solves (sequential by
// nature); the CTA re-orthogonalises against earlier members of the cluster.
constexpr int IV_THREADS = 256;

__global__ void __launch_bounds__(IV_THREADS) inviter_kernel(const double* __restrict__ d, const double* __restrict__ e,
                                                             int n, int nk, const double* __restrict__ evals,
                                                             double* __restrict__ Z, double* __restrict__ work) {
  __shared__ double red[32];
  __shared__ double s_shift;
  double* dl = work;          // L multipliers
  double* dd = work + n;      // U diagonal
  double* du = work + 2 * n;  // U first super-diagonal
  double* du2 = work + 3 * n; // U second super-diagonal
  int* piv = reinterpret_cast<int*>(work + 4 * n);
  double tnorm = 0.0;
  for (int i = 0; i < n; ++i)
    tnorm = fmax(tnorm, fabs(d[i]) + (i > 0 ? fabs(e[i - 1]) : 0.0) + (i < n - 1 ? fabs(e[i]) : 0.0));
  const double ortol = 1e-3 * tnorm;
  const double eps = DBL_EPSILON;
  const double tiny = eps * fmax(tnorm, 1e-300);
  int cluster_start = 0;
  double prev_shift = 0.0;
  for (int j = 0; j < nk; ++j) {
    double lam = evals[j];
    if (j > 0 && fabs(evals[j - 1] - lam) > ortol) cluster_start = j;
    if (j > cluster_start) {
      // separate identical shifts inside a cluster (dstein's perturbation)
      const double pert = 10.0 * eps * fmax(fabs(lam), tnorm * 1e-3);
      if (prev_shift - lam < pert) lam = prev_shift - pert;
    }
    prev_shift = lam;
    double* z = Z + (size_t)j * n;
    // deterministic start vector
    for (int i = threadIdx.x; i < n; i += IV_THREADS) {
      unsigned h = (unsigned)(i * 2654435761u) ^ (unsigned)((j + 1) * 40503u);
      h ^= h >> 13;
      h *= 0x5bd1e995u;
      h ^= h >> 15;
      z[i] = ((double)(h & 0xffffff) / 16777216.0) - 0.5;
    }
    if (threadIdx.x == 0) {
      // LU of T - lam I with partial pivoting (the dgttrf recurrence)
      for (int i = 0; i < n; ++i) {
        dd[i] = d[i] - lam;
        du[i] = i < n - 1 ? e[i] : 0.0;
        dl[i] = i < n - 1 ? e[i] : 0.0;
        du2[i] = 0.0;
      }
      for (int i = 0; i < n - 1; ++i) {
        if (fabs(dd[i]) >= fabs(dl[i])) {
          if (dd[i] == 0.0) dd[i] = tiny;
          const double f = dl[i] / dd[i];
          dl[i] = f;
          dd[i + 1] -= f * du[i];
          du2[i] = 0.0;
          piv[i] = i;
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
          piv[i] = i + 1;
        }
      }
      if (dd[n - 1] == 0.0) dd[n - 1] = tiny;
      for (int i = 0; i < n; ++i)
        if (fabs(dd[i]) < tiny) dd[i] = dd[i] < 0.0 ? -tiny : tiny;
    }
    __syncthreads();
    for (int it = 0; it < 4; ++it) {
      if (threadIdx.x == 0) {
        for (int i = 0; i < n - 1; ++i) {
          if (piv[i] == i) {
            z[i + 1] -= dl[i] * z[i];
          } else {
            const double t = z[i];
            z[i] = z[i + 1];
            z[i + 1] = t - dl[i] * z[i];
          }
        }
        z[n - 1] /= dd[n - 1];
        if (n > 1) z[n - 2] = (z[n - 2] - du[n - 2] * z[n - 1]) / dd[n - 2];
        for (int i = n - 3; i >= 0; --i) z[i] = (z[i] - du[i] * z[i + 1] - du2[i] * z[i + 2]) / dd[i];
      }
      __syncthreads();
      // re-orthogonalise against the earlier members of the cluster (twice)
      for (int pass = 0; pass < 2; ++pass)
        for (int c = cluster_start; c < j; ++c) {
          const double* zc = Z + (size_t)c * n;
          double s = 0.0;
          for (int i = threadIdx.x; i < n; i += IV_THREADS) s += zc[i] * z[i];
          s = block_sum<IV_THREADS>(s, red);
          for (int i = threadIdx.x; i < n; i += IV_THREADS) z[i] -= s * zc[i];
          __syncthreads();
        }
      double s = 0.0;
      for (int i = threadIdx.x; i < n; i += IV_THREADS) s += z[i] * z[i];
      s = block_sum<IV_THREADS>(s, red);
      const double inv = s > 0.0 ? 1.0 / sqrt(s) : 0.0;
      for (int i = threadIdx.x; i < n; i += IV_THREADS) z[i] *= inv;
      __syncthreads();
    }
    (void)s_shift;
  }
}

// y = H_0 H_1 ... H_{n-2} z for eigenvector j = blockIdx.x; H_k = I - tau_k v_k v_k^H
// acting on rows k+1..n-1, v_k stored in A column k.
__global__ void __launch_bounds__(256) backtransform_kernel(const double2* __restrict__ A, int n,
                                                            const double2* __restrict__ tau,
                                                            const double* __restrict__ Z, double2* __restrict__ Y) {
  __shared__ double red[32];
  const int j = blockIdx.x;
  double2* y = Y + (size_t)j * n;
  for (int i = threadIdx.x; i < n; i += 256) y[i] = make_double2(Z[(size_t)j * n + i], 0.0);
  __syncthreads();
  for (int k = n - 2; k >= 0; --k) {
    const int m = n - k - 1;
    double sr = 0.0, si = 0.0;
    for (int i = threadIdx.x; i < m; i += 256) {
      const double2 v = A[(size_t)(k + 1 + i) * n + k];
      const double2 yy = y[k + 1 + i];
      sr += v.x * yy.x + v.y * yy.y;  // conj(v) * y
      si += v.x * yy.y - v.y * yy.x;
    }
    sr = block_sum<256>(sr, red);
    si = block_sum<256>(si, red);
    const double2 f = zmul(tau[k], make_double2(sr, si));
    for (int i = threadIdx.x; i < m; i += 256) {
      const double2 v = A[(size_t)(k + 1 + i) * n + k];
      const double2 p = zmul(f, v);
      y[k + 1 + i].x -= p.x;
      y[k + 1 + i].y -= p.y;
    }
    __syncthreads();
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
  // workspace: vbuf, xbuf, tau (n double2 each); d, e (n double); evals (nk);
  // Z (nk*n double); LU scratch (5n double); Y (nk*n double2)
  const size_t wbytes = 3 * n * sizeof(double2) + 2 * n * sizeof(double) + nk * sizeof(double) +
                        (size_t)nk * n * sizeof(double) + 5 * n * sizeof(double) + (size_t)nk * n * sizeof(double2) +
                        16 * 64;
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
  double* d = reinterpret_cast<double*>(take(n * sizeof(double)));
  double* e = reinterpret_cast<double*>(take(n * sizeof(double)));
  double* ev = reinterpret_cast<double*>(take(nk * sizeof(double)));
  double* Z = reinterpret_cast<double*>(take((size_t)nk * n * sizeof(double)));
  double* lu = reinterpret_cast<double*>(take(5 * n * sizeof(double)));
  double2* Y = reinterpret_cast<double2*>(take((size_t)nk * n * sizeof(double2)));
  double2* A = ctx->eig_v.as<double2>();
  {
    StageScope sc(ctx, LITHO_STAGE_EIG, 4 * (n > 1 ? n - 1 : 0) + 5);
    hermitize_kernel<<<dim3((n + 127) / 128, n), 128, 0, ctx->stream>>>(static_cast<const double2*>(dtcc), A, n);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
    LITHO_CUDA_TRY(ctx, cudaMemsetAsync(e, 0, n * sizeof(double), ctx->stream));
    for (int k = 0; k + 1 < n; ++k) {
      const int m = n - k - 1;
      hh_kernel<<<1, 256, 0, ctx->stream>>>(A, n, k, vbuf, tau, d, e);
      symv_kernel<<<(m + 7) / 8, 256, 0, ctx->stream>>>(A, n, k, vbuf, tau, xbuf);
      wdot_kernel<<<1, 256, 0, ctx->stream>>>(n, k, vbuf, xbuf, tau);
      her2_kernel<<<dim3((m + 31) / 32, (m + 31) / 32), 256, 0, ctx->stream>>>(A, n, k, vbuf, xbuf);
    }
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
    last_diag_kernel<<<1, 32, 0, ctx->stream>>>(A, n, d);
    bisect_kernel<<<(nk + 63) / 64, 64, 0, ctx->stream>>>(d, e, n, nk, ev);
    inviter_kernel<<<1, IV_THREADS, 0, ctx->stream>>>(d, e, n, nk, ev, Z, lu);
    backtransform_kernel<<<nk, 256, 0, ctx->stream>>>(A, n, tau, Z, Y);
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
