// TCC assembly (litho.cpp:428-516 calcTCC):
//   TCC[i][j] = sum_s J_s P_s(i) conj(P_s(j)),  P_s(n) = exp(i dz k sqrt(1 - rho^2 NA^2))
// over the lit source points s and the pupil support rho^2 <= 1 around each.
//
// pupil_kernel  builds P (tccSize x Ns, complex float) with the reference's own
//               float32 operation order: every product, quotient and sum is
//               rounded separately (no FMA contraction), so the support tests
//               `fy*fy <= 1` and `rho2 <= 1` take the same branch as litho.cpp
//               on every grid point.
// tcc_fp64_kernel  FP64 Hermitian contraction over upper-triangle tiles with the
//               conjugate mirror written in the same pass (litho.cpp:510-515).
// The split-BF16 tensor-core contraction lives in tcc_tc.cu.
#include "litho_internal.cuh"

#include <cmath>
#include <vector>

namespace litho {

struct PupilParams {
  int Nx, Ny, tccSize, ns;
  int sh;
  float Lx_norm, Ly_norm, dzk, NA;
  double nm2;  // immersion index squared: 1 reproduces litho.cpp:463
};

// The reference's per-source support bounds (litho.cpp:449-454): C truncation.
struct SrcPt {
  int p, q;
  float J;
};

// One CTA per pupil row id, threads along the source points s: the row P[id][*] is
// written with consecutive 8-byte stores, the padding columns s >= ns as zeros.
__global__ void pupil_kernel(const int2* __restrict__ pq, PupilParams pp, float2* __restrict__ P, int ldp) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int id = blockIdx.y;
  if (s >= ldp || id >= pp.tccSize) return;
  if (s >= pp.ns) {
    P[(size_t)id * ldp + s] = make_float2(0.f, 0.f);
    return;
  }
  const int2 src = pq[s];
  const int KX = 2 * pp.Nx + 1;
  const int ny = id / KX - pp.Ny, nx = id % KX - pp.Nx;
  const float sx = __fdiv_rn((float)src.x, (float)pp.sh);
  const float sy = __fdiv_rn((float)src.y, (float)pp.sh);
  const int nxMin = (int)__fmul_rn(-1.0f - sx, pp.Lx_norm);
  const int nxMax = (int)__fmul_rn(1.0f - sx, pp.Lx_norm);
  const int nyMin = (int)__fmul_rn(-1.0f - sy, pp.Ly_norm);
  const int nyMax = (int)__fmul_rn(1.0f - sy, pp.Ly_norm);
  float2 v = make_float2(0.f, 0.f);
  if (nx >= nxMin && nx <= nxMax && ny >= nyMin && ny <= nyMax) {
    const float fy = __fadd_rn(__fdiv_rn((float)ny, pp.Ly_norm), sy);
    if (__fmul_rn(fy, fy) <= 1.0f) {
      const float fx = __fadd_rn(__fdiv_rn((float)nx, pp.Lx_norm), sx);
      const float rho2 = __fadd_rn(__fmul_rn(fx, fx), __fmul_rn(fy, fy));
      if ((double)rho2 <= 1.0) {
        const float r = __fmul_rn(__fmul_rn(rho2, pp.NA), pp.NA);
        const double val = (double)pp.dzk * sqrt(pp.nm2 - (double)r);
        const float ph = (float)val;
        float sn, cs;
        sincosf(ph, &sn, &cs);
        v = make_float2(cs, sn);
      }
    }
  }
  P[(size_t)id * ldp + s] = v;
}

// Upper-triangle tiles of TCC in FP64; tile (bi, bj) with bi <= bj.  Each CTA
// computes a 32 x 32 tile with 256 threads (2 x 2 complex outputs per thread).
constexpr int TT = 32, TK = 16;

__global__ void __launch_bounds__(256) tcc_fp64_kernel(const float2* __restrict__ P, const float* __restrict__ J,
                                                       int n, int ns, int ldp, double2* __restrict__ tcc) {
  // map the linear block index onto the upper triangle of the tile grid
  const int nt = (n + TT - 1) / TT;
  int b = blockIdx.x, bi = 0;
  while (b >= nt - bi) {
    b -= nt - bi;
    ++bi;
  }
  const int bj = bi + b;
  __shared__ double2 sA[TK][TT + 1];
  __shared__ double2 sB[TK][TT + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int i0 = bi * TT, j0 = bj * TT;
  double2 acc[2][2];
  for (int a = 0; a < 2; ++a)
    for (int c = 0; c < 2; ++c) acc[a][c] = make_double2(0.0, 0.0);
  for (int k0 = 0; k0 < ns; k0 += TK) {
    for (int idx = threadIdx.x; idx < TK * TT; idx += 256) {
      const int r = idx / TK, k = idx % TK;
      const int s = k0 + k;
      double2 a = make_double2(0.0, 0.0), bb = make_double2(0.0, 0.0);
      if (s < ns) {
        const double w = (double)J[s];
        if (i0 + r < n) {
          const float2 t = P[(size_t)(i0 + r) * ldp + s];
          a = make_double2(w * t.x, w * t.y);
        }
        if (j0 + r < n) {
          const float2 t = P[(size_t)(j0 + r) * ldp + s];
          bb = make_double2(t.x, t.y);
        }
      }
      sA[k][r] = a;
      sB[k][r] = bb;
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < TK; ++k) {
      const double2 a0 = sA[k][ty], a1 = sA[k][ty + 16];
      const double2 b0 = sB[k][tx], b1 = sB[k][tx + 16];
      const double2 av[2] = {a0, a1}, bv[2] = {b0, b1};
      for (int a = 0; a < 2; ++a)
        for (int c = 0; c < 2; ++c) {
          // a * conj(b)
          acc[a][c].x = fma(av[a].x, bv[c].x, fma(av[a].y, bv[c].y, acc[a][c].x));
          acc[a][c].y = fma(av[a].y, bv[c].x, fma(-av[a].x, bv[c].y, acc[a][c].y));
        }
    }
    __syncthreads();
  }
  for (int a = 0; a < 2; ++a)
    for (int c = 0; c < 2; ++c) {
      const int i = i0 + ty + 16 * a, j = j0 + tx + 16 * c;
      if (i >= n || j >= n || i > j) continue;
      double2 v = acc[a][c];
      if (i == j) v.y = 0.0;  // the reference's diagonal sum J|p|^2 is exactly real
      tcc[(size_t)i * n + j] = v;
      if (i != j) tcc[(size_t)j * n + i] = make_double2(v.x, -v.y);
    }
}

// Host side: enumerate lit source points in the reference's loop order and
// check that every pupil point the reference would store lies on the grid.
int tcc_sources(litho_ctx* ctx, const float* src_h, int S, float outerSigma, float wavelength, float NA,
                float defocus, int Lx, int Ly, int Nx, int Ny, std::vector<SrcPt>& pts, PupilParams& pp,
                int sh_in = -1, int oSgm_in = -1, float n_medium = 1.0f) {
  // litho.cpp:429-430; the FPGA top (calc_tcc.cpp:34-42) receives sh and oSgm from its caller instead
  const int sh = sh_in >= 0 ? sh_in : (int)((S - 1) / 2.0);
  volatile float osf = (float)sh * outerSigma;
  const int oSgm = oSgm_in >= 0 ? oSgm_in : (int)std::ceil((float)osf);
  if (sh <= 0) {
    set_error(ctx, LITHO_ERR_ARG, "source grid %d too small (sh = %d)", S, sh);
    return LITHO_ERR_ARG;
  }
  volatile float nana = NA * NA;
  volatile float q0 = nana / wavelength;
  volatile float dz = defocus / q0;
  const float k = (float)(2 * M_PI / wavelength);
  volatile float lxn = (float)Lx * NA;
  volatile float lyn = (float)Ly * NA;
  const float Lx_norm = lxn / wavelength, Ly_norm = lyn / wavelength;
  volatile float dzk = dz * k;
  pp = PupilParams{Nx, Ny, (2 * Nx + 1) * (2 * Ny + 1), 0, sh, Lx_norm, Ly_norm, (float)dzk, NA,
                   (double)n_medium * (double)n_medium};
  pts.clear();
  for (int q = -oSgm; q <= oSgm; ++q)
    for (int p = -oSgm; p <= oSgm; ++p) {
      if (p * p + q * q > sh * sh) continue;
      const int id = (q + sh) * S + p + sh;
      if (id < 0 || id >= S * S) continue;
      if (src_h[id] == 0.0f) continue;
      pts.push_back({p, q, src_h[id]});
      // support check (litho.cpp would write outside its pupil table otherwise)
      volatile float sx = (float)p / (float)sh, sy = (float)q / (float)sh;
      volatile float a = (-1.0f - sx) * Lx_norm, b = (1.0f - sx) * Lx_norm;
      volatile float c = (-1.0f - sy) * Ly_norm, d = (1.0f - sy) * Ly_norm;
      const int nxMin = (int)a, nxMax = (int)b, nyMin = (int)c, nyMax = (int)d;
      if (nxMin >= -Nx && nxMax <= Nx && nyMin >= -Ny && nyMax <= Ny) continue;
      for (int ny = nyMin; ny <= nyMax; ++ny) {
        volatile float fy0 = (float)ny / Ly_norm;
        volatile float fy = fy0 + sy;
        volatile float fyy = fy * fy;
        if (!(fyy <= 1.0f)) continue;
        for (int nx = nxMin; nx <= nxMax; ++nx) {
          if (nx >= -Nx && nx <= Nx && ny >= -Ny && ny <= Ny) continue;
          volatile float fx0 = (float)nx / Lx_norm;
          volatile float fx = fx0 + sx;
          volatile float fxx = fx * fx;
          volatile float rho2 = fxx + fyy;
          if ((double)rho2 <= 1.0) {
            set_error(ctx, LITHO_ERR_ARG,
                      "pupil point (nx=%d, ny=%d) of source (%d, %d) lies outside the (2Nx+1)x(2Ny+1) grid "
                      "(Nx=%d, Ny=%d)", nx, ny, p, q, Nx, Ny);
            return LITHO_ERR_ARG;
          }
        }
      }
    }
  pp.ns = (int)pts.size();
  return LITHO_OK;
}

int build_pupil(litho_ctx* ctx, const std::vector<SrcPt>& pts, const PupilParams& pp, float2* P, int ldp,
                float* J_dev, DevBuf& pqbuf) {
  const int ns = (int)pts.size();
  std::vector<int2> pq(ns);
  std::vector<float> J(ns);
  for (int i = 0; i < ns; ++i) {
    pq[i] = make_int2(pts[i].p, pts[i].q);
    J[i] = pts[i].J;
  }
  LITHO_RET(pqbuf.ensure(ctx, (size_t)ns * sizeof(int2)));
  LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(pqbuf.p, pq.data(), (size_t)ns * sizeof(int2), cudaMemcpyHostToDevice, ctx->stream));
  LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(J_dev, J.data(), (size_t)ns * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  dim3 grid((ldp + 127) / 128, pp.tccSize);
  pupil_kernel<<<grid, 128, 0, ctx->stream>>>(pqbuf.as<int2>(), pp, P, ldp);
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  // the host vectors must outlive the async copies
  LITHO_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return LITHO_OK;
}

int tcc_split_bf16(litho_ctx* ctx, const float2* P, const float* J, int n, int ns, int ldp, double2* tcc);
cudaError_t launch_nonfinite(cudaStream_t s, const double* x, size_t n, int* flag, int sms);
int tc_err_flag_public(litho_ctx* ctx, int** flag);

}  // namespace litho

using namespace litho;

// sh_in / oSgm_in >= 0 override the source half-size and loop bound (the FPGA
// top receives them from its caller); -1 derives them as litho.cpp:429-430.
int litho::calc_tcc_impl(litho_ctx* ctx, const float* src, int srcSize, float outerSigma, float wavelength,
                         float NA, float defocus, int Lx, int Ly, int Nx, int Ny, double* tcc, int tccPrecision,
                         int mem, int sh_in, int oSgm_in, float n_medium) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  LITHO_ARG_CHECK(ctx, src && tcc, "null pointer");
  LITHO_ARG_CHECK(ctx, srcSize >= 1 && srcSize <= 4097, "srcSize %d outside [1, 4097]", srcSize);
  LITHO_ARG_CHECK(ctx, Nx >= 0 && Ny >= 0 && (2 * Nx + 1) * (2 * Ny + 1) <= 8192, "tccSize too large");
  LITHO_ARG_CHECK(ctx, Lx >= 1 && Ly >= 1 && NA > 0.f && wavelength > 0.f, "bad optics");
  LITHO_ARG_CHECK(ctx, outerSigma >= 0.f && outerSigma <= 1.f, "outerSigma %g outside [0, 1] (litho.cpp:1298 clamps)",
                  outerSigma);
  LITHO_ARG_CHECK(ctx, tccPrecision == LITHO_TCC_FP64 || tccPrecision == LITHO_TCC_SPLIT_BF16, "bad tccPrecision");
  LITHO_ARG_CHECK(ctx, n_medium > 0.f && std::isfinite(n_medium), "n_medium %g must be positive", n_medium);
  LITHO_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  std::vector<float> src_h;
  const float* sh = src;
  if (mem == LITHO_MEM_DEVICE) {
    src_h.resize((size_t)srcSize * srcSize);
    LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(src_h.data(), src, src_h.size() * sizeof(float), cudaMemcpyDeviceToHost,
                                        ctx->stream));
    LITHO_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    sh = src_h.data();
  }
  std::vector<SrcPt> pts;
  PupilParams pp;
  LITHO_RET(tcc_sources(ctx, sh, srcSize, outerSigma, wavelength, NA, defocus, Lx, Ly, Nx, Ny, pts, pp, sh_in,
                        oSgm_in, n_medium));
  const int n = pp.tccSize, ns = pp.ns;
  const int ldp = ((ns + 63) / 64) * 64 + 64;  // padded, multiple of 64 (tensor-core K tiles)
  LITHO_RET(ctx->tcc_a.ensure(ctx, (size_t)n * ldp * sizeof(float2)));
  LITHO_RET(ctx->tcc_b.ensure(ctx, (size_t)ldp * sizeof(float)));
  double2* out = reinterpret_cast<double2*>(tcc);
  const size_t out_bytes = (size_t)n * n * sizeof(double2);
  if (mem == LITHO_MEM_HOST) {
    LITHO_RET(ctx->tcc_c.ensure(ctx, out_bytes));
    out = ctx->tcc_c.as<double2>();
  }
  float2* P = ctx->tcc_a.as<float2>();
  float* J = ctx->tcc_b.as<float>();
  {
    StageScope sc(ctx, LITHO_STAGE_TCC, 2);
    LITHO_CUDA_TRY(ctx, cudaMemsetAsync(J, 0, (size_t)ldp * sizeof(float), ctx->stream));
    LITHO_CUDA_TRY(ctx, cudaMemsetAsync(out, 0, out_bytes, ctx->stream));
    if (ns > 0) {
      LITHO_RET(build_pupil(ctx, pts, pp, P, ldp, J, ctx->tcc_pq));
      if (tccPrecision == LITHO_TCC_SPLIT_BF16) {
        LITHO_RET(tcc_split_bf16(ctx, P, J, n, ns, ldp, out));
      } else {
        const int nt = (n + TT - 1) / TT;
        tcc_fp64_kernel<<<nt * (nt + 1) / 2, 256, 0, ctx->stream>>>(P, J, n, ns, ldp, out);
        LITHO_CUDA_TRY(ctx, cudaGetLastError());
      }
    }
  }
  if (mem == LITHO_MEM_HOST) {
    // finiteness is checked on the device while the result is still there
    int* flag = nullptr;
    LITHO_RET(tc_err_flag_public(ctx, &flag));
    flag += 32;  // past the tensor-core kernels' timeout flag
    LITHO_CUDA_TRY(ctx, cudaMemsetAsync(flag, 0, sizeof(int), ctx->stream));
    LITHO_CUDA_TRY(ctx, launch_nonfinite(ctx->stream, reinterpret_cast<const double*>(out), (size_t)2 * n * n, flag,
                                         ctx->sm_count));
    int bad = 0;
    LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(tcc, out, out_bytes, cudaMemcpyDeviceToHost, ctx->stream));
    LITHO_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (tccPrecision == LITHO_TCC_SPLIT_BF16) LITHO_RET(tc_check_flag(ctx));
    if (bad) {
      set_error(ctx, LITHO_ERR_NAN,
                "non-finite TCC entry (NA > n_medium makes the pupil phase NaN, litho.cpp:463; "
                "litho_calc_tcc_medium takes an immersion index)");
      return LITHO_ERR_NAN;
    }
  }
  return LITHO_OK;
}

extern "C" int litho_calc_tcc(litho_ctx* ctx, const float* src, int srcSize, float outerSigma, float wavelength,
                              float NA, float defocus, int Lx, int Ly, int Nx, int Ny, double* tcc, int tccPrecision,
                              int mem) {
  return litho::calc_tcc_impl(ctx, src, srcSize, outerSigma, wavelength, NA, defocus, Lx, Ly, Nx, Ny, tcc,
                              tccPrecision, mem, -1, -1);
}

// Immersion extension: the pupil phase dz k sqrt(n^2 - rho^2 NA^2) (n = 1 is litho.cpp:463,
// which is NaN wherever rho NA > 1, even at zero defocus)
extern "C" int litho_calc_tcc_medium(litho_ctx* ctx, const float* src, int srcSize, float outerSigma,
                                     float wavelength, float NA, float defocus, float n_medium, int Lx, int Ly,
                                     int Nx, int Ny, double* tcc, int tccPrecision, int mem) {
  return litho::calc_tcc_impl(ctx, src, srcSize, outerSigma, wavelength, NA, defocus, Lx, Ly, Nx, Ny, tcc,
                              tccPrecision, mem, -1, -1, n_medium);
}
