// Split-BF16 TCC contraction on the tensor cores (tcgen05, kind::f16 with BF16
// operands, FP32 accumulation in TMEM).
//
// With a_s = sqrt(J_s) p_s, TCC = A A^H for A = [a_1 .. a_Ns] (tcc x Ns complex).
// In real arithmetic, with X = [Re A | Im A] and Y = [Im A | -Re A] (tcc x 2Ns):
//     Re TCC = X X^T,   Im TCC = Y X^T,
// i.e. one real GEMM C (2 tcc x tcc) = [X; Y] X^T.  Each operand is split into
// BF16 hi + lo terms (hi = bf16(v), lo = bf16(v - hi)) and the GEMM issues
// hi*hi + hi*lo + lo*hi per K slice (the three-term split product).
//
// split_kernel      P (complex float), J -> Ah/Al = [X; Y] and Bh/Bl = X, BF16,
//                   K-major rows padded to Kp (multiple of 64).
// gemm_bf16x3_kernel  128 x 128 output tile per CTA, K streamed in 64-wide
//                   (128-byte) slices through a 3-stage TMA/mbarrier ring; one
//                   thread issues 12 MMAs per slice; epilogue tcgen05.ld -> FP32 C.
// assemble_kernel   C -> interleaved complex128 TCC: upper triangle from C, the
//                   lower triangle its conjugate mirror (litho.cpp:510-515).
#include "litho_internal.cuh"
#include "tc_common.cuh"

#include <cuda_bf16.h>
#include <cudaTypedefs.h>

namespace litho {
using namespace tc;

__global__ void split_kernel(const float2* __restrict__ P, const float* __restrict__ J, int n, int ns, int ldp,
                             int Kp, __nv_bfloat16* __restrict__ Ah, __nv_bfloat16* __restrict__ Al,
                             __nv_bfloat16* __restrict__ Bh, __nv_bfloat16* __restrict__ Bl) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;  // column in [0, Kp)
  const int i = blockIdx.y;                             // pupil row in [0, n)
  if (k >= Kp || i >= n) return;
  float x = 0.f, y = 0.f;  // X[i][k], Y[i][k]
  const int s = k < ns ? k : k - ns;
  if (k < 2 * ns) {
    const float w = sqrtf(J[s]);
    const float2 p = P[(size_t)i * ldp + s];
    const float ar = w * p.x, ai = w * p.y;
    if (k < ns) {
      x = ar;
      y = ai;
    } else {
      x = ai;
      y = -ar;
    }
  }
  const __nv_bfloat16 xh = __float2bfloat16_rn(x), yh = __float2bfloat16_rn(y);
  const __nv_bfloat16 xl = __float2bfloat16_rn(x - __bfloat162float(xh));
  const __nv_bfloat16 yl = __float2bfloat16_rn(y - __bfloat162float(yh));
  Ah[(size_t)i * Kp + k] = xh;
  Al[(size_t)i * Kp + k] = xl;
  Ah[(size_t)(n + i) * Kp + k] = yh;
  Al[(size_t)(n + i) * Kp + k] = yl;
  Bh[(size_t)i * Kp + k] = xh;
  Bl[(size_t)i * Kp + k] = xl;
}

constexpr int GB_STAGES = 3;
constexpr uint32_t GB_TILE = 128 * 128;          // 128 rows x 64 bf16
constexpr uint32_t GB_STAGE_B = 4 * GB_TILE;     // Ah, Al, Bh, Bl
constexpr size_t GB_SMEM = 1024 + (size_t)GB_STAGES * GB_STAGE_B + 256;

__global__ void __launch_bounds__(128, 1) gemm_bf16x3_kernel(const __grid_constant__ CUtensorMap tAh,
                                                             const __grid_constant__ CUtensorMap tAl,
                                                             const __grid_constant__ CUtensorMap tBh,
                                                             const __grid_constant__ CUtensorMap tBl, int M, int N,
                                                             int Kp, float* __restrict__ C, int* __restrict__ err) {
  extern __shared__ unsigned char smraw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + GB_STAGES * GB_STAGE_B);
  uint64_t* empty = full + GB_STAGES;
  uint64_t* done = empty + GB_STAGES;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * 128, n0 = blockIdx.y * 128;
  const int nch = Kp / 64;

  if (warp == 0) tmem_alloc(tslot, 128);
  if (tid == 0) {
    for (int s = 0; s < GB_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    fence_mbar_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  auto tile = [&](int s, int q) { return sm + (size_t)s * GB_STAGE_B + (size_t)q * GB_TILE; };
  auto issue = [&](int c) {
    const int s = c % GB_STAGES;
    mbar_arrive_expect_tx(&full[s], GB_STAGE_B);
    tma_load_2d(tile(s, 0), &tAh, &full[s], 64 * c, m0);
    tma_load_2d(tile(s, 1), &tAl, &full[s], 64 * c, m0);
    tma_load_2d(tile(s, 2), &tBh, &full[s], 64 * c, n0);
    tma_load_2d(tile(s, 3), &tBl, &full[s], 64 * c, n0);
  };
  constexpr uint32_t IDESC = idesc_bf16(128, 128);
  int bad = 0, c = 0, issued = 0;
  if (tid == 0) {
    for (; issued < min(nch, GB_STAGES); ++issued) issue(issued);
    for (; c < nch; ++c) {
      const int s = c % GB_STAGES;
      const uint32_t ph = (uint32_t)(c / GB_STAGES) & 1u;
      if (!mbar_wait(&full[s], ph)) {
        bad = 1;
        break;
      }
      tc_fence_after();
      const uint64_t dah = desc_sw128(tile(s, 0)), dal = desc_sw128(tile(s, 1));
      const uint64_t dbh = desc_sw128(tile(s, 2)), dbl = desc_sw128(tile(s, 3));
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const uint32_t off = kk * 32;  // 16 bf16 per MMA
        mma_bf16(tmem, desc_add(dah, off), desc_add(dbh, off), IDESC, (c | kk) != 0 ? 1u : 0u);
        mma_bf16(tmem, desc_add(dah, off), desc_add(dbl, off), IDESC, 1u);
        mma_bf16(tmem, desc_add(dal, off), desc_add(dbh, off), IDESC, 1u);
      }
      mma_commit(&empty[s]);
      if (issued < nch) {
        if (!mbar_wait(&empty[s], ph)) {
          bad = 1;
          ++c;
          break;
        }
        issue(issued++);
      }
    }
    mma_commit(done);
    if (!mbar_wait(done, 0)) bad = 1;
    if (bad) {
      atomicExch(err, 1);
      for (int k = c; k < issued; ++k) mbar_wait(&full[k % GB_STAGES], (uint32_t)(k / GB_STAGES) & 1u, 200u);
    }
  }
  if (__syncthreads_or(bad)) {
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 128);
    return;
  }
  tc_fence_after();
  const int row = m0 + 32 * warp + lane;
  const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);
#pragma unroll 1
  for (int slab = 0; slab < 4; ++slab) {
    float v[32];
    tmem_ld32(trow + (uint32_t)(slab * 32), v);
    if (row < M) {
      float* out = C + (size_t)row * N + n0 + slab * 32;
#pragma unroll
      for (int j = 0; j < 32; ++j)
        if (n0 + slab * 32 + j < N) out[j] = v[j];
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 128);
}

__global__ void assemble_kernel(const float* __restrict__ C, int n, double2* __restrict__ tcc) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (i >= n || j >= n) return;
  double2 v;
  if (i < j) v = make_double2(C[(size_t)i * n + j], C[(size_t)(n + i) * n + j]);
  else if (i > j) v = make_double2(C[(size_t)j * n + i], -(double)C[(size_t)(n + j) * n + i]);
  else v = make_double2(C[(size_t)i * n + i], 0.0);
  tcc[(size_t)i * n + j] = v;
}

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn_bf16() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (fn == nullptr) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

static int map_bf16(litho_ctx* ctx, CUtensorMap* m, const void* base, uint64_t cols, uint64_t rows) {
  auto fn = encode_fn_bf16();
  if (fn == nullptr) {
    set_error(ctx, LITHO_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    return LITHO_ERR_CUDA;
  }
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {cols * 2};
  cuuint32_t box[2] = {64, 128};
  cuuint32_t es[2] = {1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error(ctx, LITHO_ERR_CUDA, "cuTensorMapEncodeTiled (bf16) failed (%d)", (int)r);
    return LITHO_ERR_CUDA;
  }
  return LITHO_OK;
}

int tc_err_flag_public(litho_ctx* ctx, int** flag);

int tcc_split_bf16(litho_ctx* ctx, const float2* P, const float* J, int n, int ns, int ldp, double2* tcc) {
  const int Kp = ((2 * ns + 63) / 64) * 64;
  const size_t op = (size_t)Kp * sizeof(__nv_bfloat16);
  // A: 2n rows (hi, lo), B: n rows (hi, lo), C: 2n x n fp32
  LITHO_RET(ctx->mx_c.ensure(ctx, op * (4 * (size_t)n + 2 * (size_t)n) + (size_t)2 * n * n * sizeof(float) + 4096));
  char* base = ctx->mx_c.as<char>();
  auto take = [&](size_t b) {
    char* p = base;
    base += (b + 1023) & ~size_t(1023);
    return p;
  };
  __nv_bfloat16* Ah = reinterpret_cast<__nv_bfloat16*>(take(op * 2 * n));
  __nv_bfloat16* Al = reinterpret_cast<__nv_bfloat16*>(take(op * 2 * n));
  __nv_bfloat16* Bh = reinterpret_cast<__nv_bfloat16*>(take(op * n));
  __nv_bfloat16* Bl = reinterpret_cast<__nv_bfloat16*>(take(op * n));
  float* C = reinterpret_cast<float*>(take((size_t)2 * n * n * sizeof(float)));
  split_kernel<<<dim3((Kp + 127) / 128, n), 128, 0, ctx->stream>>>(P, J, n, ns, ldp, Kp, Ah, Al, Bh, Bl);
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  CUtensorMap mAh, mAl, mBh, mBl;
  LITHO_RET(map_bf16(ctx, &mAh, Ah, Kp, 2 * n));
  LITHO_RET(map_bf16(ctx, &mAl, Al, Kp, 2 * n));
  LITHO_RET(map_bf16(ctx, &mBh, Bh, Kp, n));
  LITHO_RET(map_bf16(ctx, &mBl, Bl, Kp, n));
  int* err = nullptr;
  LITHO_RET(tc_err_flag_public(ctx, &err));
  LITHO_CUDA_TRY(ctx, cudaFuncSetAttribute(gemm_bf16x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)GB_SMEM));
  dim3 grid((2 * n + 127) / 128, (n + 127) / 128);
  gemm_bf16x3_kernel<<<grid, 128, GB_SMEM, ctx->stream>>>(mAh, mAl, mBh, mBl, 2 * n, n, Kp, C, err);
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  assemble_kernel<<<dim3((n + 127) / 128, n), 128, 0, ctx->stream>>>(C, n, tcc);
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  return LITHO_OK;
}

}  // namespace litho
