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
// split_kernel      P (complex float), J -> Ah/Al = [X; Y], BF16, K-major rows
//                   padded to Kp (multiple of 64); the B operand X is A's first
//                   n rows (tensor maps over the same memory).
// gemm_bf16x3_kernel  128 x 128 output tile per CTA (only the tiles the TCC
//                   reads), K streamed in 64-wide (128-byte) slices through a
//                   3-stage TMA/mbarrier ring; a producer lane refills the ring
//                   while the MMA lane issues 12 MMAs per slice; epilogue
//                   tcgen05.ld -> FP32 C.
// assemble_kernel   C -> interleaved complex128 TCC: upper triangle from C, the
//                   lower triangle its conjugate mirror (litho.cpp:510-515).
#include "litho_internal.cuh"
#include "tc_common.cuh"
#include "tcc_tiles.hpp"

#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <vector>

namespace litho {
using namespace tc;

// eight consecutive columns k per thread: 16-byte stores of the BF16 rows
__global__ void split_kernel(const float2* __restrict__ P, const float* __restrict__ J, int n, int ns, int ldp,
                             int Kp, __nv_bfloat16* __restrict__ Ah, __nv_bfloat16* __restrict__ Al) {
  const int k0 = 8 * (blockIdx.x * blockDim.x + threadIdx.x);  // first column, in [0, Kp)
  const int i = blockIdx.y;                                     // pupil row in [0, n)
  if (k0 >= Kp || i >= n) return;
  __align__(16) __nv_bfloat16 xh[8], xl[8], yh[8], yl[8];
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int k = k0 + u;
    float x = 0.f, y = 0.f;  // X[i][k], Y[i][k]
    if (k < 2 * ns) {
      const int s = k < ns ? k : k - ns;
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
    xh[u] = __float2bfloat16_rn(x);
    yh[u] = __float2bfloat16_rn(y);
    xl[u] = __float2bfloat16_rn(x - __bfloat162float(xh[u]));
    yl[u] = __float2bfloat16_rn(y - __bfloat162float(yh[u]));
  }
  *reinterpret_cast<uint4*>(Ah + (size_t)i * Kp + k0) = *reinterpret_cast<const uint4*>(xh);
  *reinterpret_cast<uint4*>(Al + (size_t)i * Kp + k0) = *reinterpret_cast<const uint4*>(xl);
  *reinterpret_cast<uint4*>(Ah + (size_t)(n + i) * Kp + k0) = *reinterpret_cast<const uint4*>(yh);
  *reinterpret_cast<uint4*>(Al + (size_t)(n + i) * Kp + k0) = *reinterpret_cast<const uint4*>(yl);
}

constexpr int GB_STAGES = 3;
constexpr uint32_t GB_TILE = 128 * 128;          // 128 rows x 64 bf16
constexpr uint32_t GB_STAGE_B = 4 * GB_TILE;     // Ah, Al, Bh, Bl
constexpr size_t GB_SMEM = 1024 + (size_t)GB_STAGES * GB_STAGE_B + 256;

// One 128 x 128 tile of C = A B^T per CTA, the tile taken from a list (only the
// tiles the TCC reads, in blocks that share operand panels in L2).  Warp 0 lane 0
// streams the K slices through the TMA ring, warp 1 lane 0 issues the MMAs as the
// slices land (so the tensor pipe is not idle while a stage is refilled), then all
// four warps drain TMEM with 16-byte stores (ldc a multiple of 4).
__global__ void __launch_bounds__(128, 1) gemm_bf16x3_kernel(const __grid_constant__ CUtensorMap tAh,
                                                             const __grid_constant__ CUtensorMap tAl,
                                                             const __grid_constant__ CUtensorMap tBh,
                                                             const __grid_constant__ CUtensorMap tBl,
                                                             const int2* __restrict__ tiles, int M, int N,
                                                             int Kp, float* __restrict__ C, int ldc,
                                                             int* __restrict__ err) {
  extern __shared__ unsigned char smraw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + GB_STAGES * GB_STAGE_B);
  uint64_t* empty = full + GB_STAGES;
  uint64_t* done = empty + GB_STAGES;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
  int* s_bad = reinterpret_cast<int*>(tslot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int2 tl = tiles[blockIdx.x];
  const int m0 = tl.x * 128, n0 = tl.y * 128;
  const int nch = Kp / 64;

  if (warp == 0) tmem_alloc(tslot, 128);
  if (tid == 0) {
    for (int s = 0; s < GB_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *s_bad = 0;
    fence_mbar_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  auto tile = [&](int s, int q) { return sm + (size_t)s * GB_STAGE_B + (size_t)q * GB_TILE; };
  volatile int* bad = s_bad;
  if (tid == 0) {  // TMA producer
    int issued = 0;
    for (; issued < nch; ++issued) {
      const int s = issued % GB_STAGES;
      if (issued >= GB_STAGES &&
          !mbar_wait_ab(&empty[s], (uint32_t)(issued / GB_STAGES - 1) & 1u, bad))
        break;
      mbar_arrive_expect_tx(&full[s], GB_STAGE_B);
      tma_load_2d(tile(s, 0), &tAh, &full[s], 64 * issued, m0);
      tma_load_2d(tile(s, 1), &tAl, &full[s], 64 * issued, m0);
      tma_load_2d(tile(s, 2), &tBh, &full[s], 64 * issued, n0);
      tma_load_2d(tile(s, 3), &tBl, &full[s], 64 * issued, n0);
    }
    if (issued < nch) {
      *bad = 1;
      // wait (bounded) for the loads still in flight before the CTA leaves
      for (int k = (issued > GB_STAGES ? issued - GB_STAGES : 0); k < issued; ++k)
        mbar_wait(&full[k % GB_STAGES], (uint32_t)(k / GB_STAGES) & 1u, 200u);
    }
  } else if (tid == 32) {  // MMA issuer
    constexpr uint32_t IDESC = idesc_bf16(128, 128);
    for (int c = 0; c < nch; ++c) {
      const int s = c % GB_STAGES;
      if (!mbar_wait_ab(&full[s], (uint32_t)(c / GB_STAGES) & 1u, bad)) {
        *bad = 1;
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
    }
    mma_commit(done);  // arrives once everything issued above has completed
  }
  __syncwarp();
  if (!mbar_wait(done, 0)) *bad = 1;
  if (__syncthreads_or(*bad)) {
    if (tid == 0) atomicExch(err, 1);
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
    const int c0 = n0 + slab * 32;
    if (row < M && c0 < N) {
      float* out = C + (size_t)row * ldc + c0;
      if (c0 + 32 <= ldc) {
#pragma unroll
        for (int j = 0; j < 32; j += 4) *reinterpret_cast<float4*>(out + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
      } else {
#pragma unroll
        for (int j = 0; j < 32; ++j)
          if (c0 + j < N) out[j] = v[j];
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 128);
}

__global__ void assemble_kernel(const float* __restrict__ C, int n, int ldc, double2* __restrict__ tcc) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (i >= n || j >= n) return;
  double2 v;
  if (i < j) v = make_double2(C[(size_t)i * ldc + j], C[(size_t)(n + i) * ldc + j]);
  else if (i > j) v = make_double2(C[(size_t)j * ldc + i], -(double)C[(size_t)(n + j) * ldc + i]);
  else v = make_double2(C[(size_t)i * ldc + i], 0.0);
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
  const int ldc = (n + 3) & ~3;  // 16-byte rows for the epilogue's vector stores
  // only the output tiles the TCC assembly reads (about half), in L2-friendly blocks
  const std::vector<TileMN> need = tcc_needed_tiles(n);
  std::vector<int2> tiles(need.size());
  for (size_t i = 0; i < need.size(); ++i) tiles[i] = make_int2(need[i].m, need[i].n);
  // A: 2n rows (hi, lo); B is A's first n rows; C: 2n x ldc fp32; the tile list
  const size_t cbytes = (size_t)2 * n * ldc * sizeof(float);
  LITHO_RET(ctx->mx_c.ensure(ctx, op * 4 * (size_t)n + cbytes + tiles.size() * sizeof(int2) + 4096));
  char* base = ctx->mx_c.as<char>();
  auto take = [&](size_t b) {
    char* p = base;
    base += (b + 1023) & ~size_t(1023);
    return p;
  };
  __nv_bfloat16* Ah = reinterpret_cast<__nv_bfloat16*>(take(op * 2 * n));
  __nv_bfloat16* Al = reinterpret_cast<__nv_bfloat16*>(take(op * 2 * n));
  float* C = reinterpret_cast<float*>(take(cbytes));
  int2* dtiles = reinterpret_cast<int2*>(take(tiles.size() * sizeof(int2)));
  LITHO_CUDA_TRY(ctx, cudaMemcpyAsync(dtiles, tiles.data(), tiles.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                      ctx->stream));
  split_kernel<<<dim3((Kp / 8 + 127) / 128, n), 128, 0, ctx->stream>>>(P, J, n, ns, ldp, Kp, Ah, Al);
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  CUtensorMap mAh, mAl, mBh, mBl;
  LITHO_RET(map_bf16(ctx, &mAh, Ah, Kp, 2 * n));
  LITHO_RET(map_bf16(ctx, &mAl, Al, Kp, 2 * n));
  LITHO_RET(map_bf16(ctx, &mBh, Ah, Kp, n));
  LITHO_RET(map_bf16(ctx, &mBl, Al, Kp, n));
  int* err = nullptr;
  LITHO_RET(tc_err_flag_public(ctx, &err));
  LITHO_CUDA_TRY(ctx, cudaFuncSetAttribute(gemm_bf16x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)GB_SMEM));
  gemm_bf16x3_kernel<<<(unsigned)tiles.size(), 128, GB_SMEM, ctx->stream>>>(mAh, mAl, mBh, mBl, dtiles, 2 * n, n, Kp,
                                                                             C, ldc, err);
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  assemble_kernel<<<dim3((n + 127) / 128, n), 128, 0, ctx->stream>>>(C, n, ldc, tcc);
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  return LITHO_OK;
}

}  // namespace litho
