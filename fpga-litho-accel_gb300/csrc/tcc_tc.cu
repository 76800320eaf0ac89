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
// gemm_bf16x3_kernel  persistent, one CTA per SM over the 128 x BN output tiles
//                   the TCC reads (BN = 64, 128 or 256), K streamed in 64-wide
//                   (128-byte) or 32-wide (64-byte swizzle) slices through a
//                   TMA/mbarrier ring; whole tiles in data-parallel rounds and,
//                   optionally, the last one or two rounds' tiles split along K
//                   over all CTAs (gemm_schedule); a double-buffered TMEM
//                   accumulator lets the epilogue warps drain one piece while the
//                   next one's MMAs run.  gemm_fixup_kernel adds the partial sums
//                   of split tiles in K order.  BN and the schedule are chosen per
//                   (n, Kp) by timing every candidate on the device (gemm_tune).
// assemble_kernel   C -> interleaved complex128 TCC: upper triangle from C, the
//                   lower triangle its conjugate mirror (litho.cpp:510-515).
#include "litho_internal.cuh"
#include "tc_common.cuh"
#include "tcc_tiles.hpp"

#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
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

// Persistent split-BF16 GEMM C = A B^T over a list of 128 x BN output tiles.  One CTA
// per SM runs the pieces (GemmSeg: a tile and a range of its 64-wide K slices) the
// host schedule gives it.  Roles (192 threads):
//   warp 0 lane 0 : TMA producer, streams [Ah | Al | Bh | Bl] K slices through an
//                   NS-stage ring (full[s] / empty[s])
//   warp 1 lane 0 : MMA issuer, hi*hi + hi*lo + lo*hi per 16-wide K step into one
//                   of two TMEM accumulators (accfull / accempty), so a piece's
//                   epilogue overlaps the next piece's main loop
//   warps 2-5     : epilogue, one TMEM lane quarter per warp (warp % 4): 32 columns
//                   per tcgen05.ld, 16-byte stores to C (whole tiles) or to the
//                   piece's partial slot (split tiles, added by gemm_fixup_kernel)
// Every wait is bounded; a role whose wait gives up sets the abort flag and the
// others' waits then return at once, the producer's issued loads are waited for,
// TMEM is freed and the error flag is raised.
template <int BN, int BK>
struct GemmCfg {
  static_assert(BK == 64 || BK == 32, "K slices of 64 (128-byte swizzle) or 32 (64-byte swizzle) bf16");
  static constexpr uint32_t A_T = 128 * BK * 2;       // 128 rows x BK bf16
  static constexpr uint32_t B_T = BN * BK * 2;        // BN rows x BK bf16
  static constexpr uint32_t STAGE = 2 * A_T + 2 * B_T;  // Ah, Al, Bh, Bl
  static constexpr int NS0 = (int)((192u * 1024u) / STAGE);
  static constexpr int NS = NS0 > 8 ? 8 : NS0;         // BK = 64: 4, 3, 2 at BN = 64, 128, 256; BK = 32: 6, 4 at 128, 256
  static constexpr size_t SMEM = 1024 + (size_t)NS * STAGE + 512;
  static constexpr uint32_t TCOLS = 2 * BN;           // two accumulators
};
constexpr int GB_THREADS = 192;

template <int BN, int BK>
__global__ void __launch_bounds__(GB_THREADS, 1) gemm_bf16x3_kernel(const __grid_constant__ CUtensorMap tAh,
                                                                    const __grid_constant__ CUtensorMap tAl,
                                                                    const __grid_constant__ CUtensorMap tBh,
                                                                    const __grid_constant__ CUtensorMap tBl,
                                                                    const int4* __restrict__ segs,
                                                                    const int* __restrict__ seg_begin,
                                                                    const int2* __restrict__ tiles, int M, int N,
                                                                    float* __restrict__ C, int ldc,
                                                                    float* __restrict__ part,
                                                                    int* __restrict__ err) {
  using P = GemmCfg<BN, BK>;
  constexpr int NS = P::NS;
  extern __shared__ unsigned char smraw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + (size_t)NS * P::STAGE);
  uint64_t* empty = full + NS;
  uint64_t* accfull = empty + NS;   // [2]
  uint64_t* accempty = accfull + 2;  // [2]
  uint64_t* done = accempty + 2;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort = reinterpret_cast<volatile int*>(tslot + 1);
  int* last_issued = reinterpret_cast<int*>(tslot + 2);  // [NS]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int sb = seg_begin[blockIdx.x], se = seg_begin[blockIdx.x + 1];

  if (warp == 0) tmem_alloc(tslot, P::TCOLS);
  if (tid == 0) {
    for (int s = 0; s < NS; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
      last_issued[s] = -1;
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accfull[b], 1);
      mbar_init(&accempty[b], 4);  // one arrival per epilogue warp
    }
    mbar_init(done, 1);
    *abort = 0;
    fence_mbar_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  auto tile = [&](int s, int q) {  // q: 0 Ah, 1 Al, 2 Bh, 3 Bl
    return sm + (size_t)s * P::STAGE + (q < 2 ? (size_t)q * P::A_T : 2 * (size_t)P::A_T + (size_t)(q - 2) * P::B_T);
  };

  if (warp == 0) {
    if (lane == 0) {  // TMA producer
      int q = 0, s = 0;
      uint32_t ph = 0;
      bool ok = true;
      for (int i = sb; i < se && ok; ++i) {
        const int4 g = segs[i];
        const int2 t = tiles[g.x];
        const int m0 = 128 * t.x, n0 = BN * t.y;
        for (int k = g.y; k < g.z; ++k, ++q) {
          if (q >= NS && !mbar_wait_ab(&empty[s], ph ^ 1u, abort)) {
            *abort = 1;
            ok = false;
            break;
          }
          mbar_arrive_expect_tx(&full[s], P::STAGE);
          tma_load_2d(tile(s, 0), &tAh, &full[s], BK * k, m0);
          tma_load_2d(tile(s, 1), &tAl, &full[s], BK * k, m0);
          tma_load_2d(tile(s, 2), &tBh, &full[s], BK * k, n0);
          tma_load_2d(tile(s, 3), &tBl, &full[s], BK * k, n0);
          last_issued[s] = q;
          if (++s == NS) {
            s = 0;
            ph ^= 1u;
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
      constexpr uint32_t IDESC = idesc_bf16(128, BN);
      int s = 0, tl = 0;
      uint32_t ph = 0;
      bool ok = true;
      for (int i = sb; i < se && ok; ++i, ++tl) {
        const int4 g = segs[i];
        const int buf = tl & 1;
        if (tl >= 2 && !mbar_wait_ab(&accempty[buf], (uint32_t)((tl - 2) >> 1) & 1u, abort)) {
          *abort = 1;
          break;
        }
        tc_fence_after();
        const uint32_t acc = tmem + (uint32_t)(buf * BN);
        for (int k = g.y; k < g.z; ++k) {
          if (!mbar_wait_ab(&full[s], ph, abort)) {
            *abort = 1;
            ok = false;
            break;
          }
          tc_fence_after();
          auto desc = [](const void* t) { return BK == 64 ? desc_sw128(t) : desc_sw64(t); };
          const uint64_t dah = desc(tile(s, 0)), dal = desc(tile(s, 1));
          const uint64_t dbh = desc(tile(s, 2)), dbl = desc(tile(s, 3));
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk) {
            const uint32_t off = kk * 32;  // 16 bf16 per MMA
            mma_bf16(acc, desc_add(dah, off), desc_add(dbh, off), IDESC, (k != g.y || kk != 0) ? 1u : 0u);
            mma_bf16(acc, desc_add(dah, off), desc_add(dbl, off), IDESC, 1u);
            mma_bf16(acc, desc_add(dal, off), desc_add(dbh, off), IDESC, 1u);
          }
          mma_commit(&empty[s]);
          if (++s == NS) {
            s = 0;
            ph ^= 1u;
          }
        }
        if (ok) mma_commit(&accfull[buf]);  // arrives when this piece's MMAs have completed
      }
      mma_commit(done);  // arrives once everything issued above has completed
      // bounded, and it starts after the last MMA was issued; the other threads meet
      // this lane at the block barrier below instead of timing the whole kernel
      if (!mbar_wait(done, 0)) *abort = 1;
    }
  } else {  // warps 2-5: epilogue
    const int quarter = warp & 3;
    const int r = 32 * quarter + lane;  // this thread's row of the tile (its TMEM lane)
    int tl = 0;
    for (int i = sb; i < se; ++i, ++tl) {
      const int4 g = segs[i];
      const int2 t = tiles[g.x];
      const int buf = tl & 1;
      // on a wait that gives up: flag it and carry on (later waits return at once)
      if (!mbar_wait_ab(&accfull[buf], (uint32_t)(tl >> 1) & 1u, abort)) *abort = 1;
      tc_fence_after();
      const uint32_t trow = tmem + (uint32_t)(buf * BN) + ((uint32_t)(32 * quarter) << 16);
      const int row = 128 * t.x + r, n0 = BN * t.y;
#pragma unroll 1
      for (int slab = 0; slab < BN / 32; ++slab) {
        float v[32];
        tmem_ld32(trow + (uint32_t)(slab * 32), v);
        const int c0 = slab * 32;
        if (g.w >= 0) {  // partial slot: the whole 128 x BN tile, row-major
          float* out = part + ((size_t)g.w * 128 + r) * BN + c0;
#pragma unroll
          for (int j = 0; j < 32; j += 4)
            *reinterpret_cast<float4*>(out + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
        } else if (row < M && n0 + c0 < N) {
          float* out = C + (size_t)row * ldc + n0 + c0;
          if (n0 + c0 + 32 <= ldc) {
#pragma unroll
            for (int j = 0; j < 32; j += 4)
              *reinterpret_cast<float4*>(out + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (n0 + c0 + j < N) out[j] = v[j];
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&accempty[buf]);  // the MMA lane may refill this accumulator
    }
  }
  __syncthreads();  // the MMA lane has seen `done`: the tensor cores have drained
  if (*abort) {
    if (tid == 0) {  // the producer lane: wait for the last load of every stage
      for (int s = 0; s < NS; ++s)
        if (last_issued[s] >= 0) mbar_wait(&full[s], (uint32_t)(last_issued[s] / NS) & 1u, 200u);
      atomicExch(err, 1);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, P::TCOLS);
}

// Split tiles: C tile = the sum of its partial slots in K order (fixed order, so the
// result is reproducible).  One CTA per (split tile, 1024 elements), four per thread.
__global__ void gemm_fixup_kernel(const float* __restrict__ part, const int* __restrict__ fix_tile,
                                  const int* __restrict__ fix_begin, const int* __restrict__ fix_slot,
                                  const int2* __restrict__ tiles, int BN, int M, int N, float* __restrict__ C,
                                  int ldc) {
  const int f = blockIdx.x;
  const int e = 4 * (blockIdx.y * blockDim.x + threadIdx.x);
  if (e >= 128 * BN) return;
  const int r = e / BN, c = e - r * BN;
  const int2 t = tiles[fix_tile[f]];
  const int row = 128 * t.x + r, col = BN * t.y + c;
  if (row >= M || col >= N) return;
  float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int j = fix_begin[f]; j < fix_begin[f + 1]; ++j) {
    const float4 v = *reinterpret_cast<const float4*>(part + (size_t)fix_slot[j] * 128 * BN + e);
    a.x += v.x;
    a.y += v.y;
    a.z += v.z;
    a.w += v.w;
  }
  float* out = C + (size_t)row * ldc + col;
  if (col + 4 <= ldc) {
    *reinterpret_cast<float4*>(out) = a;
  } else {
    const float w[4] = {a.x, a.y, a.z, a.w};
    for (int j = 0; j < 4 && col + j < N; ++j) out[j] = w[j];
  }
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

static int map_bf16(litho_ctx* ctx, CUtensorMap* m, const void* base, uint64_t cols, uint64_t rows,
                    uint32_t box_rows, int bk) {
  auto fn = encode_fn_bf16();
  if (fn == nullptr) {
    set_error(ctx, LITHO_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    return LITHO_ERR_CUDA;
  }
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {cols * 2};
  cuuint32_t box[2] = {(cuuint32_t)bk, box_rows};
  cuuint32_t es[2] = {1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, bk == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error(ctx, LITHO_ERR_CUDA, "cuTensorMapEncodeTiled (bf16) failed (%d)", (int)r);
    return LITHO_ERR_CUDA;
  }
  return LITHO_OK;
}

int tc_err_flag_public(litho_ctx* ctx, int** flag);

// Device copy of one GEMM schedule: the tile list, the CTAs' pieces and the fix-up
// lists, plus the partial-slot workspace, cached per (n, K slices, BN, schedule).
struct GemmTables {
  ~GemmTables() {
    buf.release();
    part.release();
  }
  DevBuf buf, part;
  int ctas = 0, ntiles = 0, nfix = 0, nslots = 0;
  int2* tiles = nullptr;
  int4* segs = nullptr;
  int* seg_begin = nullptr;
  int *fix_tile = nullptr, *fix_begin = nullptr, *fix_slot = nullptr;
};

static int gemm_tables(litho_ctx* ctx, int n, int nk, int bn, int sched, GemmTables** out) {
  const auto key = std::make_tuple(n, nk, bn, sched);
  auto it = ctx->gemm_tables.find(key);
  if (it != ctx->gemm_tables.end()) {
    *out = static_cast<GemmTables*>(it->second.get());
    return LITHO_OK;
  }
  const std::vector<TileMN> need = tcc_needed_tiles(n, bn);
  const int T = (int)need.size();
  const int ctas = sched != GEMM_WHOLE_TILES ? ctx->sm_count : std::min(ctx->sm_count, T);
  const GemmSchedule sc = gemm_schedule(T, nk, ctas, sched);
  // one host image of all tables, uploaded once
  std::vector<int> h;
  auto put = [&](size_t n_ints) {
    const size_t off = h.size();
    h.resize(off + ((n_ints + 3) & ~size_t(3)), 0);  // 16-byte aligned sub-arrays
    return off;
  };
  const size_t o_tiles = put(2 * (size_t)T), o_segs = put(4 * sc.segs.size()), o_beg = put(sc.begin.size()),
               o_ft = put(sc.fix_tile.size()), o_fb = put(sc.fix_begin.size()), o_fs = put(sc.fix_slot.size());
  for (int i = 0; i < T; ++i) {
    h[o_tiles + 2 * i] = need[i].m;
    h[o_tiles + 2 * i + 1] = need[i].n;
  }
  for (size_t i = 0; i < sc.segs.size(); ++i) {
    h[o_segs + 4 * i] = sc.segs[i].tile;
    h[o_segs + 4 * i + 1] = sc.segs[i].k0;
    h[o_segs + 4 * i + 2] = sc.segs[i].k1;
    h[o_segs + 4 * i + 3] = sc.segs[i].slot;
  }
  std::copy(sc.begin.begin(), sc.begin.end(), h.begin() + o_beg);
  std::copy(sc.fix_tile.begin(), sc.fix_tile.end(), h.begin() + o_ft);
  std::copy(sc.fix_begin.begin(), sc.fix_begin.end(), h.begin() + o_fb);
  std::copy(sc.fix_slot.begin(), sc.fix_slot.end(), h.begin() + o_fs);
  auto t = std::make_shared<GemmTables>();
  LITHO_RET(t->buf.ensure(ctx, h.size() * sizeof(int) + 16));
  LITHO_CUDA_TRY(ctx, cudaMemcpy(t->buf.p, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice));
  int* d = t->buf.as<int>();
  t->tiles = reinterpret_cast<int2*>(d + o_tiles);
  t->segs = reinterpret_cast<int4*>(d + o_segs);
  t->seg_begin = d + o_beg;
  t->fix_tile = d + o_ft;
  t->fix_begin = d + o_fb;
  t->fix_slot = d + o_fs;
  t->ctas = ctas;
  t->ntiles = T;
  t->nfix = (int)sc.fix_tile.size();
  t->nslots = sc.nslots;
  if (sc.nslots > 0) LITHO_RET(t->part.ensure(ctx, (size_t)sc.nslots * 128 * bn * sizeof(float)));
  ctx->gemm_tables[key] = t;
  *out = t.get();
  return LITHO_OK;
}

// One persistent GEMM of the given shape and schedule (plus the fix-up of split tiles).
template <int BN, int BK>
static int run_gemm(litho_ctx* ctx, const __nv_bfloat16* Ah, const __nv_bfloat16* Al, int n, int Kp, float* C,
                    int ldc, int sched, int* err) {
  using P = GemmCfg<BN, BK>;
  GemmTables* t = nullptr;
  LITHO_RET(gemm_tables(ctx, n, Kp / BK, BN, sched, &t));
  CUtensorMap mAh, mAl, mBh, mBl;
  LITHO_RET(map_bf16(ctx, &mAh, Ah, Kp, 2 * n, 128, BK));
  LITHO_RET(map_bf16(ctx, &mAl, Al, Kp, 2 * n, 128, BK));
  LITHO_RET(map_bf16(ctx, &mBh, Ah, Kp, n, BN, BK));  // B = A's first n rows
  LITHO_RET(map_bf16(ctx, &mBl, Al, Kp, n, BN, BK));
  static_assert(P::SMEM <= 227 * 1024, "GEMM stages exceed the shared memory of one CTA");
  LITHO_CUDA_TRY(ctx, cudaFuncSetAttribute(gemm_bf16x3_kernel<BN, BK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)P::SMEM));
  gemm_bf16x3_kernel<BN, BK><<<t->ctas, GB_THREADS, P::SMEM, ctx->stream>>>(
      mAh, mAl, mBh, mBl, t->segs, t->seg_begin, t->tiles, 2 * n, n, C, ldc, t->part.as<float>(), err);
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  if (t->nfix > 0) {
    gemm_fixup_kernel<<<dim3(t->nfix, (128 * BN / 4 + 255) / 256), 256, 0, ctx->stream>>>(
        t->part.as<float>(), t->fix_tile, t->fix_begin, t->fix_slot, t->tiles, BN, 2 * n, n, C, ldc);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
  }
  return LITHO_OK;
}

// the GEMM shapes the tuner chooses from: (column tile width, K slice)
static const int kGemmShapes[][2] = {{64, 64}, {128, 64}, {256, 64}, {128, 32}, {256, 32}};

static int run_gemm_shape(litho_ctx* ctx, int bn, int bk, int sched, const __nv_bfloat16* Ah,
                          const __nv_bfloat16* Al, int n, int Kp, float* C, int ldc, int* err) {
  if (bk == 32) {
    if (bn == 128) return run_gemm<128, 32>(ctx, Ah, Al, n, Kp, C, ldc, sched, err);
    return run_gemm<256, 32>(ctx, Ah, Al, n, Kp, C, ldc, sched, err);
  }
  switch (bn) {
    case 64: return run_gemm<64, 64>(ctx, Ah, Al, n, Kp, C, ldc, sched, err);
    case 128: return run_gemm<128, 64>(ctx, Ah, Al, n, Kp, C, ldc, sched, err);
    default: return run_gemm<256, 64>(ctx, Ah, Al, n, Kp, C, ldc, sched, err);
  }
}

// The GEMM's column tile width, K slice and schedule, chosen on the device the first
// time a (n, Kp) is seen: every candidate is run once to warm up and then timed twice
// with CUDA events on the context's stream; the fastest is cached with the timings.
static int gemm_tune(litho_ctx* ctx, const __nv_bfloat16* Ah, const __nv_bfloat16* Al, int n, int Kp, float* C,
                     int ldc, int* err, TccTune** out) {
  const auto key = std::make_pair(n, Kp);
  auto it = ctx->tcc_tune.find(key);
  if (it != ctx->tcc_tune.end()) {
    *out = &it->second;
    return LITHO_OK;
  }
  TccTune tu;
  cudaEvent_t a = nullptr, b = nullptr;
  LITHO_CUDA_TRY(ctx, cudaEventCreate(&a));
  LITHO_CUDA_TRY(ctx, cudaEventCreate(&b));
  int rc = LITHO_OK;
  float best = 0.f;
  for (const auto& sh : kGemmShapes) {
    const int bn = sh[0], bk = sh[1];
    for (int sched = 0; sched < 3 && rc == LITHO_OK; ++sched) {
      rc = run_gemm_shape(ctx, bn, bk, sched, Ah, Al, n, Kp, C, ldc, err);
      if (rc == LITHO_OK && cudaEventRecord(a, ctx->stream) != cudaSuccess) rc = LITHO_ERR_CUDA;
      for (int r = 0; r < 2 && rc == LITHO_OK; ++r) rc = run_gemm_shape(ctx, bn, bk, sched, Ah, Al, n, Kp, C, ldc, err);
      float ms = 0.f;
      if (rc == LITHO_OK && (cudaEventRecord(b, ctx->stream) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess ||
                             cudaEventElapsedTime(&ms, a, b) != cudaSuccess))
        rc = LITHO_ERR_CUDA;
      if (rc != LITHO_OK) break;
      ms *= 0.5f;
      tu.cands.push_back({bn, bk, sched, ms});
      if (tu.cands.size() == 1 || ms < best) {
        best = ms;
        tu.bn = bn;
        tu.bk = bk;
        tu.sched = sched;
      }
    }
    if (rc != LITHO_OK) break;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc == LITHO_ERR_CUDA) set_error(ctx, LITHO_ERR_CUDA, "timing the TCC GEMM candidates failed");
  if (rc != LITHO_OK) return rc;
  *out = &(ctx->tcc_tune[key] = tu);
  return LITHO_OK;
}

// any non-finite entry of n doubles sets *flag (NA > n_medium makes the pupil phase NaN):
// 16-byte loads, four in flight per thread
__global__ void nonfinite_kernel(const double2* __restrict__ x, size_t n2, const double* __restrict__ tail,
                                 int ntail, int* __restrict__ flag) {
  bool bad = false;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n2; i += 4 * stride) {
    double2 v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) v[u] = __ldcs(x + i + u * stride);
#pragma unroll
    for (int u = 0; u < 4; ++u) bad |= !isfinite(v[u].x) || !isfinite(v[u].y);
  }
  for (; i < n2; i += stride) {
    const double2 v = __ldcs(x + i);
    bad |= !isfinite(v.x) || !isfinite(v.y);
  }
  if (blockIdx.x == 0 && (int)threadIdx.x < ntail) bad |= !isfinite(tail[threadIdx.x]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicExch(flag, 1);
}

cudaError_t launch_nonfinite(cudaStream_t s, const double* x, size_t n, int* flag, int sms) {
  // complex128 data is 16-byte aligned; an odd count leaves one double for the tail
  nonfinite_kernel<<<8 * sms, 256, 0, s>>>(reinterpret_cast<const double2*>(x), n / 2, x + (n & ~size_t(1)),
                                           (int)(n & 1), flag);
  return cudaGetLastError();
}

int tcc_split_bf16(litho_ctx* ctx, const float2* P, const float* J, int n, int ns, int ldp, double2* tcc) {
  const int Kp = ((2 * ns + 63) / 64) * 64;
  const size_t op = (size_t)Kp * sizeof(__nv_bfloat16);
  const int ldc = (n + 3) & ~3;  // 16-byte rows for the epilogue's vector stores
  // A: 2n rows (hi, lo); B is A's first n rows; C: 2n x ldc fp32
  const size_t cbytes = (size_t)2 * n * ldc * sizeof(float);
  LITHO_RET(ctx->mx_c.ensure(ctx, op * 4 * (size_t)n + cbytes + 4096));
  char* base = ctx->mx_c.as<char>();
  auto take = [&](size_t b) {
    char* p = base;
    base += (b + 1023) & ~size_t(1023);
    return p;
  };
  __nv_bfloat16* Ah = reinterpret_cast<__nv_bfloat16*>(take(op * 2 * n));
  __nv_bfloat16* Al = reinterpret_cast<__nv_bfloat16*>(take(op * 2 * n));
  float* C = reinterpret_cast<float*>(take(cbytes));
  split_kernel<<<dim3((Kp / 8 + 127) / 128, n), 128, 0, ctx->stream>>>(P, J, n, ns, ldp, Kp, Ah, Al);
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  int* err = nullptr;
  LITHO_RET(tc_err_flag_public(ctx, &err));
  if (ctx->tcc_force_bn > 0) {
    LITHO_RET(run_gemm_shape(ctx, ctx->tcc_force_bn, ctx->tcc_force_bk, ctx->tcc_force_sched, Ah, Al, n, Kp, C, ldc,
                             err));
  } else {
    TccTune* tu = nullptr;
    LITHO_RET(gemm_tune(ctx, Ah, Al, n, Kp, C, ldc, err, &tu));
    LITHO_RET(run_gemm_shape(ctx, tu->bn, tu->bk, tu->sched, Ah, Al, n, Kp, C, ldc, err));
  }
  assemble_kernel<<<dim3((n + 127) / 128, n), 128, 0, ctx->stream>>>(C, n, ldc, tcc);
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  return LITHO_OK;
}

}  // namespace litho

using namespace litho;

extern "C" int litho_tcc_gemm_shape(litho_ctx* ctx, int bn, int bk, int sched) {
  if (ctx == nullptr) return LITHO_ERR_ARG;
  bool ok = bn == 0;
  for (const auto& sh : kGemmShapes) ok = ok || (sh[0] == bn && sh[1] == bk);
  LITHO_ARG_CHECK(ctx, ok, "no GEMM shape with %d-column tiles and %d-wide K slices", bn, bk);
  LITHO_ARG_CHECK(ctx, sched >= 0 && sched <= 2, "schedule %d not in {0, 1, 2}", sched);
  ctx->tcc_force_bn = bn;
  ctx->tcc_force_bk = bk;
  ctx->tcc_force_sched = sched;
  return LITHO_OK;
}

extern "C" int litho_tcc_gemm_describe(const litho_ctx* ctx, char* buf, int cap) {
  if (ctx == nullptr || buf == nullptr || cap <= 0) return 0;
  std::string o = "[";
  bool first = true;
  char t[160];
  for (const auto& kv : ctx->tcc_tune) {
    snprintf(t, sizeof t,
             "%s{\"n\": %d, \"Kp\": %d, \"bn\": %d, \"bk\": %d, \"sched\": %d, \"candidates\": [",
             first ? "" : ", ", kv.first.first, kv.first.second, kv.second.bn, kv.second.bk, kv.second.sched);
    o += t;
    first = false;
    for (size_t i = 0; i < kv.second.cands.size(); ++i) {
      const auto& c = kv.second.cands[i];
      snprintf(t, sizeof t, "%s{\"bn\": %d, \"bk\": %d, \"sched\": %d, \"ms\": %.4f}", i ? ", " : "", c.bn,
               c.bk, c.sched, c.ms);
      o += t;
    }
    o += "]}";
  }
  o += "]";
  const int n = (int)std::min<size_t>(o.size(), (size_t)cap - 1);
  memcpy(buf, o.data(), n);
  buf[n] = 0;
  return n;
}
