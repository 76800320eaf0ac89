// Mixed-precision imaging: the two dense DFT contractions of the pipeline on the
// 5th-generation tensor cores (tcgen05, kind::tf32) with split operands and
// FP32 accumulation in TMEM.  The FFTs and the intensity sum (socs_kernel) stay
// FP32 on the CUDA cores.
//
// Split products.  Every operand X is written as X = Xh + Xl with
// Xh = round_tf32(X) and Xl = X - Xh (exact in FP32); each contraction computes
// Ah*Bh + Ah*Bl + Al*Bh.  The hi and lo tiles of B sit back to back in shared
// memory, so Ah*[Bh; Bl] is ONE MMA of twice the width (the mask or Cy tile is
// read once for both products) and the epilogue adds the two column halves.  The
// dropped Al*Bl term and the TF32 rounding of Xl leave a relative error of about
// 2^-22 per product.
//
// Both kernels are persistent (one CTA per SM), warp-specialised and synchronised
// only by mbarriers, so TMA traffic, tensor-core work and CUDA-core work overlap.
//
// win_dft_tc_kernel   D[y][j] = sum_x mask[y][x] * T[x][j]  (M = 128 mask rows
//                     per tile, N = 2 NB (hi | lo) for the 2Nx+1 column twiddles
//                     padded to NB, K = the tile's columns).  448 threads: TMA
//                     streams 128 x 32 mask tiles (SWIZZLE_128B), two per
//                     stage, through a ring of as many stages as shared memory
//                     holds (4 at Nx = 8); warps 0-7 check each landed tile for TF32
//                     exactness (no low 13 mantissa bit set) and split it in
//                     place only when it has a residual; the accumulator is
//                     double-buffered in TMEM and warps 10-13 run each tile's
//                     row-DFT epilogue while the next tile streams.
// fi_tc_kernel        image[Y][X] = T0[X] + sum_r Cy[Y][r] * Tm[r][X]  (M = 128
//                     image rows, N = 2 BN per tile, K = 4Ny rows padded to
//                     32*KBLK; the DC row T0 is added in FP32 by the epilogue).
//                     320 threads over output tiles ordered (row band, image,
//                     column tile): Cy is reloaded only when a CTA's range crosses
//                     a row band, Tm tiles stream through a TMA ring, and two
//                     epilogue groups drain the double-buffered accumulator
//                     through swizzled staging tiles with TMA bulk stores (the
//                     image is written exactly once).
#include "litho_internal.cuh"
#include "tc_common.cuh"
#include "win_tiles.hpp"

#include <cstring>

#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>

namespace litho {
using namespace tc;

// ---------------------------------------------------------------------------
// operand tables (built once per geometry, cached on the context)
// ---------------------------------------------------------------------------
// twT[j][x] (NB rows): j <= Nx cos(2 pi j x'/Fx); Nx < j <= 2Nx -sin(2 pi (j-Nx) x'/Fx); else 0
__global__ void twT_init_kernel(float* __restrict__ hi, float* __restrict__ lo, int Lx, int Fx, int Nx, int NB) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (x >= Lx || j >= NB) return;
  const long long xp = (long long)x + (Fx - Lx) / 2 - Fx / 2;
  double v = 0.0;
  if (j <= 2 * Nx) {
    const int u = j <= Nx ? j : j - Nx;
    long long m = ((long long)u * xp) % Fx;
    if (m < 0) m += Fx;
    double s, c;
    sincospi(2.0 * (double)m / (double)Fx, &s, &c);
    v = j <= Nx ? c : -s;
  }
  const float h = tf32_round((float)v);
  hi[(size_t)j * Lx + x] = h;
  lo[(size_t)j * Lx + x] = (float)(v - (double)h);
}

// ytab[v][y] = e^{-2 pi i v y'/Fy} (v = 0..Ny), y' = y + (Fy - Ly)/2 - Fy/2: the row
// twiddles of the window DFT's epilogue
// yt[v][y] = e^{-2 pi i v y' / Fy} for the rows y < Ly, rows padded to Lyp (a multiple
// of 128) with zeros, so that a 128-row tile reads whole rows of it.
__global__ void ytab_init_kernel(float2* __restrict__ yt, int Ly, int Lyp, int Fy) {
  const int y = blockIdx.x * blockDim.x + threadIdx.x;
  const int v = blockIdx.y;
  if (y >= Lyp) return;
  float2 t = make_float2(0.f, 0.f);
  if (y < Ly) {
    const long long oyc = (long long)(Fy - Ly) / 2 - Fy / 2;
    long long m = ((long long)v * (y + oyc)) % Fy;
    if (m < 0) m += Fy;
    float sn, cs;
    sincospif(2.0f * (float)m / (float)Fy, &sn, &cs);
    t = make_float2(cs, -sn);
  }
  yt[(size_t)v * Lyp + y] = t;
}

// CyT[Y][r] (KP columns): r < 2Ny -> 2cos(2 pi (r+1) y'/Fy); 2Ny <= r < 4Ny ->
// -2sin(2 pi (r-2Ny+1) y'/Fy); else 0.  The fy = 0 (DC) row is not a column: the
// FI epilogue adds T0[X] in FP32, so 4Ny rows fill the K blocks exactly when Ny is
// a multiple of 8.
__global__ void cyT_init_kernel(float* __restrict__ hi, float* __restrict__ lo, int Ly, int Fy, int Ny, int KP) {
  const int Y = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (Y >= Ly || r >= KP) return;
  const long long yp = (long long)Y + (Fy - Ly) / 2 - Fy / 2;
  double v = 0.0;
  if (r < 4 * Ny) {
    const int dy = r < 2 * Ny ? r + 1 : r - 2 * Ny + 1;
    long long m = ((long long)dy * yp) % Fy;
    if (m < 0) m += Fy;
    double s, c;
    sincospi(2.0 * (double)m / (double)Fy, &s, &c);
    v = r < 2 * Ny ? 2.0 * c : -2.0 * s;
  }
  const float h = tf32_round((float)v);
  hi[(size_t)Y * KP + r] = h;
  lo[(size_t)Y * KP + r] = (float)(v - (double)h);
}

// ---------------------------------------------------------------------------
// window DFT on the tensor cores
// ---------------------------------------------------------------------------

// Persistent window DFT: one CTA per SM streams its tiles (image, 128-row block,
// column range) through one TMA ring; the TMEM accumulator is double-buffered so
// a tile's row-DFT epilogue (its own four warps) overlaps the next tile's loads
// and MMAs.  Roles (448 threads):
//   warps 0-7   check each landed mask tile for TF32-exactness (warp vote); only
//               a tile with a residual is split in place (hi, then lo)
//   warp 8      TMA producer (one lane), warp 9 MMA issuer (one lane)
//   warps 10-13 epilogue: TMEM -> registers -> shared -> row DFT -> partials
// Per stage s and running chunk q (parity (q / S) & 1; every role keeps s and the
// parity as running counters, since a division by the launch-time S on the
// per-chunk path measurably slows the ring):
//   producer  : [wait empty[s]] -> TMA mask tile + twiddle [hi; lo] tile -> full[s]
//   consumers : wait full[s]; vote residual (nzflag); if any: Ah = round_tf32(A) in
//               place; arrive ready[s]; if residual: wait hidone[s], write Al,
//               arrive ready2[s]
//   MMA lane  : [tile start: wait accempty[buf]]; wait ready[s]; Ah*[Bh; Bl] as one
//               N = 2 NBH MMA per K step (the epilogue adds the two column halves);
//               if residual: commit hidone[s], wait ready2[s], Al*Bh; commit empty[s];
//               [tile end: commit accfull[buf]]
//   epilogue  : wait accfull[buf]; TMEM -> sR (hi + lo halves); arrive accempty[buf];
//               row DFT with one thread per output pair (+v, -v)
// hidone/ready2 complete only on chunks with a residual, so their parities are
// tracked per stage in bit masks that both sides flip identically.
//
// The ring is as deep as shared memory allows: under full load a mask tile takes
// ~3 us from TMA issue to landing, so the bytes in flight per SM, not the work per
// tile, set the throughput.  Hence the twiddle tile carries only the 2Nx+1 used
// rows of each half (NBH = 2Nx+1 rounded up to 8), the epilogue keeps only the 2Nx+1
// used accumulator columns in shared memory and reads the row twiddles from their
// table (through L1), and the stage count S is chosen at launch: four stages (128 KB of
// mask in flight) up to Nx = 16.
template <int NBH>
struct WinTC {
  // a stage carries a 64-column chunk as two 32-column K blocks: each pipeline round
  // trip (land, check, MMA, release) then moves 32 KB of mask, which halves the
  // per-chunk handshakes that bound this ring
  static constexpr int KB = 2;                       // K blocks (32 columns each) per stage
  static constexpr uint32_t A_KB = 128 * 128;        // 128 rows x 32 fp32 (split in place: hi, then lo)
  static constexpr uint32_t A_B = KB * A_KB;
  static constexpr uint32_t B_KB = 2 * NBH * 128;    // [hi NBH rows; lo NBH rows] x 32 fp32
  static constexpr uint32_t B_B = KB * B_KB;
  static constexpr uint32_t STAGE_B = A_B + B_B;     // a multiple of 2048: every stage is 1024-aligned
  // one accumulator holds A*Bh in columns [0, NBH) and A*Bl in [NBH, 2 NBH): one
  // N = 2 NBH MMA reads the mask tile once for both products
  static constexpr uint32_t NCOL = 2 * NBH <= 32 ? 32 : (2 * NBH <= 64 ? 64 : 128);
  static constexpr int NLO = (NBH + 15) / 16 * 16;  // N of the residual pass Al*Bh (>= NBH, multiple of 16)
};
constexpr int WP_THREADS = 448;  // warps 0-7 split, 8 TMA, 9 MMA, 10-13 epilogue
constexpr int WP_CONS = 256;     // consumer threads
// padded row strides of the epilogue buffers: multiples of 4 floats so the row DFT
// reads 16-byte vectors, and 33 / 65 float4 slots apart so the threads of a warp
// (different u, different |v|) land in different bank groups
constexpr int WP_RSR = 132;      // sR rows (fp32)
constexpr int WP_MAX_STAGES = 12;
constexpr int WP_TQ = 8;         // tile ring: tiles the producer may publish ahead of the slowest role
constexpr size_t WP_SMEM_CAP = 227 * 1024;

// epilogue buffer: sR [2Nx+1][RSR] fp32 (a multiple of 16 bytes)
static inline size_t win_epi_bytes(int Nx) { return (size_t)(2 * Nx + 1) * WP_RSR * 4; }
// The mask geometries of one window-DFT launch (the mask sizes of a batch class share the
// period, the kernels and the partial array): per geometry its masks' and twiddles' tensor
// maps, its row twiddles, width, row blocks, column splits and first image in the partial
// array.  Tiles are numbered geometry after geometry (tile0: the prefix).
constexpr int WP_MAX_GEO = WIN_MAX_SIZES;
struct WinGeo {
  CUtensorMap mM[WP_MAX_GEO];  // masks [img][Ly][Lx]
  CUtensorMap mB[WP_MAX_GEO];  // twiddles [hi; lo] x Lx
  const float2* ytab[WP_MAX_GEO];
  WinTiles T;                  // widths, row blocks, splits, first images and tiles (win_tiles.hpp)
};

// mbarriers and flags after the epilogue buffers (S <= WP_MAX_STAGES): 5 per stage, 5 more,
// two per tile-ring slot; the TMEM slot, abort flag, per-stage ints, tile ring and the two
// groups' current tiles
static inline size_t win_bar_bytes(int S) {
  return (size_t)(5 * S + 5 + 2 * WP_TQ) * 8 + 16 + 8 * (size_t)S + 4 * WP_TQ + 8;
}

template <int NBH>
__global__ void __launch_bounds__(WP_THREADS, 1) win_dft_tc_kernel(const __grid_constant__ WinGeo G, int Fx, int Fy,
                                                                   int Nx, int Ny, int S,
                                                                   float2* __restrict__ win_part, int part_stride,
                                                                   int* __restrict__ err, int stall_at) {
  using P = WinTC<NBH>;
  extern __shared__ unsigned char smraw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  constexpr int RS = WP_RSR;
  const int KXw = 2 * Nx + 1;                                          // used accumulator columns
  float* sR = reinterpret_cast<float*>(sm + (size_t)S * P::STAGE_B);  // [KXw][RS]
  uint64_t* full = reinterpret_cast<uint64_t*>(sR + KXw * RS);
  uint64_t* ready = full + S;
  uint64_t* hidone = ready + S;
  uint64_t* ready2 = hidone + S;
  uint64_t* empty = ready2 + S;
  uint64_t* accfull = empty + S;
  uint64_t* accempty = accfull + 2;
  uint64_t* done = accempty + 2;
  uint64_t* tqf = done + 1;       // [WP_TQ] tile-ring slot published (producer)
  uint64_t* tqe = tqf + WP_TQ;    // [WP_TQ] slot read by all three reading roles
  uint32_t* tslot = reinterpret_cast<uint32_t*>(tqe + WP_TQ);
  volatile int* abort = reinterpret_cast<volatile int*>(tslot + 1);
  int* last_issued = reinterpret_cast<int*>(tslot + 2);  // [S]
  int* nzflag = last_issued + S;                          // [S]
  volatile int* tq = nzflag + S;                          // [WP_TQ] tile index, -1 = no more tiles
  volatile int* gtile = tq + WP_TQ;                       // [2] consumers' / epilogue's current tile
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int T = G.T.tile0[G.T.n];

  if (warp == 0) tmem_alloc(tslot, 2 * P::NCOL);
  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&ready[s], WP_CONS / 32);  // one arrival per consumer warp
      mbar_init(&hidone[s], 1);
      mbar_init(&ready2[s], WP_CONS / 32);
      mbar_init(&empty[s], 1);
      last_issued[s] = -1;
      nzflag[s] = 0;
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accfull[b], 1);
      mbar_init(&accempty[b], 128);
    }
    mbar_init(done, 1);
    for (int j = 0; j < WP_TQ; ++j) {
      mbar_init(&tqf[j], 1);
      mbar_init(&tqe[j], 3);  // the consumers' leader, the MMA lane, the epilogue's leader
    }
    *abort = 0;
    fence_mbar_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  // Tiles come through a ring of WP_TQ slots: the producer takes the next tile of its
  // sequence (blockIdx.x + k gridDim.x) and publishes it; the MMA lane and one leader
  // thread of the consumer and epilogue groups read it (a named barrier hands the
  // leader's copy to its group, so a group never splits at a barrier) and release the
  // slot.  The end of the sequence is published as -1, so every role stops on the same
  // tile.
  auto ring_read = [&](int seq, int& t) {  // false: the wait gave up (abort is set)
    const int j = seq & (WP_TQ - 1);
    if (!mbar_wait_ab(&tqf[j], (uint32_t)(seq / WP_TQ) & 1u, abort)) {
      *abort = 1;
      t = -1;
      return false;
    }
    t = tq[j];
    mbar_arrive(&tqe[j]);
    return true;
  };

  auto sA = [&](int s) { return sm + (size_t)s * P::STAGE_B; };
  auto sBh = [&](int s) { return sm + (size_t)s * P::STAGE_B + P::A_B; };  // [Bh; Bl], 2 NBH rows
  // tile t -> (geometry, image, row block, column split) and its chunk range (chunks of
  // 32 KB columns)
  auto decode = [&](int t, int& g, int& img, int& rb, int& cs, int& c0, int& c1) {
    win_tile(G.T, t, 32 * P::KB, g, img, rb, cs, c0, c1);
  };

  if (warp == 8) {
    if (lane == 0) {  // TMA producer
      int q = 0, s = 0;
      uint32_t ph = 0;
      bool ok = true;
      for (int seq = 0; ok; ++seq) {
        const int j = seq & (WP_TQ - 1);
        if (seq >= WP_TQ && !mbar_wait_ab(&tqe[j], (uint32_t)(seq / WP_TQ - 1) & 1u, abort)) {
          *abort = 1;
          break;
        }
        int t = (int)blockIdx.x + seq * (int)gridDim.x;
        if (t >= T) t = -1;
        tq[j] = t;
        mbar_arrive(&tqf[j]);  // release: the slot's tile index is visible to the readers
        if (t < 0) break;
        int g, img, rb, cs, c0, c1;
        decode(t, g, img, rb, cs, c0, c1);
        for (int c = c0; c < c1; ++c, ++q) {
          if (q == stall_at) {  // error-path test hook: the producer is lost here
            ok = false;
            break;
          }
          if (q >= S && !mbar_wait_ab(&empty[s], ph ^ 1u, abort)) {
            *abort = 1;
            ok = false;
            break;
          }
          mbar_arrive_expect_tx(&full[s], P::STAGE_B);
#pragma unroll
          for (int kb = 0; kb < P::KB; ++kb) {
            tma_load_3d(sA(s) + kb * P::A_KB, &G.mM[g], &full[s], 32 * (P::KB * c + kb), 128 * rb, img);
            tma_load_2d(sBh(s) + kb * P::B_KB, &G.mB[g], &full[s], 32 * (P::KB * c + kb), 0);
          }
          last_issued[s] = q;
          if (++s == S) {
            s = 0;
            ph ^= 1u;
          }
        }
      }
    }
  } else if (warp == 9) {
    if (lane == 0) {  // MMA issuer
      constexpr uint32_t IDESC2 = idesc_tf32(128, 2 * NBH);  // A x [Bh; Bl]
      // Al x Bh over the first NLO twiddle rows: the hi rows, plus (when NBH is not
      // a multiple of 16) a few lo rows whose Al*Bl terms only add accuracy
      constexpr uint32_t IDESC1 = idesc_tf32(128, P::NLO);
      uint32_t ph2 = 0;  // per-stage parity of hidone / ready2
      int tl = 0, s = 0;
      uint32_t ph = 0;
      bool ok = true;
      for (int seq = 0; ok; ++seq, ++tl) {
        int t;
        if (!ring_read(seq, t) || t < 0) break;
        int g, img, rb, cs, c0, c1;
        decode(t, g, img, rb, cs, c0, c1);
        const int buf = tl & 1;
        if (tl >= 2 && !mbar_wait_ab(&accempty[buf], (uint32_t)((tl - 2) >> 1) & 1u, abort)) {
          *abort = 1;
          break;
        }
        tc_fence_after();
        const uint32_t acc = tmem + (uint32_t)buf * P::NCOL;
        for (int c = c0; c < c1; ++c) {
          if (!mbar_wait_ab(&ready[s], ph, abort)) {
            *abort = 1;
            ok = false;
            break;
          }
          tc_fence_after();
          const bool two = *reinterpret_cast<volatile int*>(&nzflag[s]) != 0;
          nzflag[s] = 0;  // every consumer read it before arriving on ready[s]
#pragma unroll
          for (int kb = 0; kb < P::KB; ++kb) {
            const uint64_t da = desc_sw128(sA(s) + kb * P::A_KB), dbh = desc_sw128(sBh(s) + kb * P::B_KB);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              const uint32_t off = kk * 32;
              mma_tf32(acc, desc_add(da, off), desc_add(dbh, off), IDESC2, (c != c0 || kb != 0 || kk != 0) ? 1u : 0u);
            }
          }
          if (two) {
            mma_commit(&hidone[s]);
            if (!mbar_wait_ab(&ready2[s], (ph2 >> s) & 1u, abort)) {
              *abort = 1;
              ok = false;
              break;
            }
            ph2 ^= 1u << s;
            tc_fence_after();
#pragma unroll
            for (int kb = 0; kb < P::KB; ++kb) {
              const uint64_t da = desc_sw128(sA(s) + kb * P::A_KB), dbh = desc_sw128(sBh(s) + kb * P::B_KB);
#pragma unroll
              for (int kk = 0; kk < 4; ++kk) {
                const uint32_t off = kk * 32;
                mma_tf32(acc, desc_add(da, off), desc_add(dbh, off), IDESC1, 1u);
              }
            }
          }
          mma_commit(&empty[s]);
          if (++s == S) {
            s = 0;
            ph ^= 1u;
          }
        }
        if (ok) mma_commit(&accfull[buf]);  // arrives when this tile's MMAs have completed
      }
      mma_commit(done);  // arrives once everything issued above has completed
    }
  } else if (warp < 8) {  // warps 0-7: check / split the landed tiles in place
    uint32_t ph2 = 0, ph = 0;
    int s = 0;
    // a wait that gives up flags the error and the thread carries on through the
    // named barriers with the others (later waits return at once): a thread that
    // left alone would strand the rest at the next barrier
    for (int seq = 0;; ++seq) {
      if (tid == 0) {
        int t;
        ring_read(seq, t);
        gtile[0] = t;
      }
      named_bar(1, WP_CONS);
      const int t = gtile[0];
      named_bar(1, WP_CONS);  // every consumer holds t before the leader may overwrite it
      if (t < 0) break;
      int g, img, rb, cs, c0, c1;
      decode(t, g, img, rb, cs, c0, c1);
      for (int c = c0; c < c1; ++c) {
        if (!mbar_wait_ab(&full[s], ph, abort)) *abort = 1;
        float4* a = reinterpret_cast<float4*>(sA(s));
        float4 v[4 * P::KB];
        // x is exact in TF32 (x == round_tf32(x)) iff its low 13 mantissa bits are zero
        uint32_t low = 0;
#pragma unroll
        for (int i = 0; i < 4 * P::KB; ++i) {
          v[i] = a[tid + WP_CONS * i];
          low |= __float_as_uint(v[i].x) | __float_as_uint(v[i].y) | __float_as_uint(v[i].z) | __float_as_uint(v[i].w);
        }
        const bool nz = (low & 0x1FFFu) != 0u;
        if (__any_sync(0xffffffffu, nz) && lane == 0) atomicOr(&nzflag[s], 1);
        named_bar(1, WP_CONS);
        const bool two = *reinterpret_cast<volatile int*>(&nzflag[s]) != 0;
        if (two) {  // write Ah = round_tf32(A) in place; exact tiles are used as landed
#pragma unroll
          for (int i = 0; i < 4 * P::KB; ++i)
            a[tid + WP_CONS * i] =
                make_float4(tf32_round(v[i].x), tf32_round(v[i].y), tf32_round(v[i].z), tf32_round(v[i].w));
          fence_proxy_async();
        }
        // release: the warp's reads of nzflag and its Ah stores precede its one arrival
        __syncwarp();
        if (lane == 0) mbar_arrive(&ready[s]);
        if (two) {
          if (!mbar_wait_ab(&hidone[s], (ph2 >> s) & 1u, abort)) *abort = 1;
          ph2 ^= 1u << s;
#pragma unroll
          for (int i = 0; i < 4 * P::KB; ++i)
            a[tid + WP_CONS * i] = make_float4(v[i].x - tf32_round(v[i].x), v[i].y - tf32_round(v[i].y),
                                               v[i].z - tf32_round(v[i].z), v[i].w - tf32_round(v[i].w));
          fence_proxy_async();
          __syncwarp();
          if (lane == 0) mbar_arrive(&ready2[s]);
        }
        if (++s == S) {
          s = 0;
          ph ^= 1u;
        }
      }
    }
  } else {  // warps 10-13: epilogue
    const int etid = tid - 320, quarter = warp & 3;
    const int row = 32 * quarter + lane;
    const int KY = 2 * Ny + 1, NU = Nx + 1;
    const float inv_ff = 1.0f / ((float)Fx * (float)Fy);
    int tl = 0;
    for (int seq = 0;; ++seq, ++tl) {
      if (etid == 0) {
        int t;
        ring_read(seq, t);
        gtile[1] = t;
      }
      named_bar(2, 128);
      const int t = gtile[1];
      named_bar(2, 128);  // every epilogue thread holds t before the leader may overwrite it
      if (t < 0) break;
      int g, img, rb, cs, c0, c1;
      decode(t, g, img, rb, cs, c0, c1);
      const int buf = tl & 1;
      // on a wait that gives up: flag it and carry on with the group (see above)
      if (!mbar_wait_ab(&accfull[buf], (uint32_t)(tl >> 1) & 1u, abort)) *abort = 1;
      tc_fence_after();
      const uint32_t trow = tmem + (uint32_t)buf * P::NCOL + ((uint32_t)(32 * quarter) << 16);
      // sR[j] = (A Bh)[j] + (A Bl)[j]: 2 NBH columns in 8-column loads, one wait
      {
        uint32_t v[2 * NBH];
#pragma unroll
        for (int g = 0; g < 2 * NBH / 8; ++g) tmem_ld8_async(trow + 8u * g, &v[8 * g]);
        tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < NBH; ++j)
          if (j < KXw) sR[j * RS + row] = __uint_as_float(v[j]) + __uint_as_float(v[NBH + j]);
      }
      tc_fence_before();
      mbar_arrive(&accempty[buf]);  // the MMA lane may refill this accumulator
      const int y0 = 128 * rb;
      named_bar(2, 128);
      const int rows = G.T.rows[g], ncs = G.T.ncs[g];
      const int nps = part_stride > 0 ? part_stride : rows * ncs;
      float2* out = win_part + ((size_t)(G.T.img0[g] + img) * nps + (rb * ncs + cs)) * KY * NU;
      // one thread per (|v|, u): four row sums give both outputs +v and -v
      //   S1 = sum c tx, S2 = sum s ty, S3 = sum c ty, S4 = sum s tx
      //   (+v): (S1 - S2, S3 + S4)    (-v): (S1 + S2, S4 - S3)
      // with c, s the cos / -sin accumulator columns of u (s = 0 for u = 0)
      for (int pq = etid; pq < (Ny + 1) * NU; pq += 128) {
        const int av = pq / NU, u = pq - av * NU;
        const float4* rc = reinterpret_cast<const float4*>(sR + u * RS);
        const float4* rs = reinterpret_cast<const float4*>(sR + (Nx + u) * RS);
        // the tile's row twiddles of |v| (zero past Ly), two rows per vector, from L1
        const float4* rt = reinterpret_cast<const float4*>(G.ytab[g] + (size_t)av * (128 * rows) + y0);
        float s1 = 0.f, s2 = 0.f, s3 = 0.f, s4 = 0.f;
        if (u == 0) {
#pragma unroll 4
          for (int r4 = 0; r4 < 32; ++r4) {
            const float4 c = rc[r4], ta = __ldg(rt + 2 * r4), tb = __ldg(rt + 2 * r4 + 1);
            s1 = fmaf(c.x, ta.x, s1);
            s3 = fmaf(c.x, ta.y, s3);
            s1 = fmaf(c.y, ta.z, s1);
            s3 = fmaf(c.y, ta.w, s3);
            s1 = fmaf(c.z, tb.x, s1);
            s3 = fmaf(c.z, tb.y, s3);
            s1 = fmaf(c.w, tb.z, s1);
            s3 = fmaf(c.w, tb.w, s3);
          }
        } else {
#pragma unroll 4
          for (int r4 = 0; r4 < 32; ++r4) {
            const float4 c = rc[r4], sn = rs[r4], ta = __ldg(rt + 2 * r4), tb = __ldg(rt + 2 * r4 + 1);
            s1 = fmaf(c.x, ta.x, s1);
            s2 = fmaf(sn.x, ta.y, s2);
            s3 = fmaf(c.x, ta.y, s3);
            s4 = fmaf(sn.x, ta.x, s4);
            s1 = fmaf(c.y, ta.z, s1);
            s2 = fmaf(sn.y, ta.w, s2);
            s3 = fmaf(c.y, ta.w, s3);
            s4 = fmaf(sn.y, ta.z, s4);
            s1 = fmaf(c.z, tb.x, s1);
            s2 = fmaf(sn.z, tb.y, s2);
            s3 = fmaf(c.z, tb.y, s3);
            s4 = fmaf(sn.z, tb.x, s4);
            s1 = fmaf(c.w, tb.z, s1);
            s2 = fmaf(sn.w, tb.w, s2);
            s3 = fmaf(c.w, tb.w, s3);
            s4 = fmaf(sn.w, tb.z, s4);
          }
        }
        out[(Ny + av) * NU + u] = make_float2((s1 - s2) * inv_ff, (s3 + s4) * inv_ff);
        if (av > 0) out[(Ny - av) * NU + u] = make_float2((s1 + s2) * inv_ff, (s4 - s3) * inv_ff);
      }
      named_bar(2, 128);  // sR is free for the next tile
    }
  }
  // the MMA lane always commits `done`; everyone waits for the tensor cores to drain
  if (!mbar_wait(done, 0)) *abort = 1;
  __syncthreads();
  if (*abort) {
    if (tid == 256)  // warp 8 lane 0: wait for the last load of every stage
      for (int s = 0; s < S; ++s)
        if (last_issued[s] >= 0) mbar_wait(&full[s], (uint32_t)(last_issued[s] / S) & 1u, 200u);
    if (tid == 0) atomicExch(err, 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 2 * P::NCOL);
}

// ---------------------------------------------------------------------------
// FI contraction on the tensor cores
// ---------------------------------------------------------------------------
template <int KBLK, int BN>
struct FiTC {
  static constexpr uint32_t A_KB = 128 * 128;     // 128 rows x 32 fp32
  static constexpr uint32_t B_KB = BN * 128;      // BN rows x 32 fp32
  static constexpr uint32_t A_BYTES = 2 * KBLK * A_KB;
  // a B stage is one K block of a tile (its hi and lo halves back to back); a tile takes
  // KBLK consecutive stages.  K = 32 tiles: two stages and four staging tiles per
  // epilogue warp; K = 64 tiles: three stages and two staging tiles.
  static constexpr uint32_t STAGE_B = 2 * B_KB;
  static constexpr int NS = KBLK == 1 ? 2 : 3;
  static constexpr int NOUT = KBLK == 1 ? 4 : 2;
  static constexpr uint32_t OUT_B = 32 * 128;     // 32 rows x 32 fp32 staging tile of one warp
  static constexpr size_t SMEM = 1024 + A_BYTES + (size_t)NS * STAGE_B + 8 * NOUT * OUT_B + 3 * BN * 4 + 512;
};
constexpr int FI_THREADS = 320;  // warps 0-7 epilogue (two groups), 8 TMA, 9 MMA
constexpr int FI_TQ = 8;         // tile ring slots

// Persistent FI contraction: one CTA per SM takes a contiguous range of output tiles
// ordered (row band, image, column tile), so the Cy operand (A, the row band's
// twiddles) is reloaded only when the range crosses a row band.  Tm tiles (B) stream through an NS-stage TMA ring; the two TMEM
// accumulators alternate between tiles.  Roles (320 threads):
//   warp 8   : TMA producer  [band change: wait emptyA] A -> fullA;
//              [wait emptyB[s]] B -> fullB[s]
//   warp 9   : MMA issuer    [band change: commit emptyA, wait fullA]; wait fullB[s],
//              accEmpty[b]; Ah x [Bh; Bl] (N = 2 BN) + Al x Bh; commit emptyB[s], accFull[b]
//   warps 0-7: epilogue, each warp on its own: warp w drains TMEM lane quarter w % 4
//              for the 32-column slabs w / 4, w / 4 + 2, ...: hi + lo halves + T0[X] ->
//              its swizzled 32-row staging tile -> its TMA store; each warp arrives on
//              accEmpty[b] once it has read the tile.
// The epilogue is latency-bound per slab (TMEM load, staging, store issue); with no
// barrier between the warps each keeps NOUT stores of its own in flight.
template <int KBLK, int BN>
__global__ void __launch_bounds__(FI_THREADS, 1) fi_tc_kernel(const __grid_constant__ CUtensorMap tmCh,
                                                              const __grid_constant__ CUtensorMap tmCl,
                                                              const __grid_constant__ CUtensorMap tmTh,
                                                              const __grid_constant__ CUtensorMap tmTl,
                                                              const __grid_constant__ CUtensorMap tmOut, int Lx,
                                                              int batch, int ntile, int ntiles,
                                                              const float* __restrict__ t0g, int* __restrict__ err) {
  using P = FiTC<KBLK, BN>;
  constexpr int NS = P::NS, NOUT = P::NOUT;
  extern __shared__ unsigned char smraw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  unsigned char* sAh = sm;
  unsigned char* sAl = sm + KBLK * P::A_KB;
  unsigned char* sB = sm + P::A_BYTES;               // [NS][kb][hi, lo]
  unsigned char* sOut = sB + NS * P::STAGE_B;        // [8 epilogue warps][NOUT][OUT_B]
  float* sT0 = reinterpret_cast<float*>(sOut + 8 * NOUT * P::OUT_B);  // [3][BN]: the DC rows of tiles q % 3
  uint64_t* fullA = reinterpret_cast<uint64_t*>(sT0 + 3 * BN);
  uint64_t* emptyA = fullA + 1;
  uint64_t* fullB = fullA + 2;           // [NS]
  uint64_t* emptyB = fullB + NS;         // [NS]
  uint64_t* accFull = emptyB + NS;       // [2]
  uint64_t* accEmpty = accFull + 2;      // [2]
  uint64_t* drain = accEmpty + 2;
  uint64_t* tqf = drain + 1;             // [FI_TQ] tile-ring slot published (producer)
  uint64_t* tqe = tqf + FI_TQ;           // [FI_TQ] slot read by the MMA lane and both epilogue groups
  uint32_t* tslot = reinterpret_cast<uint32_t*>(tqe + FI_TQ);
  volatile int* abort = reinterpret_cast<volatile int*>(tslot + 1);
  int* last_issued = reinterpret_cast<int*>(tslot + 2);  // [NS], then the last A generation
  volatile int* tq = last_issued + NS + 1;               // [FI_TQ] tile index, -1 = no more tiles
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int i0 = (int)((long long)ntiles * blockIdx.x / gridDim.x);
  const int i1 = (int)((long long)ntiles * (blockIdx.x + 1) / gridDim.x);
  // tile i -> (row band, image, column tile)
  auto band_of = [&](int i) { return i / (batch * ntile); };
  auto decode = [&](int i, int& yb, int& img, int& xt) {
    yb = i / (batch * ntile);
    const int r = i - yb * batch * ntile;
    img = r / ntile;
    xt = r - img * ntile;
  };

  if (warp == 0) tmem_alloc(tslot, 4 * BN);  // two accumulators of [A Bh | A Bl]
  if (tid == 0) {
    mbar_init(fullA, 1);
    mbar_init(emptyA, 1);
    for (int s = 0; s < NS; ++s) {
      mbar_init(&fullB[s], 1);
      mbar_init(&emptyB[s], 1);
      last_issued[s] = -1;
    }
    last_issued[NS] = -1;
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accFull[b], 1);
      mbar_init(&accEmpty[b], 8);  // one arrival per epilogue warp
    }
    mbar_init(drain, 1);
    for (int j = 0; j < FI_TQ; ++j) {
      mbar_init(&tqf[j], 1);
      mbar_init(&tqe[j], 9);  // the MMA lane and the eight epilogue warps
    }
    *abort = 0;
    fence_mbar_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  // Tiles come through a ring of FI_TQ slots, as in the window kernel: the producer takes
  // the next tile of its contiguous range [i0, i1) and publishes it (-1 at the end); the
  // MMA lane and every epilogue warp (its lane 0) read it and release the slot.  The
  // epilogue peeks at the next slot to fetch that tile's DC row one tile ahead.
  auto ring_read = [&](int seq, int& t) {  // false: the wait gave up (abort is set)
    const int j = seq & (FI_TQ - 1);
    if (!mbar_wait_ab(&tqf[j], (uint32_t)(seq / FI_TQ) & 1u, abort)) {
      *abort = 1;
      t = -1;
      return false;
    }
    t = tq[j];
    mbar_arrive(&tqe[j]);
    return true;
  };
  // the hi and lo tiles of one K block sit back to back, so Ah x [Bh; Bl] is one N = 2 BN MMA
  auto Bh = [&](int s) { return sB + (size_t)s * P::STAGE_B; };
  auto Bl = [&](int s) { return sB + (size_t)s * P::STAGE_B + P::B_KB; };

  if (warp == 8) {
    if (lane == 0) {  // TMA producer
      int cur = -1, gen = 0;
      for (int seq = 0;; ++seq) {
        const int j = seq & (FI_TQ - 1);
        if (seq >= FI_TQ && !mbar_wait_ab(&tqe[j], (uint32_t)(seq / FI_TQ - 1) & 1u, abort)) {
          *abort = 1;
          break;
        }
        int i = i0 + seq;
        if (i >= i1) i = -1;
        tq[j] = i;
        mbar_arrive(&tqf[j]);  // release: the slot's tile index is visible to the readers
        if (i < 0) break;
        int yb, img, xt;
        decode(i, yb, img, xt);
        if (yb != cur) {  // (re)load the row band's Cy tiles once the MMAs on the previous ones are done
          if (gen > 0 && !mbar_wait_ab(emptyA, (uint32_t)(gen - 1) & 1u, abort)) {
            *abort = 1;
            break;
          }
          mbar_arrive_expect_tx(fullA, P::A_BYTES);
          for (int kb = 0; kb < KBLK; ++kb) {
            tma_load_2d(sAh + (size_t)kb * P::A_KB, &tmCh, fullA, 32 * kb, 128 * yb);
            tma_load_2d(sAl + (size_t)kb * P::A_KB, &tmCl, fullA, 32 * kb, 128 * yb);
          }
          last_issued[NS] = gen;
          ++gen;
          cur = yb;
        }
        bool stop = false;
        for (int kb = 0; kb < KBLK; ++kb) {  // stage g: K block kb of tile seq
          const int g = seq * KBLK + kb, s = g % NS;
          if (g >= NS && !mbar_wait_ab(&emptyB[s], (uint32_t)((g - NS) / NS) & 1u, abort)) {
            *abort = 1;
            stop = true;
            break;
          }
          mbar_arrive_expect_tx(&fullB[s], P::STAGE_B);
          tma_load_3d(Bh(s), &tmTh, &fullB[s], 32 * kb, xt * BN, img);
          tma_load_3d(Bl(s), &tmTl, &fullB[s], 32 * kb, xt * BN, img);
          last_issued[s] = g;
        }
        if (stop) break;
      }
    }
  } else if (warp == 9) {
    if (lane == 0) {  // MMA issuer
      constexpr uint32_t IDESC2 = idesc_tf32(128, 2 * BN);  // Ah x [Bh; Bl]
      constexpr uint32_t IDESC1 = idesc_tf32(128, BN);      // Al x Bh
      int cur = -1, gen = 0;
      bool ok = true;
      for (int seq = 0; ok; ++seq) {
        int i;
        if (!ring_read(seq, i)) {
          ok = false;
          break;
        }
        if (i < 0) break;
        const int q = seq, b = q & 1;
        const int yb = band_of(i);
        if (yb != cur) {
          // every MMA on the previous band's A tiles is issued: they may be replaced once those complete
          if (cur >= 0) mma_commit(emptyA);
          if (!mbar_wait_ab(fullA, (uint32_t)gen & 1u, abort)) {
            ok = false;
            break;
          }
          ++gen;
          cur = yb;
        }
        if (q >= 2 && !mbar_wait_ab(&accEmpty[b], (uint32_t)((q - 2) >> 1) & 1u, abort)) {
          ok = false;
          break;
        }
        const uint32_t acc = tmem + (uint32_t)(b * 2 * BN);
#pragma unroll
        for (int kb = 0; kb < KBLK; ++kb) {
          const int g = q * KBLK + kb, s = g % NS;
          if (!mbar_wait_ab(&fullB[s], (uint32_t)(g / NS) & 1u, abort)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint64_t dah = desc_sw128(sAh + (size_t)kb * P::A_KB), dal = desc_sw128(sAl + (size_t)kb * P::A_KB);
          const uint64_t dbh = desc_sw128(Bh(s));
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {
            const uint32_t off = kk * 32;
            mma_tf32(acc, desc_add(dah, off), desc_add(dbh, off), IDESC2, (kb | kk) != 0 ? 1u : 0u);
            mma_tf32(acc, desc_add(dal, off), desc_add(dbh, off), IDESC1, 1u);
          }
          mma_commit(&emptyB[s]);
        }
        if (!ok) break;
        mma_commit(&accFull[b]);
      }
      if (!ok) *abort = 1;
    }
  } else {  // warps 0-7: epilogue, every warp on its own
    // Warp w drains TMEM lane quarter w % 4 (32 image rows) for the slabs w / 4,
    // w / 4 + 2, ... of every tile: 32 rows x 32 columns per slab, hi + lo halves + the DC
    // row, through its own swizzled staging tiles and its own 32-row TMA stores.  No
    // barrier joins the warps, so each keeps NOUT stores of its own in flight.
    const int quarter = warp & 3, half = warp >> 2;
    unsigned char* stg = sOut + (size_t)warp * NOUT * P::OUT_B;
    int slab_count = 0;
    constexpr int NSL = BN / 64;  // slabs per warp per tile (1 or 2)
    // the DC row values this lane writes into the shared row of its slabs: column
    // slab * 32 + lane of tile i
    auto t0_of = [&](int i, float (&t)[NSL]) {
      int yb, img, xt;
      decode(i, yb, img, xt);
#pragma unroll
      for (int k = 0; k < NSL; ++k) {
        const int X = xt * BN + (half + 2 * k) * 32 + lane;
        t[k] = X < Lx ? __ldg(t0g + (size_t)img * Lx + X) : 0.f;
      }
    };
    float t0n[NSL];  // DC row values of tile tn, fetched one tile ahead when the ring holds it
    int tn = -1;
    for (int seq = 0;; ++seq) {
      int i = -1, nx = -1;
      if (lane == 0) {
        ring_read(seq, i);
        if (i >= 0) {  // peek: is the next tile published already?
          const int j1 = (seq + 1) & (FI_TQ - 1);
          if (mbar_poll(&tqf[j1], (uint32_t)((seq + 1) / FI_TQ) & 1u)) nx = tq[j1];
        }
      }
      i = __shfl_sync(0xffffffffu, i, 0);
      nx = __shfl_sync(0xffffffffu, nx, 0);
      if (i < 0) break;
      const int q = seq, b = q & 1;
      int yb, img, xt;
      decode(i, yb, img, xt);
      float t0c[NSL];
      if (tn == i) {
#pragma unroll
        for (int k = 0; k < NSL; ++k) t0c[k] = t0n[k];
      } else {
        t0_of(i, t0c);
      }
      // the shared DC row of tile q, in row buffer q % 3: this warp writes and then reads only
      // its own slabs' columns (warps of the other quarters write the same values).  A warp
      // writes it before waiting for the accumulator, so a fast warp writes tile q's row
      // while a slow one may still read tile q - 2's (the MMA lane refills an accumulator only
      // after every warp has released it, so no warp is three tiles ahead of another): three
      // row buffers keep those apart.
      float* t0s = sT0 + (q % 3) * BN;
#pragma unroll
      for (int k = 0; k < NSL; ++k) t0s[(half + 2 * k) * 32 + lane] = t0c[k];
      __syncwarp();
      if (nx >= 0) {
        t0_of(nx, t0n);
        tn = nx;
      } else {
        tn = -1;
      }
      // a wait that gives up flags the error and carries on (later waits return at once)
      if (!mbar_wait_ab(&accFull[b], (uint32_t)(q >> 1) & 1u, abort)) *abort = 1;
      tc_fence_after();
      const uint32_t trow = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(b * 2 * BN);
#pragma unroll 1
      for (int slab = half; slab < BN / 32; slab += 2, ++slab_count) {
        uint32_t v[32], w[32];
        tmem_ld32_async(trow + (uint32_t)(slab * 32), v);
        tmem_ld32_async(trow + (uint32_t)(BN + slab * 32), w);
        tmem_ld_wait();
        unsigned char* st = stg + (size_t)(slab_count % NOUT) * P::OUT_B;
        if (lane == 0) bulk_wait_read<NOUT - 1>();  // the store that used this staging tile has read it
        __syncwarp();
        const float4* t04 = reinterpret_cast<const float4*>(t0s + slab * 32);
        float4 d[8];
#pragma unroll
        for (int q4 = 0; q4 < 8; ++q4) d[q4] = t04[q4];
        float4* rowp = reinterpret_cast<float4*>(st + (size_t)lane * 128);
#pragma unroll
        for (int q4 = 0; q4 < 8; ++q4) {
          const int j = 4 * q4;
          rowp[q4 ^ (lane & 7)] = make_float4(__uint_as_float(v[j]) + (__uint_as_float(w[j]) + d[q4].x),
                                              __uint_as_float(v[j + 1]) + (__uint_as_float(w[j + 1]) + d[q4].y),
                                              __uint_as_float(v[j + 2]) + (__uint_as_float(w[j + 2]) + d[q4].z),
                                              __uint_as_float(v[j + 3]) + (__uint_as_float(w[j + 3]) + d[q4].w));
        }
        fence_proxy_async();
        __syncwarp();
        if (lane == 0) {
          // evict-first: the images are not read again here, and keeping them from
          // displacing the T tiles and twiddles in L2 measured 52 -> 46.5 us per 64 images
          tma_store_3d_hint(&tmOut, st, xt * BN + slab * 32, 128 * yb + 32 * quarter, img, policy_evict_first());
          bulk_commit();
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&accEmpty[b]);
    }
    if (lane == 0) bulk_wait0();
  }
  __syncthreads();
  if (*abort) {
    if (tid == 288) {  // the MMA lane: drain what it issued
      mma_commit(drain);
      mbar_wait(drain, 0, 200u);
    }
    if (tid == 256) {  // the producer: wait for its last loads
      if (last_issued[NS] >= 0) mbar_wait(fullA, (uint32_t)last_issued[NS] & 1u, 200u);
      for (int s = 0; s < NS; ++s)
        if (last_issued[s] >= 0) mbar_wait(&fullB[s], (uint32_t)(last_issued[s] / NS) & 1u, 200u);
    }
    if (tid == 0) atomicExch(err, 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 4 * BN);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
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

// FP32 tensor map with a 128-byte swizzle and a {32, box1(, 1)} box.
static int make_map(litho_ctx* ctx, CUtensorMap* m, const void* base, int rank, uint64_t d0, uint64_t d1,
                    uint64_t d2, uint32_t box1) {
  auto fn = encode_fn();
  if (fn == nullptr) {
    set_error(ctx, LITHO_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    return LITHO_ERR_CUDA;
  }
  cuuint64_t dims[3] = {d0, d1, d2};
  cuuint64_t strides[2] = {d0 * 4, d0 * d1 * 4};
  cuuint32_t box[3] = {32, box1, 1};
  cuuint32_t es[3] = {1, 1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, rank, const_cast<void*>(base), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error(ctx, LITHO_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return LITHO_ERR_CUDA;
  }
  return LITHO_OK;
}

// twiddle rows of each half of the window DFT's B tile: 2Nx+1 rounded up to 8
static int nb_for(int Nx) {
  const int nj = 2 * Nx + 1;
  return nj <= 40 ? (nj + 7) / 8 * 8 : -1;
}
static int kblk_for(int Ny) { return std::max(1, (4 * Ny + 31) / 32); }  // 4Ny K rows (the DC row is separate)

bool tc_supported(const ImgGeom& g) {
  return (g.Lx % 4) == 0 && g.Nx <= 16 && g.Ny <= 16 && nb_for(g.Nx) > 0 && kblk_for(g.Ny) <= 2;
}

static int tc_err_flag(litho_ctx* ctx, int** flag) {
  if (ctx->mx_d.p == nullptr) {
    LITHO_RET(ctx->mx_d.ensure(ctx, 256));
    LITHO_CUDA_TRY(ctx, cudaMemsetAsync(ctx->mx_d.p, 0, 256, ctx->stream));
  }
  *flag = ctx->mx_d.as<int>();
  return LITHO_OK;
}

int tc_err_flag_public(litho_ctx* ctx, int** flag) { return tc_err_flag(ctx, flag); }

// Read and clear the device-side timeout flag of the tensor-core kernels
// (the caller has synchronised the stream).
int tc_check_flag(litho_ctx* ctx) {
  if (ctx->mx_d.p == nullptr) return LITHO_OK;
  int v = 0;
  LITHO_CUDA_TRY(ctx, cudaMemcpy(&v, ctx->mx_d.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (v != 0) {
    LITHO_CUDA_TRY(ctx, cudaMemset(ctx->mx_d.p, 0, 256));
    set_error(ctx, LITHO_ERR_TIMEOUT, "a tensor-core pipeline wait gave up (bounded mbarrier wait)");
    return LITHO_ERR_TIMEOUT;
  }
  return LITHO_OK;
}

static int cached_table(litho_ctx* ctx, std::tuple<int, int, int, int> key, size_t bytes, bool* fresh,
                        float** out) {
  auto it = ctx->twx_tables.find(key);
  *fresh = false;
  if (it == ctx->twx_tables.end()) {
    DevBuf b;
    LITHO_RET(b.ensure(ctx, bytes));
    it = ctx->twx_tables.emplace(key, b).first;
    *fresh = true;
  }
  *out = it->second.as<float>();
  return LITHO_OK;
}

// Column twiddles (hi/lo TF32 rows) and epilogue row twiddles of one window geometry,
// cached in the context and built on first use on the context's stream.
template <int NBH>
static int win_tc_tables(litho_ctx* ctx, const ImgGeom& g, float** twh, float** yt) {
  bool fresh = false;
  float* tw = nullptr;
  LITHO_RET(cached_table(ctx, std::make_tuple(g.Lx, g.Fx, g.Nx, -NBH), (size_t)2 * NBH * g.Lx * sizeof(float),
                         &fresh, &tw));
  if (fresh) {
    StageScope sc(ctx, LITHO_STAGE_UPLOAD);
    twT_init_kernel<<<dim3((g.Lx + 127) / 128, NBH), 128, 0, ctx->stream>>>(tw, tw + (size_t)NBH * g.Lx, g.Lx, g.Fx,
                                                                            g.Nx, NBH);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
  }
  // row twiddles of the epilogue, rows padded to a multiple of 128, cached per (Ly, Fy, Ny)
  const int Lyp = (g.Ly + 127) / 128 * 128;
  LITHO_RET(cached_table(ctx, std::make_tuple(g.Ly, g.Fy, g.Ny, -3001), (size_t)(g.Ny + 1) * Lyp * sizeof(float2),
                         &fresh, yt));
  if (fresh) {
    StageScope sc(ctx, LITHO_STAGE_UPLOAD);
    ytab_init_kernel<<<dim3(Lyp / 128, g.Ny + 1), 128, 0, ctx->stream>>>(reinterpret_cast<float2*>(*yt), g.Ly,
                                                                          Lyp, g.Fy);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
  }
  *twh = tw;
  return LITHO_OK;
}

template <int NBH>
static int launch_win_tc(litho_ctx* ctx, const WinPart* parts, int n, float2* win_part, int* err) {
  WinGeo G;
  std::memset(&G, 0, sizeof(G));
  G.T.n = n;
  int tiles = 0;
  for (int i = 0; i < n; ++i) {
    const ImgPlan& p = parts[i].plan;
    const ImgGeom& g = p.g;
    float *twh = nullptr, *yt = nullptr;
    LITHO_RET(win_tc_tables<NBH>(ctx, g, &twh, &yt));
    LITHO_RET(make_map(ctx, &G.mM[i], parts[i].masks, 3, g.Lx, g.Ly, p.batch, 128));
    LITHO_RET(make_map(ctx, &G.mB[i], twh, 2, g.Lx, 2 * NBH, 1, 2 * NBH));  // hi rows, then lo rows
    G.ytab[i] = reinterpret_cast<const float2*>(yt);
    G.T.Lx[i] = g.Lx;
    G.T.rows[i] = (g.Ly + 127) / 128;
    G.T.ncs[i] = std::max(1, p.colSplits);
    G.T.img0[i] = parts[i].img0;
    G.T.tile0[i] = tiles;
    tiles += G.T.rows[i] * p.batch * G.T.ncs[i];
  }
  G.T.tile0[n] = tiles;
  const ImgGeom& g0 = parts[0].plan.g;
  // as many ring stages as shared memory holds
  using P = WinTC<NBH>;
  const size_t fixed = 1024 + win_epi_bytes(g0.Nx) + win_bar_bytes(WP_MAX_STAGES);
  const int S = (int)std::min<size_t>(WP_MAX_STAGES, (WP_SMEM_CAP - fixed) / P::STAGE_B);
  const size_t smem = 1024 + (size_t)S * P::STAGE_B + win_epi_bytes(g0.Nx) + win_bar_bytes(S);
  LITHO_CUDA_TRY(ctx, cudaFuncSetAttribute(win_dft_tc_kernel<NBH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
  const int grid = std::min(tiles, ctx->sm_count);  // persistent: one CTA per SM
  StageScope sc(ctx, LITHO_STAGE_WIN_DFT);
  win_dft_tc_kernel<NBH><<<grid, WP_THREADS, smem, ctx->stream>>>(G, g0.Fx, g0.Fy, g0.Nx, g0.Ny, S, win_part,
                                                                  parts[0].plan.part_stride, err,
                                                                  ctx->test_stall_chunk);
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  return LITHO_OK;
}

// One persistent launch over the masks of up to WP_MAX_GEO sizes that share the period,
// the kernel support and the partial array (their plans' Fx, Fy, Nx, Ny and part_stride).
int run_win_dft_tc_multi(litho_ctx* ctx, const WinPart* parts, int n, float2* win_part) {
  if (n < 1 || n > WP_MAX_GEO) {
    set_error(ctx, LITHO_ERR_ARG, "window DFT over %d mask sizes (1..%d)", n, WP_MAX_GEO);
    return LITHO_ERR_ARG;
  }
  const ImgGeom& g0 = parts[0].plan.g;
  for (int i = 1; i < n; ++i) {
    const ImgPlan& p = parts[i].plan;
    if (p.g.Fx != g0.Fx || p.g.Fy != g0.Fy || p.g.Nx != g0.Nx || p.g.Ny != g0.Ny ||
        p.part_stride != parts[0].plan.part_stride) {
      set_error(ctx, LITHO_ERR_ARG, "window DFT mask sizes of one launch must share the period and the kernels");
      return LITHO_ERR_ARG;
    }
  }
  int* err = nullptr;
  LITHO_RET(tc_err_flag(ctx, &err));
  switch (nb_for(g0.Nx)) {
    case 8: return launch_win_tc<8>(ctx, parts, n, win_part, err);
    case 16: return launch_win_tc<16>(ctx, parts, n, win_part, err);
    case 24: return launch_win_tc<24>(ctx, parts, n, win_part, err);
    case 32: return launch_win_tc<32>(ctx, parts, n, win_part, err);
    case 40: return launch_win_tc<40>(ctx, parts, n, win_part, err);
    default:
      set_error(ctx, LITHO_ERR_UNSUPPORTED, "tensor-core window DFT supports Nx <= 16");
      return LITHO_ERR_UNSUPPORTED;
  }
}

int run_win_dft_tc(litho_ctx* ctx, const ImgPlan& p, const float* masks, float2* win_part) {
  const WinPart part{p, masks, 0};
  return run_win_dft_tc_multi(ctx, &part, 1, win_part);
}

template <int KBLK, int BN>
static int launch_fi_tc(litho_ctx* ctx, const ImgPlan& p, const float* cyh, const float* cyl, const float* tmh,
                        const float* tml, const float* t0, float* images, int* err) {
  const ImgGeom& g = p.g;
  const int KP = 32 * KBLK;
  CUtensorMap mCh, mCl, mTh, mTl, mO;
  LITHO_RET(make_map(ctx, &mCh, cyh, 2, KP, g.Ly, 1, 128));
  LITHO_RET(make_map(ctx, &mCl, cyl, 2, KP, g.Ly, 1, 128));
  LITHO_RET(make_map(ctx, &mTh, tmh, 3, KP, g.Lx, p.batch, BN));
  LITHO_RET(make_map(ctx, &mTl, tml, 3, KP, g.Lx, p.batch, BN));
  LITHO_RET(make_map(ctx, &mO, images, 3, g.Lx, g.Ly, p.batch, 32));  // one warp's 32-row store
  static_assert(FiTC<KBLK, BN>::SMEM <= 227 * 1024, "FI tiles exceed the shared memory of one CTA");
  const size_t smem = FiTC<KBLK, BN>::SMEM;
  LITHO_CUDA_TRY(ctx, cudaFuncSetAttribute(fi_tc_kernel<KBLK, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
  // persistent: one CTA per SM over all (row band, image, column tile) tiles
  const int ntile = (g.Lx + BN - 1) / BN, rows = (g.Ly + 127) / 128;
  const int ntiles = rows * p.batch * ntile;
  const int grid = std::min(ntiles, ctx->sm_count);
  StageScope sc(ctx, LITHO_STAGE_FI_OUT);
  fi_tc_kernel<KBLK, BN><<<grid, FI_THREADS, smem, ctx->stream>>>(mCh, mCl, mTh, mTl, mO, g.Lx, p.batch, ntile,
                                                                  ntiles, t0, err);
  LITHO_CUDA_TRY(ctx, cudaGetLastError());
  return LITHO_OK;
}

// hi/lo T rows [2][batch][Lx][KP] float, then the DC row T0 [batch][Lx] float
size_t fi_tc_workspace_bytes(const ImgGeom& g, int batch) {
  return (size_t)2 * batch * g.Lx * 32 * kblk_for(g.Ny) * sizeof(float) + (size_t)batch * g.Lx * sizeof(float);
}

// Pointers of one run of images inside the FI workspace of a batch of `total` images:
// hi rows [total][Lx][KP], lo rows likewise, then the DC rows [total][Lx].
FiTcBufs fi_tc_bufs(float* base, const ImgGeom& g, int total, int first) {
  const size_t KP = 32 * (size_t)kblk_for(g.Ny), plane = (size_t)total * g.Lx * KP;
  FiTcBufs b;
  b.tmh = base + (size_t)first * g.Lx * KP;
  b.tml = base + plane + (size_t)first * g.Lx * KP;
  b.t0 = base + 2 * plane + (size_t)first * g.Lx;
  return b;
}

// FI step 1 on the tensor-core layout: the band's interpolation rows as K-major hi/lo
// TF32 splits and the DC row, on the context's stream.
int run_fi_rows_tc(litho_ctx* ctx, const ImgPlan& p, const float2* band_part, const FiTcBufs& b) {
  const ImgGeom& g = p.g;
  const int KP = 32 * kblk_for(g.Ny);
  const float2* twF = nullptr;
  LITHO_RET(fi_twiddles(ctx, g, &twF));
  StageScope sc(ctx, LITHO_STAGE_FI_PREP);
  LITHO_CUDA_TRY(ctx, launch_fi_rows(ctx->stream, p, band_part, twF, KP, nullptr, b.tmh, b.tml, b.t0));
  return LITHO_OK;
}

// FI step 2: the tensor-core contraction writing the images, on the context's stream.
int run_fi_out_tc(litho_ctx* ctx, const ImgPlan& p, const FiTcBufs& b, float* images) {
  const ImgGeom& g = p.g;
  const int KBLK = kblk_for(g.Ny);
  const int KP = 32 * KBLK;
  int* err = nullptr;
  LITHO_RET(tc_err_flag(ctx, &err));
  // Cy table, cached per (Ly, Fy, Ny)
  bool fresh = false;
  float* cy = nullptr;
  LITHO_RET(cached_table(ctx, std::make_tuple(g.Ly, g.Fy, g.Ny, -1000 - KP), (size_t)2 * g.Ly * KP * sizeof(float),
                         &fresh, &cy));
  float* cyh = cy;
  float* cyl = cy + (size_t)g.Ly * KP;
  if (fresh) {
    StageScope sc(ctx, LITHO_STAGE_UPLOAD);
    cyT_init_kernel<<<dim3((g.Ly + 127) / 128, KP), 128, 0, ctx->stream>>>(cyh, cyl, g.Ly, g.Fy, g.Ny, KP);
    LITHO_CUDA_TRY(ctx, cudaGetLastError());
  }
  if (KBLK == 1) return launch_fi_tc<1, 128>(ctx, p, cyh, cyl, b.tmh, b.tml, b.t0, images, err);
  // K = 64: 128-column tiles with two B stages and one staging tile per epilogue warp
  // (measured faster than 64-column tiles with three stages and two staging tiles once
  // the epilogue warps stopped waiting on one another: the batched 2048 class 0.46 ->
  // 0.40 ms)
  return launch_fi_tc<2, 128>(ctx, p, cyh, cyl, b.tmh, b.tml, b.t0, images, err);
}

// tmT: caller-provided workspace of fi_tc_workspace_bytes(g, batch) bytes, or
// nullptr to use the context's grow-only buffer.
int run_fi_tc(litho_ctx* ctx, const ImgPlan& p, const float2* band_part, float* tmT, float* images) {
  if (tmT == nullptr) {
    LITHO_RET(ctx->mx_b.ensure(ctx, fi_tc_workspace_bytes(p.g, p.batch)));
    tmT = ctx->mx_b.as<float>();
  }
  const FiTcBufs b = fi_tc_bufs(tmT, p.g, p.batch, 0);
  LITHO_RET(run_fi_rows_tc(ctx, p, band_part, b));
  return run_fi_out_tc(ctx, p, b, images);
}

}  // namespace litho
