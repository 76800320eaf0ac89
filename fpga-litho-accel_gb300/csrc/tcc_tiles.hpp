// Output tiles of the split-BF16 TCC product that the TCC assembly reads, and the
// persistent GEMM's work schedule over them.  Plain C++ with no CUDA, so both are
// also checked on the CPU.
#pragma once
#include <algorithm>
#include <vector>

namespace litho {

struct TileMN {
  int m, n;  // 128-row tile index (of 2n rows), bn-column tile index (of n columns)
};

// C = A A_top^T with A = [X; Y] (2n rows): rows < n hold X X^T (the real part,
// symmetric), rows >= n hold Y X^T (the imaginary part, antisymmetric).  The TCC
// reads C[a][b] with a <= b and C[n + a][b] with a < b, so only the 128 x bn
// tiles that hold such entries are listed (about half), in blocks of 12 row
// tiles by 12 * 128 / bn column tiles that share their A and B panels in L2.
inline std::vector<TileMN> tcc_needed_tiles(int n, int bn = 128) {
  const int MT = (2 * n + 127) / 128, NT = (n + bn - 1) / bn;
  const int mblk = 12, nblk = std::max(1, 12 * 128 / bn);
  std::vector<TileMN> tiles;
  for (int mb = 0; mb < MT; mb += mblk)
    for (int nb = 0; nb < NT; nb += nblk)
      for (int mt = mb; mt < std::min(MT, mb + mblk); ++mt)
        for (int nt = nb; nt < std::min(NT, nb + nblk); ++nt) {
          const int r0 = mt * 128, r1 = std::min(r0 + 128, 2 * n);
          const int cmax = std::min(nt * bn + bn - 1, n - 1);
          const bool top = r0 < n && r0 <= cmax;                      // some a <= b with a < n
          const bool bottom = r1 > n && std::max(r0, n) - n < cmax;  // some n + a with a < b
          if (top || bottom) tiles.push_back({mt, nt});
        }
  return tiles;
}

// One piece of a persistent CTA's work: K slices [k0, k1) of tile `tile`.
// slot < 0: the whole K range, written straight to C; slot >= 0: a partial sum
// written to partial slot `slot`, added into C by the fix-up in K order.
struct GemmSeg {
  int tile, k0, k1, slot;
};

struct GemmSchedule {
  std::vector<int> begin;      // [ctas + 1]: CTA b runs segs[begin[b] .. begin[b + 1])
  std::vector<GemmSeg> segs;
  std::vector<int> fix_tile;   // tiles summed from partial slots
  std::vector<int> fix_begin;  // [fix_tile.size() + 1] into fix_slot
  std::vector<int> fix_slot;   // the partial slots of each such tile, in K order
  int nslots = 0;
};

// ntiles tiles of nk K slices each on `ctas` persistent CTAs (ctas >= 1, nk >= 1).
// sched 0 (GEMM_WHOLE_TILES): data-parallel rounds, tile t on CTA t % ctas.
// sched 1 (GEMM_SPLIT_LAST_ROUNDS): the first ntiles / ctas - 1 rounds (if any) as whole
//   tiles, tile r * ctas + b on CTA b, so the tiles running at one time are neighbours in
//   the list (L2 reuse); the K slices of the remaining tiles (between one and two rounds'
//   worth) are dealt out contiguously and evenly (stream-K).
// sched 2 (GEMM_SPLIT_LAST_ROUND): every full round as whole tiles and only the last,
//   partial round's tiles dealt out along K: the split tiles are few, so the CTAs sharing
//   them read the same operand panels at the same time.
// With sched 1 or 2 every CTA ends within one K slice of the others and the last round
// has no idle SMs.  A tile whose slices are shared by several CTAs is summed from their
// partial slots by the fix-up.
enum { GEMM_WHOLE_TILES = 0, GEMM_SPLIT_LAST_ROUNDS = 1, GEMM_SPLIT_LAST_ROUND = 2 };

inline GemmSchedule gemm_schedule(int ntiles, int nk, int ctas, int sched) {
  GemmSchedule s;
  s.begin.assign(1, 0);
  std::vector<std::vector<int>> parts(ntiles);  // partial slots per tile, in K order
  const int dp_rounds = sched == GEMM_SPLIT_LAST_ROUNDS ? std::max(0, ntiles / ctas - 1)
                        : sched == GEMM_SPLIT_LAST_ROUND ? ntiles / ctas
                                                         : (ntiles + ctas - 1) / ctas;
  const int dp_tiles = std::min(ntiles, dp_rounds * ctas);
  const long long iters = (long long)(ntiles - dp_tiles) * nk;
  for (int b = 0; b < ctas; ++b) {
    for (int t = b; t < dp_tiles; t += ctas) s.segs.push_back({t, 0, nk, -1});
    long long i = iters * b / ctas;
    const long long e = iters * (b + 1) / ctas;
    while (i < e) {
      const int t = dp_tiles + (int)(i / nk);
      const int k0 = (int)(i % nk);
      const int k1 = (int)std::min<long long>(nk, k0 + (e - i));
      int slot = -1;
      if (k0 != 0 || k1 != nk) {
        slot = s.nslots++;
        parts[t].push_back(slot);
      }
      s.segs.push_back({t, k0, k1, slot});
      i += k1 - k0;
    }
    s.begin.push_back((int)s.segs.size());
  }
  s.fix_begin.assign(1, 0);
  for (int t = 0; t < ntiles; ++t)
    if (!parts[t].empty()) {
      s.fix_tile.push_back(t);
      s.fix_slot.insert(s.fix_slot.end(), parts[t].begin(), parts[t].end());
      s.fix_begin.push_back((int)s.fix_slot.size());
    }
  return s;
}

}  // namespace litho
