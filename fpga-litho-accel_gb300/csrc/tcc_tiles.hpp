// Output tiles of the split-BF16 TCC product that the TCC assembly reads.  Plain
// C++ with no CUDA, so the tile list is also checked on the CPU.
#pragma once
#include <algorithm>
#include <vector>

namespace litho {

struct TileMN {
  int m, n;  // 128-row tile index (of 2n rows), 128-column tile index (of n columns)
};

// C = A A_top^T with A = [X; Y] (2n rows): rows < n hold X X^T (the real part,
// symmetric), rows >= n hold Y X^T (the imaginary part, antisymmetric).  The TCC
// reads C[a][b] with a <= b and C[n + a][b] with a < b, so only the 128 x 128
// tiles that hold such entries are listed (about half), in 12 x 12 blocks of
// tiles that share their A and B panels in L2.
inline std::vector<TileMN> tcc_needed_tiles(int n) {
  const int MT = (2 * n + 127) / 128, NT = (n + 127) / 128;
  std::vector<TileMN> tiles;
  for (int mb = 0; mb < MT; mb += 12)
    for (int nb = 0; nb < NT; nb += 12)
      for (int mt = mb; mt < std::min(MT, mb + 12); ++mt)
        for (int nt = nb; nt < std::min(NT, nb + 12); ++nt) {
          const int r0 = mt * 128, r1 = std::min(r0 + 128, 2 * n);
          const int cmax = std::min(nt * 128 + 127, n - 1);
          const bool top = r0 < n && r0 <= cmax;                      // some a <= b with a < n
          const bool bottom = r1 > n && std::max(r0, n) - n < cmax;  // some n + a with a < b
          if (top || bottom) tiles.push_back({mt, nt});
        }
  return tiles;
}

}  // namespace litho
