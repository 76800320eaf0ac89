// Tiles of one mixed window-DFT launch over up to WIN_MAX_SIZES mask sizes (imaging_tc.cu,
// win_dft_tc_kernel): per size its width, 128-row blocks, column splits, first image in the
// shared partial array and first tile; tiles are numbered size after size, then image, row
// block and column split.  Plain C++ (host and device), so the numbering is also checked on
// the CPU.
#pragma once

#ifdef __CUDACC__
#define LITHO_WT_HD __host__ __device__
#else
#define LITHO_WT_HD
#endif

namespace litho {

constexpr int WIN_MAX_SIZES = 4;  // mask sizes one window launch takes

struct WinTiles {
  int n;                              // mask sizes
  int Lx[WIN_MAX_SIZES];              // mask width
  int rows[WIN_MAX_SIZES];            // 128-row blocks
  int ncs[WIN_MAX_SIZES];             // column splits
  int img0[WIN_MAX_SIZES];            // first image in the partial array
  int tile0[WIN_MAX_SIZES + 1];       // first tile (tile0[n]: all tiles)
};

// tile t -> (size g, image, row block, column split) and its range [c0, c1) of column chunks
// of `chunk` columns
LITHO_WT_HD inline void win_tile(const WinTiles& T, int t, int chunk, int& g, int& img, int& rb, int& cs, int& c0,
                                 int& c1) {
  g = 0;
  while (g + 1 < T.n && t >= T.tile0[g + 1]) ++g;
  const int l = t - T.tile0[g], rows = T.rows[g], ncs = T.ncs[g];
  const int nch = (T.Lx[g] + chunk - 1) / chunk;
  img = l / (rows * ncs);
  const int r = l - img * rows * ncs;
  rb = r / ncs;
  cs = r - rb * ncs;
  c0 = (int)((long long)nch * cs / ncs);
  c1 = (int)((long long)nch * (cs + 1) / ncs);
}

}  // namespace litho
