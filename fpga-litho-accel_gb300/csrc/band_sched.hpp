// Work schedule of the TCC band kernel (band_tcc.cu): task-chunks over the band rows,
// the column slots of every lane, and the table sizes.  Plain C++ (host and device),
// so the schedule is also checked on the CPU.
//
// For one band row fy, the pairs (p, q) with p - q = (fy, fx) are, for every window row
// py in [fy, 2Ny] (q row py - fy), the pairs of columns (px, qx) with px - qx = fx.  Lane
// j of an image (2Nx lanes) owns the p column px = j: in slot s < 2Nx+1 it takes q column
// qx = s (band column j - s).  The last p column, px = 2Nx, is shared out: in slot 2Nx+1
// lane j takes (2Nx, j) (band column 2Nx - j), and in slot 2Nx+2 lane 0 takes (2Nx, 2Nx)
// (band column 0; the other lanes idle there).  So every lane runs the same 2Nx+3 slots
// per window row, with its p value fixed along them.
#pragma once
#include <algorithm>
#include <cstddef>

#ifdef __CUDACC__
#define LITHO_HD __host__ __device__
#else
#define LITHO_HD
#endif

namespace litho {

// T bytes of one task-chunk: the kernel holds it in shared memory beside one window per
// image of every warp, and two CTAs should fit an SM at Nx = Ny = 8 (one chunk per task)
constexpr size_t BT_TAB_BUDGET = 48 * 1024;
constexpr int BT_MAX_CHUNKS = 16;

struct BandTask {
  int nfy;                // 1 or 2 rows of the band
  int fy[2], py0[2], npy[2];
  int group;
  long long toff;         // first T entry of the chunk
  int size;               // T entries of the chunk
};

LITHO_HD inline int bt_rows(int Ny, int fy) { return 2 * Ny + 1 - fy; }
LITHO_HD inline int bt_slots(int Nx) { return 2 * Nx + 3; }

// task-chunk b = t * nc + c: t < Ny pairs fy = t with 2Ny - t, t = Ny is alone; chunk c
// takes the window rows [R c / nc, R (c + 1) / nc) of the task's R = rows(fy0) + rows(fy1)
// (fy0's rows first); its partial band goes to group c
LITHO_HD inline BandTask bt_task_shape(int b, int Nx, int Ny, int nc) {
  BandTask d;
  const int t = b / nc, c = b - t * nc;
  d.nfy = t < Ny ? 2 : 1;
  d.fy[0] = t;
  d.fy[1] = t < Ny ? 2 * Ny - t : -1;
  const int R0 = bt_rows(Ny, d.fy[0]), R1 = d.nfy == 2 ? bt_rows(Ny, d.fy[1]) : 0, R = R0 + R1;
  const int r0 = R * c / nc, r1 = R * (c + 1) / nc;
  // rows [r0, r1) of the concatenation: fy0's part, then fy1's
  const int a0 = r0 < R0 ? r0 : R0, b0 = r1 < R0 ? r1 : R0;
  const int a1 = (r0 > R0 ? r0 : R0) - R0, b1 = (r1 > R0 ? r1 : R0) - R0;
  d.py0[0] = d.fy[0] + a0;
  d.npy[0] = b0 - a0;
  d.py0[1] = d.nfy == 2 ? d.fy[1] + a1 : 0;
  d.npy[1] = d.nfy == 2 ? b1 - a1 : 0;
  d.group = c;
  d.size = (d.npy[0] + d.npy[1]) * bt_slots(Nx) * (2 * Nx);
  d.toff = 0;
  return d;
}

LITHO_HD inline BandTask bt_task(int b, int Nx, int Ny, int nc) {
  long long off = 0;
  for (int i = 0; i < b; ++i) off += bt_task_shape(i, Nx, Ny, nc).size;
  BandTask d = bt_task_shape(b, Nx, Ny, nc);
  d.toff = off;
  return d;
}

// Slot s of lane j: the p and q columns, and whether the slot carries a pair (in the
// last slot lane 0 alone does).  Its band column is px - qx.
LITHO_HD inline bool bt_slot(int j, int s, int Nx, int* px, int* qx) {
  const int KX = 2 * Nx + 1;
  if (s < KX) {
    *px = j;
    *qx = s;
    return true;
  }
  *px = 2 * Nx;
  *qx = s == KX ? j : 2 * Nx;
  return s == KX || j == 0;
}

// T entry of (band row l of the task, row r of the chunk's rows of l, slot s, lane j)
LITHO_HD inline int bt_entry(const BandTask& d, int l, int r, int s, int j, int Nx) {
  const int NS = bt_slots(Nx), NL = 2 * Nx;
  return ((l ? d.npy[0] : 0) + r) * NS * NL + s * NL + j;
}

inline int band_tcc_chunks(int Nx, int Ny) {
  if (Nx < 1 || Nx > 16 || Ny < 0 || Ny > 16) return 0;
  for (int nc = 1; nc <= BT_MAX_CHUNKS; ++nc) {
    int most = 0;
    for (int b = 0; b < (Ny + 1) * nc; ++b) most = std::max(most, bt_task_shape(b, Nx, Ny, nc).size);
    if ((size_t)most * 2 * sizeof(float) <= BT_TAB_BUDGET) return nc;  // complex FP32 entries
  }
  return 0;
}

// Expected band-stage time (us) of each form for `batch` images of a kernel set, fitted to
// GB300 measurements (1024^2 and 512^2 masks, K = 8 / 24 / 48, 64-1024 images; mixed form).
// The TCC form costs ~20 us (28 when its table is cut into chunks) plus 0.6 ps (1.1 ps) per
// window pair (p, q) with fy >= 0 and image; the FFT form ~10 us (29 on the 128 grid) plus
// 4.2 / 6.8 / 42 ns per kernel and image on the 32 / 64 / 128 conv grids.  LITHO_BAND_AUTO
// takes the TCC form where it is expected to be faster: at K = 24 and 256 masks for
// Nx = Ny <= 10 and at 16 (where the FFT form needs the 128 grid), not for 11..15.
inline double band_tcc_cost_us(int Nx, int Ny, int nc, int batch) {
  const double KX = 2 * Nx + 1, KY = 2 * Ny + 1, pairs = KY * (KY + 1) / 2 * KX * KX;
  return nc > 1 ? 28.0 + 1.1e-6 * pairs * batch : 20.0 + 0.6e-6 * pairs * batch;
}
inline double band_fft_cost_us(int convN, int nk, int batch) {
  const double per = convN <= 32 ? 4.2e-3 : convN <= 64 ? 6.8e-3 : 42e-3;
  return (convN >= 128 ? 29.0 : 10.0) + per * nk * batch;
}

inline size_t band_tcc_entries(int Nx, int Ny, int nc) {
  size_t n = 0;
  for (int b = 0; b < (Ny + 1) * nc; ++b) n += (size_t)bt_task_shape(b, Nx, Ny, nc).size;
  return n;
}

}  // namespace litho
