// Work schedule of the TCC band kernel (band_tcc.cu): task-chunks over the band rows,
// the three column segments of every lane, and the table sizes.  Plain C++ (host and
// device), so the schedule is also checked on the CPU.
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
  int st0, nst;           // the chunk's column steps [st0, st0 + nst)
  int group;
  long long toff;         // first T entry of the chunk
  int size;               // T entries of the chunk
};

LITHO_HD inline int bt_rows(int Ny, int fy) { return 2 * Ny + 1 - fy; }

// task-chunk b = t * nc + c: t < Ny pairs fy = t with 2Ny - t, t = Ny is alone; a
// task's rows are all of its band rows' window rows (py in [fy, 2Ny]), and chunk c takes
// the column steps [S c / nc, S (c + 1) / nc) of the S = 2Nx + 3 (every chunk keeps whole
// row loops; its partial band goes to group c)
LITHO_HD inline BandTask bt_task_shape(int b, int Nx, int Ny, int nc) {
  BandTask d;
  const int t = b / nc, c = b - t * nc, S = 2 * Nx + 3;
  d.nfy = t < Ny ? 2 : 1;
  d.fy[0] = t;
  d.fy[1] = t < Ny ? 2 * Ny - t : -1;
  for (int l = 0; l < 2; ++l) {
    d.py0[l] = l < d.nfy ? d.fy[l] : 0;
    d.npy[l] = l < d.nfy ? bt_rows(Ny, d.fy[l]) : 0;
  }
  d.st0 = S * c / nc;
  d.nst = S * (c + 1) / nc - d.st0;
  d.group = c;
  d.size = (d.npy[0] + d.npy[1]) * d.nst * (2 * Nx);
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

// Lane j's three segments (length, start column of p, start column of q, band column):
// see the header.  Segment 3 of lanes j >= 1 is an idle step (its T entries are zero).
struct BtLane {
  int len1, len2;
  int p1, q1, p2, q2, p3, q3;
  int f1, f2, f3;  // band columns fx; f3 < -2Nx: none
};

LITHO_HD inline BtLane bt_lane(int j, int Nx) {
  BtLane s;
  const int KX = 2 * Nx + 1;
  if (j == 0) {
    s.len1 = 1; s.p1 = 2 * Nx; s.q1 = 0; s.f1 = 2 * Nx;
    s.len2 = 1; s.p2 = 0; s.q2 = 2 * Nx; s.f2 = -2 * Nx;
    s.p3 = 0; s.q3 = 0; s.f3 = 0;
  } else {
    s.len1 = KX - j; s.p1 = j; s.q1 = 0; s.f1 = j;
    s.len2 = j + 1; s.p2 = 0; s.q2 = 2 * Nx - j; s.f2 = j - 2 * Nx;
    s.p3 = 0; s.q3 = 0; s.f3 = -(1 << 20);
  }
  return s;
}

// column step it of lane s: (px, qx, segment 1..3)
LITHO_HD inline void bt_step(const BtLane& s, int it, int* px, int* qx, int* seg) {
  if (it < s.len1) {
    *px = s.p1 + it; *qx = s.q1 + it; *seg = 1;
  } else if (it < s.len1 + s.len2) {
    const int k = it - s.len1;
    *px = s.p2 + k; *qx = s.q2 + k; *seg = 2;
  } else {
    const int k = it - s.len1 - s.len2;
    *px = s.p3 + k; *qx = s.q3 + k; *seg = 3;
  }
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

inline size_t band_tcc_entries(int Nx, int Ny, int nc) {
  size_t n = 0;
  for (int b = 0; b < (Ny + 1) * nc; ++b) n += (size_t)bt_task_shape(b, Nx, Ny, nc).size;
  return n;
}

}  // namespace litho
