"""Work schedule of the TCC band kernel (csrc/band_sched.hpp), compiled with g++ and
checked on the CPU.

The band of an image is band(f) = sum_{p - q = f} W(p) conj(W(q)) T(p, q) over the
(2Ny+1) x (2Nx+1) window, for the rows fy >= 0 the interpolation reads.  The kernel
splits that sum into task-chunks (a pair of band rows fy, 2Ny - fy, or the row Ny
alone, its window rows cut into chunks that write separate partial groups) and, inside
a chunk, into 2Nx lanes that each own a p column and walk the q columns (plus a share of
the last p column).  The schedule must visit every pair (p, q) of every band entry
exactly once, cover every window row of every band row once over the chunks, address
every table entry of a chunk once, and fit a chunk's table in the kernel's
shared-memory budget.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "fpga-litho-accel_gb300", "csrc")

DRIVER = r"""
#include "band_sched.hpp"
#include <cstdio>
#include <map>
#include <tuple>
#include <vector>
using namespace litho;
static int fail(const char* m, int a, int b, int c) { std::printf("fail %s %d %d %d\n", m, a, b, c); return 1; }
static int check(int Nx, int Ny) {
  const int nc = band_tcc_chunks(Nx, Ny);
  if (nc <= 0) return fail("no chunking", Nx, Ny, nc);
  const int KX = 2 * Nx + 1, KY = 2 * Ny + 1, NL = 2 * Nx, NS = bt_slots(Nx);
  std::map<std::tuple<int, int, int, int, int, int>, int> seen;  // (fy, fx, py, px, qy, qx)
  std::vector<int> rows_seen(KY * KY, 0);                        // (fy, py) covered once over chunks
  long long off = 0;
  for (int b = 0; b < (Ny + 1) * nc; ++b) {
    const BandTask d = bt_task(b, Nx, Ny, nc);
    if (d.toff != off) return fail("table offset", b, (int)d.toff, (int)off);
    off += d.size;
    if ((size_t)d.size * 8 > BT_TAB_BUDGET) return fail("chunk over budget", b, d.size, 0);
    if (d.size % 2) return fail("odd chunk (16-byte copies)", b, d.size, 0);
    if (d.group != b % nc) return fail("group", b, d.group, 0);
    std::vector<int> used(d.size, 0);
    for (int l = 0; l < d.nfy; ++l) {
      const int fy = d.fy[l];
      if (fy < 0 || fy > 2 * Ny) return fail("band row", b, l, fy);
      if (d.npy[l] < 0 || d.py0[l] < fy || d.py0[l] + d.npy[l] > KY) return fail("rows", b, l, d.py0[l]);
      for (int r = 0; r < d.npy[l]; ++r) {
        const int py = d.py0[l] + r, qy = py - fy;
        rows_seen[fy * KY + py]++;
        for (int s = 0; s < NS; ++s)
          for (int j = 0; j < NL; ++j) {
            const int e = bt_entry(d, l, r, s, j, Nx);
            if (e < 0 || e >= d.size || used[e]++) return fail("table entry", b, e, d.size);
            int px, qx;
            if (!bt_slot(j, s, Nx, &px, &qx)) continue;
            if (px < 0 || px >= KX || qx < 0 || qx >= KX) return fail("column range", j, s, px);
            seen[std::make_tuple(fy, px - qx, py, px, qy, qx)]++;
          }
      }
    }
    for (int e = 0; e < d.size; ++e)
      if (used[e] != 1) return fail("table hole", b, e, used[e]);
  }
  if ((size_t)off != band_tcc_entries(Nx, Ny, nc)) return fail("table size", (int)off, 0, 0);
  for (int fy = 0; fy <= 2 * Ny; ++fy)
    for (int py = 0; py < KY; ++py)
      if (rows_seen[fy * KY + py] != (py >= fy ? 1 : 0)) return fail("window row", fy, py, rows_seen[fy * KY + py]);
  // every pair of every band entry once
  size_t want = 0;
  for (int fy = 0; fy <= 2 * Ny; ++fy)
    for (int fx = -2 * Nx; fx <= 2 * Nx; ++fx)
      for (int py = fy; py < KY; ++py)
        for (int px = std::max(0, fx); px < KX + std::min(0, fx); ++px) {
          ++want;
          auto it = seen.find(std::make_tuple(fy, fx, py, px, py - fy, px - fx));
          if (it == seen.end() || it->second != 1) return fail("pair", fy, fx, py * KX + px);
        }
  if (want != seen.size()) return fail("extra pairs", (int)want, (int)seen.size(), 0);
  std::printf("ok %d %zu\n", nc, want);
  return 0;
}
int main(int argc, char** argv) {
  int Nx, Ny;
  if (argc > 1) {  // band cost model: "Nx Ny nk convN batch" -> 1 where the TCC form is cheaper
    int nk, convN, batch;
    while (std::scanf("%d %d %d %d %d", &Nx, &Ny, &nk, &convN, &batch) == 5)
      std::printf("%d\n", band_tcc_cost_us(Nx, Ny, band_tcc_chunks(Nx, Ny), batch) <=
                               band_fft_cost_us(convN, nk, batch) ? 1 : 0);
    return 0;
  }
  while (std::scanf("%d %d", &Nx, &Ny) == 2)
    if (check(Nx, Ny)) return 1;
  return 0;
}
"""

# (Nx, Ny): the metric's 1024^2 optics (8, 8), the 2048^2 class (16, 16), the small
# configurations, rectangular windows and the edges of the supported range
CASES = [(8, 8), (16, 16), (2, 2), (1, 0), (1, 1), (4, 7), (7, 4), (12, 12), (16, 3), (3, 16), (5, 5), (9, 13)]


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("band_sched")
    src, exe = d / "drv.cpp", d / "drv"
    src.write_text(DRIVER)
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    return str(exe)


def test_schedule_visits_every_pair_once(driver):
    inp = "".join(f"{nx} {ny}\n" for nx, ny in CASES)
    r = subprocess.run([driver], input=inp, capture_output=True, text=True)
    lines = r.stdout.split("\n")
    assert r.returncode == 0, r.stdout
    got = [ln.split() for ln in lines if ln]
    assert len(got) == len(CASES)
    for (nx, ny), g in zip(CASES, got):
        assert g[0] == "ok"
        kx, ky = 2 * nx + 1, 2 * ny + 1
        # pairs with fy >= 0: sum over fy of (rows) x sum over fx of (diagonal length)
        assert int(g[2]) == (ky * (ky + 1) // 2) * kx * kx, (nx, ny)


def test_chunking_of_the_metric_optics(driver):
    # a chunk's table shares shared memory with a window per image of every warp: at
    # Nx = Ny = 8 a whole task fits (one partial group), at Nx = Ny = 16 the tasks'
    # window rows are cut into chunks
    r = subprocess.run([driver], input="8 8\n16 16\n", capture_output=True, text=True)
    (a, b) = [ln.split() for ln in r.stdout.split("\n") if ln]
    assert a[1] == "1"
    assert 2 < int(b[1]) <= 16


def _conv(nx, ny):
    n = 32
    while n < 4 * max(nx, ny) + 1:
        n *= 2
    return n


def test_auto_band_cost_model(driver):
    # (Nx, K, masks) -> TCC form expected faster, from band-stage timings on GB300 (mixed
    # form, 1024^2 masks): TCC 23.5 / FFT 50.3 us at Nx = 8, K = 24, 256 masks; 50.8 / 51.3
    # at Nx = 10; 87.4 / 53.5 at Nx = 12; 205 / 55.4 at Nx = 15; 236 / 287 at Nx = 16 (FFT on the
    # 128 grid); 236 / 121 at Nx = 16, K = 8; 23 / 88 at Nx = 8, K = 48; 43 / 143 at Nx = 8,
    # K = 24, 1024 masks; 24.0 / 20.9 at Nx = 8, K = 24, 64 masks
    cases = [((8, 24, 256), 1), ((12, 24, 256), 0), ((15, 24, 256), 0), ((16, 24, 256), 1),
             ((16, 8, 256), 0), ((8, 48, 256), 1), ((8, 24, 1024), 1), ((8, 24, 64), 0),
             ((12, 48, 256), 1), ((4, 24, 256), 1)]
    inp = "".join(f"{nx} {nx} {k} {_conv(nx, nx)} {b}\n" for (nx, k, b), _ in cases)
    r = subprocess.run([driver, "model"], input=inp, capture_output=True, text=True, check=True)
    got = [int(x) for x in r.stdout.split()]
    assert got == [w for _, w in cases], list(zip([c for c, _ in cases], got))
