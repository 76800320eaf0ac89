"""Tile numbering of the mixed window DFT over several mask sizes (csrc/win_tiles.hpp),
compiled with g++ and checked on the CPU.

One launch covers up to four mask sizes of a batch class.  Its tiles, numbered size after
size, must cover every (size, image, 128-row block, 64-column chunk) exactly once, with the
image inside its size's batch and the chunk range of each tile inside the mask width.
"""
import os
import random
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "fpga-litho-accel_gb300", "csrc")

DRIVER = r"""
#include "win_tiles.hpp"
#include <cstdio>
#include <map>
#include <tuple>
using namespace litho;
int main() {
  int n;
  const int chunk = 64;
  while (std::scanf("%d", &n) == 1) {
    WinTiles T{};
    T.n = n;
    int batch[WIN_MAX_SIZES], tiles = 0, img0 = 0;
    for (int g = 0; g < n; ++g) {
      int Lx, Ly, b, ncs;
      if (std::scanf("%d %d %d %d", &Lx, &Ly, &b, &ncs) != 4) return 2;
      T.Lx[g] = Lx;
      T.rows[g] = (Ly + 127) / 128;
      T.ncs[g] = ncs;
      T.img0[g] = img0;
      T.tile0[g] = tiles;
      batch[g] = b;
      img0 += b;
      tiles += T.rows[g] * b * ncs;
    }
    T.tile0[n] = tiles;
    std::map<std::tuple<int, int, int, int>, int> seen;
    for (int t = 0; t < tiles; ++t) {
      int g, img, rb, cs, c0, c1;
      win_tile(T, t, chunk, g, img, rb, cs, c0, c1);
      const int nch = (T.Lx[g] + chunk - 1) / chunk;
      if (g < 0 || g >= n || img < 0 || img >= batch[g] || rb < 0 || rb >= T.rows[g] || cs < 0 || cs >= T.ncs[g] ||
          c0 < 0 || c1 > nch || c0 > c1) {
        std::printf("range %d %d %d %d %d %d %d\n", t, g, img, rb, cs, c0, c1);
        return 1;
      }
      for (int c = c0; c < c1; ++c) seen[std::make_tuple(g, img, rb, c)]++;
    }
    size_t want = 0;
    for (int g = 0; g < n; ++g) want += (size_t)batch[g] * T.rows[g] * ((T.Lx[g] + chunk - 1) / chunk);
    if (seen.size() != want) { std::printf("coverage %zu %zu\n", seen.size(), want); return 1; }
    for (auto& kv : seen)
      if (kv.second != 1) { std::printf("twice\n"); return 1; }
  }
  std::printf("ok\n");
  return 0;
}
"""


def test_tiles_cover_every_chunk_once(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src, exe = tmp_path / "drv.cpp", tmp_path / "drv"
    src.write_text(DRIVER)
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    rng = random.Random(7)
    cases = ["4 1024 1024 62 1 768 768 52 1 512 512 49 1 256 256 49 1",   # the bench's 1024 class
             "1 2048 2048 44 1", "1 2048 2048 44 3", "2 96 64 3 2 40 300 5 1"]
    for _ in range(200):
        n = rng.randint(1, 4)
        parts = []
        for _ in range(n):
            lx = 4 * rng.randint(1, 512)
            nch = (lx + 63) // 64
            parts.append(f"{lx} {rng.randint(2, 2048)} {rng.randint(1, 9)} {rng.randint(1, max(1, min(4, nch)))}")
        cases.append(f"{n} " + " ".join(parts))
    r = subprocess.run([str(exe)], input="\n".join(cases) + "\n", capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout
