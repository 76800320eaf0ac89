"""Output tiles of the split-BF16 TCC product (csrc/tcc_tiles.hpp), compiled with g++
and checked on the CPU.  The product C = [X; Y] X^T (2n x n) is computed only on the
128 x 128 tiles the TCC assembly reads: C[a][b] with a <= b (real part) and C[n + a][b]
with a < b (imaginary part).  The list must hold exactly the tiles that contain such an
entry, once each, in 12 x 12 blocks; at n = 3025 (Nx = 27) that is 623 of 1,152."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "fpga-litho-accel_gb300", "csrc")

DRIVER = r"""
#include "tcc_tiles.hpp"
#include <cstdio>
int main() {
  int n;
  while (std::scanf("%d", &n) == 1) {
    const std::vector<litho::TileMN> t = litho::tcc_needed_tiles(n);
    std::printf("%zu", t.size());
    for (const litho::TileMN& x : t) std::printf(" %d %d", x.m, x.n);
    std::printf("\n");
  }
  return 0;
}
"""

# TCC sizes (2Nx+1)^2 of the configurations in use, plus tile-boundary cases
SIZES = [1, 2, 3, 25, 81, 127, 128, 129, 255, 256, 257, 289, 300, 1089, 1536, 1537, 3025]


@pytest.fixture(scope="module")
def tile_lists(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("tcc_tiles")
    src, exe = d / "drv.cpp", d / "drv"
    src.write_text(DRIVER)
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], input="".join(f"{n}\n" for n in SIZES), capture_output=True, text=True,
                         check=True).stdout.splitlines()
    assert len(out) == len(SIZES)
    res = {}
    for n, line in zip(SIZES, out):
        v = [int(x) for x in line.split()]
        assert len(v) == 1 + 2 * v[0]
        res[n] = [(v[1 + 2 * i], v[2 + 2 * i]) for i in range(v[0])]
    return res


def _read_tiles(n):
    """Tiles (row tile, column tile) holding an entry the TCC assembly reads."""
    a = np.arange(n)
    upper = a[:, None] <= a[None, :]          # C[a][b], a <= b
    strict = a[:, None] < a[None, :]          # C[n + a][b], a < b
    need = np.concatenate([upper, strict], axis=0)  # 2n x n
    MT, NT = (2 * n + 127) // 128, (n + 127) // 128
    pad = np.zeros((MT * 128, NT * 128), bool)
    pad[:2 * n, :n] = need
    t = pad.reshape(MT, 128, NT, 128).any(axis=(1, 3))
    return {(int(m), int(c)) for m, c in zip(*np.nonzero(t))}


def test_tiles_exactly_cover_the_read_entries(tile_lists):
    for n, tiles in tile_lists.items():
        assert len(set(tiles)) == len(tiles), n
        assert set(tiles) == _read_tiles(n), n


def test_tiles_come_in_12x12_blocks(tile_lists):
    for n, tiles in tile_lists.items():
        keys = [(m // 12, c // 12, m, c) for m, c in tiles]
        assert keys == sorted(keys), n


def test_large_tcc_tile_count(tile_lists):
    n = 3025
    assert len(tile_lists[n]) == 623
    assert ((2 * n + 127) // 128) * ((n + 127) // 128) == 1152
