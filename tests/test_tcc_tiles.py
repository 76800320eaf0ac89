"""Output tiles of the split-BF16 TCC product and the persistent GEMM's schedule
(csrc/tcc_tiles.hpp), compiled with g++ and checked on the CPU.

The product C = [X; Y] X^T (2n x n) is computed only on the 128 x bn tiles the TCC
assembly reads: C[a][b] with a <= b (real part) and C[n + a][b] with a < b (imaginary
part).  The list must hold exactly the tiles that contain such an entry, once each, in
blocks; at n = 3025 (Nx = 27) and bn = 128 that is 623 of 1,152.

The schedule hands every (tile, K slice) to exactly one persistent CTA: whole tiles in
data-parallel rounds, and with a split schedule (1: the last one or two rounds, 2: the last
partial round) the remaining tiles' K slices dealt out evenly; a tile shared by several CTAs
is summed from partial slots listed in K order."""
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
  int n, bn;
  while (std::scanf("%d %d", &n, &bn) == 2) {
    const std::vector<litho::TileMN> t = litho::tcc_needed_tiles(n, bn);
    std::printf("%zu", t.size());
    for (const litho::TileMN& x : t) std::printf(" %d %d", x.m, x.n);
    std::printf("\n");
  }
  return 0;
}
"""

SCHED_DRIVER = r"""
#include "tcc_tiles.hpp"
#include <cstdio>
int main() {
  int T, nk, ctas, split;
  while (std::scanf("%d %d %d %d", &T, &nk, &ctas, &split) == 4) {
    const litho::GemmSchedule s = litho::gemm_schedule(T, nk, ctas, split);
    std::printf("%d %zu %zu %zu", s.nslots, s.begin.size(), s.segs.size(), s.fix_tile.size());
    for (int v : s.begin) std::printf(" %d", v);
    for (const litho::GemmSeg& g : s.segs) std::printf(" %d %d %d %d", g.tile, g.k0, g.k1, g.slot);
    for (int v : s.fix_tile) std::printf(" %d", v);
    for (int v : s.fix_begin) std::printf(" %d", v);
    std::printf(" %zu", s.fix_slot.size());
    for (int v : s.fix_slot) std::printf(" %d", v);
    std::printf("\n");
  }
  return 0;
}
"""

# TCC sizes (2Nx+1)^2 of the configurations in use, plus tile-boundary cases
SIZES = [1, 2, 3, 25, 81, 127, 128, 129, 255, 256, 257, 289, 300, 1089, 1536, 1537, 3025]


BNS = [64, 128, 256]


def _build(tmp_path_factory, name, text):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp(name)
    src, exe = d / "drv.cpp", d / "drv"
    src.write_text(text)
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    return exe


@pytest.fixture(scope="module")
def tile_lists(tmp_path_factory):
    exe = _build(tmp_path_factory, "tcc_tiles", DRIVER)
    cases = [(n, bn) for bn in BNS for n in SIZES]
    out = subprocess.run([str(exe)], input="".join(f"{n} {bn}\n" for n, bn in cases), capture_output=True,
                         text=True, check=True).stdout.splitlines()
    assert len(out) == len(cases)
    res = {}
    for key, line in zip(cases, out):
        v = [int(x) for x in line.split()]
        assert len(v) == 1 + 2 * v[0]
        res[key] = [(v[1 + 2 * i], v[2 + 2 * i]) for i in range(v[0])]
    return res


def _read_tiles(n, bn):
    """Tiles (row tile, column tile) holding an entry the TCC assembly reads."""
    a = np.arange(n)
    upper = a[:, None] <= a[None, :]          # C[a][b], a <= b
    strict = a[:, None] < a[None, :]          # C[n + a][b], a < b
    need = np.concatenate([upper, strict], axis=0)  # 2n x n
    MT, NT = (2 * n + 127) // 128, (n + bn - 1) // bn
    pad = np.zeros((MT * 128, NT * bn), bool)
    pad[:2 * n, :n] = need
    t = pad.reshape(MT, 128, NT, bn).any(axis=(1, 3))
    return {(int(m), int(c)) for m, c in zip(*np.nonzero(t))}


def test_tiles_exactly_cover_the_read_entries(tile_lists):
    for (n, bn), tiles in tile_lists.items():
        assert len(set(tiles)) == len(tiles), (n, bn)
        assert set(tiles) == _read_tiles(n, bn), (n, bn)


def test_tiles_come_in_blocks(tile_lists):
    for (n, bn), tiles in tile_lists.items():
        nb = max(1, 12 * 128 // bn)
        keys = [(m // 12, c // nb, m, c) for m, c in tiles]
        assert keys == sorted(keys), (n, bn)


def test_large_tcc_tile_count(tile_lists):
    n = 3025
    assert len(tile_lists[(n, 128)]) == 623
    assert ((2 * n + 127) // 128) * ((n + 127) // 128) == 1152


# (tiles, K slices, CTAs): the large TCC at each tile width (623 / 1,241 / 317 tiles of 127 slices
# on 152 SMs), the 1024^2 workload's TCC (n = 289, 62 slices), fewer tiles than CTAs, one slice
SCHED_CASES = [(623, 127, 152), (1241, 127, 152), (317, 127, 152), (10, 62, 152), (7, 3, 152), (152, 5, 152),
               (153, 5, 152), (304, 9, 152), (1, 1, 1), (5, 1, 8), (40, 7, 3)]


@pytest.fixture(scope="module")
def schedules(tmp_path_factory):
    exe = _build(tmp_path_factory, "gemm_sched", SCHED_DRIVER)
    cases = [(T, nk, c, sp) for T, nk, c in SCHED_CASES for sp in (0, 1, 2)]
    out = subprocess.run([str(exe)], input="".join(f"{T} {nk} {c} {sp}\n" for T, nk, c, sp in cases),
                         capture_output=True, text=True, check=True).stdout.splitlines()
    assert len(out) == len(cases)
    res = {}
    for key, line in zip(cases, out):
        v = [int(x) for x in line.split()]
        nslots, nbeg, nseg, nfix = v[:4]
        p = 4
        begin = v[p:p + nbeg]
        p += nbeg
        segs = [tuple(v[p + 4 * i:p + 4 * i + 4]) for i in range(nseg)]
        p += 4 * nseg
        fix_tile = v[p:p + nfix]
        p += nfix
        fix_begin = v[p:p + nfix + 1]
        p += nfix + 1
        nfs = v[p]
        fix_slot = v[p + 1:p + 1 + nfs]
        assert p + 1 + nfs == len(v)
        res[key] = dict(nslots=nslots, begin=begin, segs=segs, fix_tile=fix_tile, fix_begin=fix_begin,
                        fix_slot=fix_slot)
    return res


def test_schedule_covers_every_slice_once(schedules):
    for (T, nk, ctas, sp), s in schedules.items():
        assert len(s["begin"]) == ctas + 1 and s["begin"][0] == 0 and s["begin"][-1] == len(s["segs"])
        assert all(a <= b for a, b in zip(s["begin"], s["begin"][1:]))
        cover = np.zeros((T, nk), int)
        for t, k0, k1, slot in s["segs"]:
            assert 0 <= t < T and 0 <= k0 < k1 <= nk
            cover[t, k0:k1] += 1
            assert (slot < 0) == (k0 == 0 and k1 == nk)
        assert (cover == 1).all(), (T, nk, ctas, sp)


def test_schedule_partial_slots_and_fixups(schedules):
    for key, s in schedules.items():
        slots = [g[3] for g in s["segs"] if g[3] >= 0]
        assert sorted(slots) == list(range(s["nslots"])), key
        seg_of = {g[3]: g for g in s["segs"] if g[3] >= 0}
        assert len(s["fix_begin"]) == len(s["fix_tile"]) + 1 and s["fix_begin"][-1] == len(s["fix_slot"])
        assert sorted(s["fix_slot"]) == list(range(s["nslots"]))
        for f, t in enumerate(s["fix_tile"]):
            parts = [seg_of[j] for j in s["fix_slot"][s["fix_begin"][f]:s["fix_begin"][f + 1]]]
            assert all(p[0] == t for p in parts)
            # in K order and contiguous from 0 to nk: the fix-up's summation order is the K order
            assert parts[0][1] == 0 and parts[-1][2] == key[1]
            assert all(a[2] == b[1] for a, b in zip(parts, parts[1:]))


def test_schedule_balance(schedules):
    for (T, nk, ctas, sp), s in schedules.items():
        load = [sum(g[2] - g[1] for g in s["segs"][s["begin"][b]:s["begin"][b + 1]]) for b in range(ctas)]
        if sp:
            # every CTA ends within one K slice of the others
            assert max(load) - min(load) <= 1, (T, nk, ctas)
        else:
            # whole tiles, tile t on CTA t % ctas
            assert all(g[3] < 0 for g in s["segs"])
            for b in range(ctas):
                assert [g[0] for g in s["segs"][s["begin"][b]:s["begin"][b + 1]]] == list(range(b, T, ctas))


def test_schedule_data_parallel_rounds_come_first(schedules):
    for (T, nk, ctas, sp), s in schedules.items():
        if not sp:
            continue
        rounds = max(0, T // ctas - 1) if sp == 1 else T // ctas
        for b in range(ctas):
            segs = s["segs"][s["begin"][b]:s["begin"][b + 1]]
            whole = [g[0] for g in segs[:rounds]]
            assert whole == [b + r * ctas for r in range(rounds)]
