"""Chunk schedule of the host-buffer imaging path (csrc/host_chunks.hpp), compiled with
g++ and checked on the CPU.  litho_image_batch with host pointers copies masks in and
images out chunk by chunk; the schedule must cover the batch exactly, keep every chunk
within the staging slot (1..CH masks, CH from the chunk byte cap, 128 MB unless the
context sets another), and ramp 1, 2, 4, ... up and back down only while a full chunk
stays in the middle."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "fpga-litho-accel_gb300", "csrc")

DRIVER = r"""
#include "host_chunks.hpp"
#include <cstdio>
int main() {
  int batch;
  long long img, cap;
  while (std::scanf("%d %lld %lld", &batch, &img, &cap) == 3) {
    const int ch = cap ? litho::host_chunk_masks(batch, (size_t)img, (size_t)cap)
                       : litho::host_chunk_masks(batch, (size_t)img);
    std::vector<int> s;
    litho::chunk_schedule(batch, ch, s);
    std::printf("%d", ch);
    for (int v : s) std::printf(" %d", v);
    std::printf("\n");
  }
  return 0;
}
"""

MIB = 1 << 20
IMG_BYTES = [256 * 256 * 4, 512 * 512 * 4, 4 * MIB, 16 * MIB, 64 * MIB, 256 * MIB]
CAPS = [0, 16 * MIB, 3 * MIB]  # 0: the default (128 MB)
BATCHES = list(range(0, 70)) + [97, 128, 255, 256, 257, 384, 1000, 4096]


@pytest.fixture(scope="module")
def schedules(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("chunks")
    src, exe = d / "drv.cpp", d / "drv"
    src.write_text(DRIVER)
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    cases = [(b, i, c) for c in CAPS for i in IMG_BYTES for b in BATCHES]
    out = subprocess.run([str(exe)], input="".join(f"{b} {i} {c}\n" for b, i, c in cases), capture_output=True,
                         text=True, check=True).stdout.splitlines()
    assert len(out) == len(cases)
    res = {}
    for (b, i, c), line in zip(cases, out):
        v = [int(x) for x in line.split()]
        res[(b, i, c)] = (v[0], v[1:])
    return res


def _ramp(sizes):
    r = []
    for k, s in enumerate(sizes):
        if s != 1 << k:
            break
        r.append(s)
    return r


def test_chunk_size_rule(schedules):
    for (b, img, cap), (ch, _) in schedules.items():
        want = max(1, min((cap or 128 * MIB) // img, (b + 7) // 8))
        assert ch == want, (b, img, cap)


def test_schedule_covers_batch(schedules):
    for (b, img, cap), (ch, sizes) in schedules.items():
        assert sum(sizes) == b, (b, img, cap)
        assert all(1 <= s <= ch for s in sizes), (b, img, cap, sizes)


def test_ramp_is_mirrored_and_leaves_a_full_middle(schedules):
    for (b, img, cap), (ch, sizes) in schedules.items():
        ramp = [r for r in _ramp(sizes) if r < ch]
        n = len(ramp)
        if n:
            assert sizes[-n:] == ramp[::-1], (b, img, sizes)
            middle = sizes[n:-n]
            assert middle and middle[0] == ch, (b, img, sizes)
            assert b - 2 * sum(ramp) >= ch
        # a further ramp step was possible only if it would still leave a full chunk
        nxt = 1 << n
        if nxt < ch:
            assert 2 * (sum(ramp) + nxt) + ch > b, (b, img, sizes)


def test_known_schedules(schedules):
    # 256 masks of 1024^2 float32 at the default 128 MB: 32 masks per chunk, ramp 1..16
    ch, sizes = schedules[(256, 4 * MIB, 0)]
    assert ch == 32
    assert sizes == [1, 2, 4, 8, 16] + [32] * 6 + [2] + [16, 8, 4, 2, 1]
    # at 16 MB: four masks per chunk, ramp 1, 2
    ch, sizes = schedules[(256, 4 * MIB, 16 * MIB)]
    assert ch == 4
    assert sizes == [1, 2] + [4] * 62 + [2] + [2, 1]
    # 2048^2 masks: eight per chunk by default, one at 16 MB (no ramp)
    assert schedules[(64, 16 * MIB, 0)] == (8, [1, 2, 4] + [8] * 6 + [2] + [4, 2, 1])
    assert schedules[(64, 16 * MIB, 16 * MIB)] == (1, [1] * 64)
    # masks larger than the chunk still move one at a time
    assert schedules[(5, 256 * MIB, 0)] == (1, [1] * 5)
    # an empty batch has no chunks
    assert schedules[(0, 4 * MIB, 0)] == (1, [])
