"""Row pairing of the FP32 interpolation kernel (csrc/fi_mirror.hpp), compiled with g++ and
checked on the CPU.

The kernel forms A (the cos rows of Tm) and B (the sin rows) once per base row b and
writes A + B to the image row with centred coordinate y' = +b and A - B to y' = -b, with
y' = Y + (Fy - Ly)/2 - Fy/2 as in FT_r2c_padded's centring (litho.cpp:242-318).  Over the
base rows 0 .. nbase-1 every image row must be written exactly once, at its own y'.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "fpga-litho-accel_gb300", "csrc")

DRIVER = r"""
#include "fi_mirror.hpp"
#include <cstdio>
#include <vector>
using namespace litho;
int main() {
  int Ly, Fy;
  while (std::scanf("%d %d", &Ly, &Fy) == 2) {
    std::vector<int> seen(Ly, 0);
    const int nb = fo_nbase(Ly, Fy);
    for (int b = 0; b < nb; ++b)
      for (int sgn = 0; sgn < 2; ++sgn) {
        const int Y = fo_row(b, sgn, Ly, Fy);
        if (Y < 0) continue;
        if (Y >= Ly) { std::printf("range %d %d %d\n", Ly, Fy, Y); return 1; }
        const int yp = Y + fo_oy(Ly, Fy);
        if (yp != (sgn == 0 ? b : -b)) { std::printf("coord %d %d %d\n", Ly, Fy, Y); return 1; }
        seen[Y]++;
      }
    for (int Y = 0; Y < Ly; ++Y)
      if (seen[Y] != 1) { std::printf("row %d %d %d %d\n", Ly, Fy, Y, seen[Y]); return 1; }
    // the base rows are all needed: the last one writes a row
    if (fo_row(nb - 1, 0, Ly, Fy) < 0 && fo_row(nb - 1, 1, Ly, Fy) < 0) { std::printf("extra %d %d\n", Ly, Fy); return 1; }
  }
  std::printf("ok\n");
  return 0;
}
"""


def _pow2(n):
    p = 1
    while p < n:
        p *= 2
    return p


def test_every_image_row_written_once(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src, exe = tmp_path / "drv.cpp", tmp_path / "drv"
    src.write_text(DRIVER)
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    # every size up to 600 at its own FFT size and at twice it, plus the bench's sizes
    cases = [(ly, _pow2(ly)) for ly in range(2, 601)] + [(ly, 2 * _pow2(ly)) for ly in range(2, 601)]
    cases += [(1024, 1024), (2048, 2048), (301, 512), (129, 256), (16384, 16384)]
    r = subprocess.run([str(exe)], input="".join(f"{a} {b}\n" for a, b in cases), capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout
