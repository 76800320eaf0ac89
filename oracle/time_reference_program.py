"""Time the reference's own litho program on its 1024^2 configuration.

TEST INFRASTRUCTURE ONLY.  Runs oracle/_ref/litho (1 thread) and
oracle/_ref/litho_thread (OpenMP, all cores), built unmodified from the
reference's sources by oracle/build_oracle.py, on input/config/golden_1024.json
(annular 0.6/0.9 on 101^2, NA 0.8, 193 nm, defocus 0.2, Nx = 8) with the mask
input/mask/1024x1024.png (tests/golden/mask1024_t1.npz) at kernel.count K, and
reports the median over runs of the program's own [TIME] lines for Module 3
(FFT of the mask, litho.cpp:1318-1346) and Module 7 (calcSOCS + FI,
litho.cpp:1436-1451): the operations one mask -> image conversion with fixed
kernels costs.  Both binaries link the project's FFTW-API shim, which is slower
than FFTW itself.

    python oracle/time_reference_program.py [--runs 5] [--nk 24]
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def _config(td, nk):
    d = np.load(os.path.join(GOLDEN, "mask1024_t1.npz"))
    mask = np.unpackbits(d["bits"]).reshape(tuple(d["shape"])).astype(np.float32)
    os.makedirs(os.path.join(td, "input", "config"), exist_ok=True)
    os.makedirs(os.path.join(td, "input", "mask"), exist_ok=True)
    mask.tofile(os.path.join(td, "input", "mask", "m.bin"))
    cfg = {"mask": {"period": {"Lx": 1024, "Ly": 1024}, "size": {"maskSizeX": 1024, "maskSizeY": 1024},
                    "type": "Import", "inputFile": "input/mask/m.bin", "dose": 1.0},
           "source": {"gridSize": 101, "type": "Annular", "annular": {"innerRadius": 0.6, "outerRadius": 0.9}},
           "optics": {"NA": 0.8, "wavelength": 193.0, "defocus": 0.2},
           "kernel": {"count": nk, "targetIntensity": 0.225}}
    path = os.path.join(td, "input", "config", "c.json")
    json.dump(cfg, open(path, "w"))
    return path


def _module_us(stdout):
    out = {}
    for m, v in re.findall(r"Module (\d) \([^)]*\):\s+(\d+) us", stdout):
        out[int(m)] = int(v)
    return out


def time_program(exe, runs, nk, threads=None):
    env = dict(os.environ)
    if threads is not None:
        env["OMP_NUM_THREADS"] = str(threads)
    m3, m7 = [], []
    with tempfile.TemporaryDirectory() as td:
        cfg = _config(td, nk)
        for r in range(runs + 1):
            res = subprocess.run([exe, cfg, os.path.join(td, f"out{r}")], capture_output=True, text=True,
                                 check=True, env=env)
            t = _module_us(res.stdout)
            if r > 0:  # the first run warms the page cache
                m3.append(t[3] / 1e3)
                m7.append(t[7] / 1e3)
    a, b = statistics.median(m3), statistics.median(m7)
    return {"module3_ms": a, "module7_ms": b, "images_per_s": 1e3 / (a + b), "runs": runs}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--runs", type=int, default=5)
    ap.add_argument("--nk", type=int, default=24)
    a = ap.parse_args()
    ref = os.path.join(HERE, "_ref")
    if not os.path.exists(os.path.join(ref, "litho")):
        sys.exit("oracle/_ref/litho is not built (python oracle/build_oracle.py <reference checkout>)")
    cores = os.cpu_count() or 1
    res = {"nk": a.nk, "cores": cores,
           "litho_1thread": time_program(os.path.join(ref, "litho"), a.runs, a.nk),
           "litho_thread_all_cores": time_program(os.path.join(ref, "litho_thread"), a.runs, a.nk, cores)}
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    main()
