"""Run the reference's own litho program (built unmodified by oracle/build_oracle.py)
and store its outputs as fixtures.

Needs the reference checkout (for the build and the mask PNG); the GPU host
never runs this.

    python oracle/build_oracle.py && python tests/golden/make_golden_ref.py

Writes tests/golden/ref_litho_<name>.npz with the program's own BIN outputs:
mskf window (9x9 around DC) and full planes, tcc (25x25 complex), scales,
kernels (complex, k-major), aerial_image_tcc_direct, aerial_image_socs_kernel,
tmpImgp_full_128, plus the mask and the optics.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
from make_golden import read_png_gray8  # noqa: E402

LITHO = os.path.join(ROOT, "oracle", "_ref", "litho")

CASES = {
    # the reference's binary golden mask, its golden optics (defocus 0.2, annular 0.6/0.9 on 101^2)
    "bin256": dict(mask="golden_mask256", gridSize=101, inner=0.6, outer=0.9, NA=0.8, wavelength=193.0,
                   defocus=0.2, nk=10),
    # a grey-level PNG mask / 255 (tool/png_bin_converter.py semantics), small source, focus
    "grey256": dict(mask="png256", gridSize=21, inner=0.5, outer=0.8, NA=0.8, wavelength=193.0,
                    defocus=0.0, nk=12),
}


def _mask(kind, ref):
    if kind == "golden_mask256":
        return np.fromfile(os.path.join(ref, "source/TCC_HLS/hls/tb/golden/mask_256x256.bin"),
                           np.float32).reshape(256, 256)
    u8 = read_png_gray8(os.path.join(ref, "input/mask/Different_resolution_tests/256x256.png"))
    return (u8.astype(np.float32) / np.float32(255)).astype(np.float32)


def run_case(name, c, ref):
    mask = _mask(c["mask"], ref)
    L = mask.shape[0]
    with tempfile.TemporaryDirectory() as td:
        os.makedirs(os.path.join(td, "input", "config"))
        os.makedirs(os.path.join(td, "input", "mask"))
        mask.tofile(os.path.join(td, "input", "mask", "m.bin"))
        cfg = {"mask": {"period": {"Lx": L, "Ly": L}, "size": {"maskSizeX": L, "maskSizeY": L}, "type": "Import",
                        "inputFile": "input/mask/m.bin", "dose": 1.0},
               "source": {"gridSize": c["gridSize"], "type": "Annular",
                          "annular": {"innerRadius": c["inner"], "outerRadius": c["outer"]}},
               "optics": {"NA": c["NA"], "wavelength": c["wavelength"], "defocus": c["defocus"]},
               "kernel": {"count": c["nk"], "targetIntensity": 0.225}}
        cpath = os.path.join(td, "input", "config", "c.json")
        json.dump(cfg, open(cpath, "w"))
        out = os.path.join(td, "out")
        subprocess.run([LITHO, cpath, out], check=True, capture_output=True)
        rd = lambda f, shape: np.fromfile(os.path.join(out, f), np.float32).reshape(shape)  # noqa: E731
        meta = dict(l.split() for l in open(os.path.join(out, "fft_meta.txt")) if l.strip())
        nx = int(meta["Nx"])
        n = (2 * nx + 1) ** 2
        F = int(meta["fft_size_x"])
        scales = np.fromfile(os.path.join(out, "scales.bin"), np.float32)
        nk = scales.size
        krn = np.stack([rd(f"kernels/krn_{k}_r.bin", (n,)) + 1j * rd(f"kernels/krn_{k}_i.bin", (n,))
                        for k in range(nk)]).astype(np.complex64)
        mr, mi = rd("mskf_r.bin", (F, F)), rd("mskf_i.bin", (F, F))
        np.savez_compressed(
            os.path.join(HERE, f"ref_litho_{name}.npz"),
            mask=mask, Nx=nx, F=F, nk=nk, gridSize=c["gridSize"], inner=c["inner"], outer=c["outer"],
            NA=c["NA"], wavelength=c["wavelength"], defocus=c["defocus"],
            mskf_r=mr, mskf_i=mi,
            tcc=(rd("tcc_r.bin", (n, n)) + 1j * rd("tcc_i.bin", (n, n))).astype(np.complex64),
            scales=scales, krn=krn,
            image_tcc=rd("aerial_image_tcc_direct.bin", (L, L)),
            image_socs=rd("aerial_image_socs_kernel.bin", (L, L)),
            tmpimgp128=rd("tmpImgp_full_128.bin", (128, 128)))
        print(name, "Nx", nx, "nk", nk, "F", F)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    for k, v in CASES.items():
        run_case(k, v, ref)
