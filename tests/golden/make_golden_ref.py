"""Run the reference's own litho program (built unmodified by oracle/build_oracle.py)
and store its outputs as fixtures.

Needs the reference checkout (for the build and the mask PNGs); the GPU host
never runs this.  The checkout is named by the first argument or by the
LITHO_REFERENCE_DIR environment variable:

    python oracle/build_oracle.py <reference> && python tests/golden/make_golden_ref.py <reference>

Writes, in tests/golden/:

* ref_litho_<name>.npz for the two 256^2 cases, with the program's own BIN
  outputs: full mskf planes, tcc (25x25 complex), scales, kernels (complex,
  k-major), aerial_image_tcc_direct, aerial_image_socs_kernel,
  tmpImgp_full_128, plus the mask and the optics.
* ref_litho_golden1024.npz: the program run on the reference's own 1024^2
  configuration (input/config/golden_1024.json: annular 0.6/0.9 on 101^2, NA
  0.8, lambda 193, defocus 0.2, Nx = 8, tcc 289) with the mask
  input/mask/1024x1024.png (tests/golden/mask1024_t1.npz), at kernel.count 10
  and 24.  To keep the file small it holds the 65x65 mask-spectrum window
  around DC, the full TCC, and per count the scales, kernels and
  tmpImgp_full_128; of each 1024^2 image it holds every 16th row (rows 0, 16,
  ...) exactly as the program wrote them and float64 statistics (mean, std,
  max, min) of the whole image.
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

# input/config/golden_1024.json (the reference's 1024^2 configuration, run_log_10kernels.txt)
GOLDEN1024 = dict(mask="mask1024", gridSize=101, inner=0.6, outer=0.9, NA=0.8, wavelength=193.0, defocus=0.2)
GOLDEN1024_COUNTS = (10, 24)
ROW_STRIDE = 16
WIN = 32  # mask-spectrum window half-width stored (65 x 65 around DC)


def _mask(kind, ref):
    if kind == "golden_mask256":
        return np.fromfile(os.path.join(ref, "source/TCC_HLS/hls/tb/golden/mask_256x256.bin"),
                           np.float32).reshape(256, 256)
    if kind == "mask1024":
        d = np.load(os.path.join(HERE, "mask1024_t1.npz"))
        return np.unpackbits(d["bits"]).reshape(tuple(d["shape"])).astype(np.float32)
    u8 = read_png_gray8(os.path.join(ref, "input/mask/Different_resolution_tests/256x256.png"))
    return (u8.astype(np.float32) / np.float32(255)).astype(np.float32)


def _run_program(mask, c, nk, td):
    """Write the mask and a litho JSON config into td, run the program, return (out dir, stdout)."""
    L = mask.shape[0]
    os.makedirs(os.path.join(td, "input", "config"), exist_ok=True)
    os.makedirs(os.path.join(td, "input", "mask"), exist_ok=True)
    mask.tofile(os.path.join(td, "input", "mask", "m.bin"))
    cfg = {"mask": {"period": {"Lx": L, "Ly": L}, "size": {"maskSizeX": L, "maskSizeY": L}, "type": "Import",
                    "inputFile": "input/mask/m.bin", "dose": 1.0},
           "source": {"gridSize": c["gridSize"], "type": "Annular",
                      "annular": {"innerRadius": c["inner"], "outerRadius": c["outer"]}},
           "optics": {"NA": c["NA"], "wavelength": c["wavelength"], "defocus": c["defocus"]},
           "kernel": {"count": nk, "targetIntensity": 0.225}}
    cpath = os.path.join(td, "input", "config", f"c{nk}.json")
    json.dump(cfg, open(cpath, "w"))
    out = os.path.join(td, f"out{nk}")
    r = subprocess.run([LITHO, cpath, out], check=True, capture_output=True, text=True)
    return out, r.stdout


def _reader(out):
    return lambda f, shape: np.fromfile(os.path.join(out, f), np.float32).reshape(shape)


def _kernels(out, n):
    rd = _reader(out)
    scales = np.fromfile(os.path.join(out, "scales.bin"), np.float32)
    krn = np.stack([rd(f"kernels/krn_{k}_r.bin", (n,)) + 1j * rd(f"kernels/krn_{k}_i.bin", (n,))
                    for k in range(scales.size)]).astype(np.complex64)
    return scales, krn


def run_case(name, c, ref):
    mask = _mask(c["mask"], ref)
    L = mask.shape[0]
    with tempfile.TemporaryDirectory() as td:
        out, _ = _run_program(mask, c, c["nk"], td)
        rd = _reader(out)
        meta = dict(l.split() for l in open(os.path.join(out, "fft_meta.txt")) if l.strip())
        nx = int(meta["Nx"])
        n = (2 * nx + 1) ** 2
        F = int(meta["fft_size_x"])
        scales, krn = _kernels(out, n)
        mr, mi = rd("mskf_r.bin", (F, F)), rd("mskf_i.bin", (F, F))
        np.savez_compressed(
            os.path.join(HERE, f"ref_litho_{name}.npz"),
            mask=mask, Nx=nx, F=F, nk=scales.size, gridSize=c["gridSize"], inner=c["inner"], outer=c["outer"],
            NA=c["NA"], wavelength=c["wavelength"], defocus=c["defocus"],
            mskf_r=mr, mskf_i=mi,
            tcc=(rd("tcc_r.bin", (n, n)) + 1j * rd("tcc_i.bin", (n, n))).astype(np.complex64),
            scales=scales, krn=krn,
            image_tcc=rd("aerial_image_tcc_direct.bin", (L, L)),
            image_socs=rd("aerial_image_socs_kernel.bin", (L, L)),
            tmpimgp128=rd("tmpImgp_full_128.bin", (128, 128)))
        print(name, "Nx", nx, "nk", scales.size, "F", F)


def _stats(img):
    x = img.astype(np.float64)
    return np.asarray([x.mean(), x.std(), x.max(), x.min()])


def run_golden1024(ref):
    c = GOLDEN1024
    mask = _mask(c["mask"], ref)
    L = mask.shape[0]
    fx = {"gridSize": c["gridSize"], "inner": c["inner"], "outer": c["outer"], "NA": c["NA"],
          "wavelength": c["wavelength"], "defocus": c["defocus"], "row_stride": ROW_STRIDE, "win": WIN,
          "counts": np.asarray(GOLDEN1024_COUNTS)}
    with tempfile.TemporaryDirectory() as td:
        for nk in GOLDEN1024_COUNTS:
            out, _ = _run_program(mask, c, nk, td)
            rd = _reader(out)
            meta = dict(l.split() for l in open(os.path.join(out, "fft_meta.txt")) if l.strip())
            nx, F = int(meta["Nx"]), int(meta["fft_size_x"])
            n = (2 * nx + 1) ** 2
            scales, krn = _kernels(out, n)
            socs = rd("aerial_image_socs_kernel.bin", (L, L))
            fx.update({f"scales_{nk}": scales, f"krn_{nk}": krn,
                       f"tmpimgp128_{nk}": rd("tmpImgp_full_128.bin", (128, 128)),
                       f"socs_rows_{nk}": socs[::ROW_STRIDE].copy(), f"socs_stats_{nk}": _stats(socs)})
            if nk == GOLDEN1024_COUNTS[0]:
                mskf = rd("mskf_r.bin", (F, F)) + 1j * rd("mskf_i.bin", (F, F))
                img_tcc = rd("aerial_image_tcc_direct.bin", (L, L))
                fx.update({"Nx": nx, "F": F,
                           "mskf_win": mskf[F // 2 - WIN:F // 2 + WIN + 1, F // 2 - WIN:F // 2 + WIN + 1]
                           .astype(np.complex64),
                           "tcc": (rd("tcc_r.bin", (n, n)) + 1j * rd("tcc_i.bin", (n, n))).astype(np.complex64),
                           "tcc_rows": img_tcc[::ROW_STRIDE].copy(), "tcc_stats": _stats(img_tcc)})
            print("golden1024 nk", nk, "Nx", nx, "F", F, "scales", scales[:3], "...")
    np.savez_compressed(os.path.join(HERE, "ref_litho_golden1024.npz"), **fx)


def reference_dir(argv):
    ref = argv[1] if len(argv) > 1 else os.environ.get("LITHO_REFERENCE_DIR")
    if not ref:
        sys.exit("usage: make_golden_ref.py <reference checkout>  (or set LITHO_REFERENCE_DIR)")
    return ref


if __name__ == "__main__":
    ref = reference_dir(sys.argv)
    for k, v in CASES.items():
        run_case(k, v, ref)
    run_golden1024(ref)
