"""The litho-compatible CLI writes the reference program's file set.

Runs litho_gb300_cli on the configuration the reference program was run on
(tests/golden/ref_litho_bin256.npz, produced by the reference's own litho.cpp)
and compares every BIN output with the program's.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import PKG_DIR, load_golden
from oracle import np_ref as R

CLI = os.path.join(PKG_DIR, "litho_gb300", "litho_gb300_cli")


def _write_case(tmp_path, d):
    L = d["mask"].shape[0]
    (tmp_path / "input" / "config").mkdir(parents=True)
    (tmp_path / "input" / "mask").mkdir(parents=True)
    d["mask"].astype(np.float32).tofile(tmp_path / "input" / "mask" / "m.bin")
    cfg = {"mask": {"period": {"Lx": L, "Ly": L}, "size": {"maskSizeX": L, "maskSizeY": L}, "type": "Import",
                    "inputFile": "input/mask/m.bin", "dose": 1.0},
           "source": {"gridSize": int(d["gridSize"]), "type": "Annular",
                      "annular": {"innerRadius": float(d["inner"]), "outerRadius": float(d["outer"])}},
           "optics": {"NA": float(d["NA"]), "wavelength": float(d["wavelength"]), "defocus": float(d["defocus"])},
           "kernel": {"count": int(d["nk"]), "targetIntensity": 0.225}}
    p = tmp_path / "input" / "config" / "c.json"
    p.write_text(json.dumps(cfg))
    return str(p)


def test_cli_binary_built():
    if not os.path.exists(CLI):
        pytest.fail("litho_gb300_cli not built (run __graft_entry__.build())")


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["bin256", "grey256"])
def test_cli_matches_reference_program_outputs(tmp_path, name):
    d = load_golden(f"ref_litho_{name}.npz")
    d = {k: d[k] for k in d.files}
    cfg = _write_case(tmp_path, d)
    out = tmp_path / "out"
    r = subprocess.run([CLI, cfg, str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "[TIME] SOCS Image" in r.stdout
    L, F, nx, nk = d["mask"].shape[0], int(d["F"]), int(d["Nx"]), int(d["nk"])
    n = (2 * nx + 1) ** 2
    rd = lambda f, shape: np.fromfile(out / f, np.float32).reshape(shape)  # noqa: E731
    meta = dict(line.split() for line in open(out / "fft_meta.txt") if line.strip())
    assert int(meta["Nx"]) == nx and int(meta["fft_size_x"]) == F
    mskf = rd("mskf_r.bin", (F, F)) + 1j * rd("mskf_i.bin", (F, F))
    assert np.linalg.norm(mskf - (d["mskf_r"] + 1j * d["mskf_i"])) / np.linalg.norm(d["mskf_r"] + 1j * d["mskf_i"]) < 1e-5
    tcc = rd("tcc_r.bin", (n, n)) + 1j * rd("tcc_i.bin", (n, n))
    assert np.linalg.norm(tcc - d["tcc"]) / np.linalg.norm(d["tcc"]) < 1e-6
    assert R.rel_l2(rd("aerial_image_tcc_direct.bin", (L, L)), d["image_tcc"]) < 1e-5
    np.testing.assert_allclose(np.fromfile(out / "scales.bin", np.float32), d["scales"], rtol=1e-5,
                               atol=1e-7 * float(d["scales"][0]))
    info = open(out / "kernels" / "kernel_info.txt").read()
    assert f"- Kernel Size: {2 * nx + 1}x{2 * nx + 1}" in info and f"- Number of Kernels: {nk}" in info
    assert os.path.exists(out / "kernels" / f"krn_{nk - 1}_i.bin")
    # bin256's 10th eigenvalue lies 4.8e-7 from a degenerate pair (see test_reference_program)
    tol = 2e-4 if name == "bin256" else 1e-5
    assert R.rel_l2(rd("aerial_image_socs_kernel.bin", (L, L)), d["image_socs"]) < tol
    assert R.rel_l2(rd("tmpImgp_full_128.bin", (128, 128)), d["tmpimgp128"]) < tol
    assert os.path.getsize(out / "tmpImgp_pad128.bin") == 4 * (4 * nx + 1) ** 2
