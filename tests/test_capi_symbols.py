"""The C-ABI library loads on the CPU and exports every entry point that
include/*.h declares (no compute calls: there is no GPU here)."""
import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", src):
            n = m.group(1)
            if n.startswith(("litho_", "calc_")) and not n.endswith("_t"):
                names.add(n)
    return sorted(names)


def test_header_declares_entry_points():
    names = _declared()
    for need in ("litho_ctx_create", "litho_fft_mask", "litho_calc_socs", "litho_image",
                 "litho_image_batch", "litho_calc_tcc", "litho_calc_kernels"):
        assert need in names


def test_library_exports_every_declared_symbol():
    lib_path = os.path.join(ROOT, "fpga-litho-accel_gb300", "litho_gb300", "liblitho_gb300.so")
    if not os.path.exists(lib_path):
        pytest.fail("liblitho_gb300.so not built (run __graft_entry__.build())")
    lib = ctypes.CDLL(lib_path)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings_and_version():
    import litho_gb300 as L
    assert L.lib().litho_status_string(L.LITHO_ERR_ARG) == b"LITHO_ERR_ARG"
    assert L.lib().litho_version() >= 10000


def test_optics_helpers_match_oracle():
    """getOuterSigma / Nx (litho.cpp:414-426, 1297-1301) are host code: checked on CPU."""
    import numpy as np
    import litho_gb300 as L
    from litho_gb300 import synth
    from oracle import np_ref as R
    for src in (R.normalize_source(R.create_annular(101, 0.6, 0.9)), synth.annular_source(21, 0.6, 0.9),
                synth.quasar_source()[0]):
        s_lib = L.outer_sigma(src)
        s_ref = min(R.get_outer_sigma(src), 1.0)
        assert s_lib == np.float32(s_ref)
        for Lp in (256, 512, 1024, 2048):
            assert L.optics_n(0.8, Lp, s_lib, 193.0) == R.optics_nx(0.8, Lp, s_ref, 193.0)
