"""The C++-linkage shims with the reference's FPGA top-function signatures
(include/litho_gb300_hls.hpp), called the way the reference's C-simulation
testbenches call the HLS tops, checked against the reference's goldens."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden
from oracle import np_ref as R

pytestmark = pytest.mark.gpu

SOCS_V18 = "_Z40calc_socs_2048_hls_stream_refactored_v18PfS_S_S_S_S_S_iiiii"
CALC_TCC = "_Z8calc_tccPfiPSt7complexIfER13OpticalParamsiii"


class OpticalParams(C.Structure):   # source/TCC_HLS/hls/src/data_types.h layout
    _fields_ = [("NA", C.c_float), ("lambda_", C.c_float), ("defocus", C.c_float), ("Lx", C.c_float),
                ("Ly", C.c_float), ("outerSigma", C.c_float), ("srcSize", C.c_int), ("Nx", C.c_int),
                ("Ny", C.c_int)]


def _fn(name, nargs):
    import litho_gb300 as L
    f = getattr(L.lib(), name)
    f.restype = None
    return f


def test_socs_v18_shim_matches_reference_program_tmpimgp():
    """v18 top: 128^2 fftshifted intensity (litho.cpp's tmpImgp_full_128) into both outputs."""
    d = load_golden("ref_litho_bin256.npz")
    nx, nk, F = int(d["Nx"]), int(d["nk"]), int(d["F"])
    f = _fn(SOCS_V18, 12)
    f.argtypes = [C.c_void_p] * 7 + [C.c_int] * 5
    mr = np.ascontiguousarray(d["mskf_r"], np.float32)
    mi = np.ascontiguousarray(d["mskf_i"], np.float32)
    kr = np.ascontiguousarray(d["krn"].real, np.float32)
    ki = np.ascontiguousarray(d["krn"].imag, np.float32)
    sc = np.ascontiguousarray(d["scales"], np.float32)
    tmp = np.zeros(128 * 128, np.float32)
    out = np.zeros(128 * 128, np.float32)
    f(mr.ctypes.data, mi.ctypes.data, kr.ctypes.data, ki.ctypes.data, sc.ctypes.data, tmp.ctypes.data,
      out.ctypes.data, nk, nx, nx, F, F)
    assert np.array_equal(tmp, out)
    assert R.rel_l2(out.reshape(128, 128), d["tmpimgp128"]) < 1e-5


def test_calc_tcc_shim_matches_tcc_golden():
    """calc_tcc top with the testbench's parameters (tb_calc_tcc_correct.cpp:22-34)."""
    g = load_golden("tcc_golden.npz")
    gold = g["tcc_r"].astype(np.float64) + 1j * g["tcc_i"].astype(np.float64)
    src = R.normalize_source(R.create_annular(101, 0.6, 0.9)).astype(np.float32)
    prm = OpticalParams(0.8, 193.0, 0.2, 512.0, 512.0, 0.9, 101, 4, 4)
    out = np.zeros(81 * 81, np.complex64)
    f = _fn(CALC_TCC, 7)
    f.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int]
    sh = 50
    f(src.ctypes.data, 101, out.ctypes.data, C.addressof(prm), 81, sh, int(np.ceil(np.float32(sh) * np.float32(0.9))))
    t = out.reshape(81, 81).astype(np.complex128)
    assert np.linalg.norm(t - gold) / np.linalg.norm(gold) < 1e-6
