"""Host-side helpers of the C ABI (no GPU): source/mask generators against the
oracle's restatement of common/source.cpp and common/mask.cpp, and the BIN and
kernel_info.txt formats of common/file_io.cpp."""
import ctypes as C

import numpy as np
import pytest

from oracle import np_ref as R


@pytest.fixture(scope="module")
def lib():
    import litho_gb300 as L
    lb = L.lib()
    lb.litho_create_source.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int]
    lb.litho_create_linespace.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
    lb.litho_place_mask.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_void_p, C.c_int, C.c_int]
    lb.litho_write_bin.argtypes = [C.c_char_p, C.c_void_p, C.c_longlong]
    lb.litho_read_bin.argtypes = [C.c_char_p, C.c_void_p, C.c_longlong]
    lb.litho_write_kernel_info.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
    lb.litho_read_kernel_info.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    return lb


def _src(lib, S, typ, params, normalize=1):
    out = np.zeros((S, S), np.float32)
    p = np.asarray(params, np.float32)
    assert lib.litho_create_source(out.ctypes.data, S, typ, p.ctypes.data, normalize) == 0
    return out


@pytest.mark.parametrize("S", [21, 51, 101])
def test_sources_match_oracle(lib, S):
    assert np.array_equal(_src(lib, S, 0, [0.6, 0.9]), R.normalize_source(R.create_annular(S, 0.6, 0.9)))
    assert np.array_equal(_src(lib, S, 2, [0.3, 0.5], 0), R.create_cross_quadrupole(S, 0.3, 0.5))
    for onx in (0, 1):
        assert np.array_equal(_src(lib, S, 1, [0.25, 0.55, onx], 0), R.create_dipole(S, 0.25, 0.55, bool(onx)))


def test_point_source_and_bad_args(lib):
    s = _src(lib, 21, 3, [0.0, 0.0], 0)
    # source.cpp:121-128: round(0*S/2 + S/2) = round(10.5) = 11, then -1 for x >= 0 and -y >= 0
    assert s.sum() == 1.0 and s[10, 10] == 1.0
    out = np.zeros((5, 5), np.float32)
    assert lib.litho_create_source(out.ctypes.data, 5, 99, None, 1) != 0


def test_linespace_and_place_mask(lib):
    for horiz in (0, 1):
        m = np.zeros((48, 64), np.float32)
        assert lib.litho_create_linespace(m.ctypes.data, 64, 48, 6, 10, horiz) == 0
        assert np.array_equal(m, R.line_space(64, 48, 6, 10, bool(horiz)))
    rng = np.random.default_rng(1)
    pat = rng.random((30, 50)).astype(np.float32)
    out = np.zeros((64, 80), np.float32)
    assert lib.litho_place_mask(pat.ctypes.data, 50, 30, 0.75, out.ctypes.data, 80, 64) == 0
    assert np.array_equal(out, R.create_mask(pat, 80, 64, 0.75))


def test_bin_roundtrip_and_size_mismatch(lib, tmp_path):
    a = np.arange(10, dtype=np.float32)
    p = str(tmp_path / "a.bin").encode()
    assert lib.litho_write_bin(p, a.ctypes.data, 10) == 0
    b = np.full(14, -1, np.float32)
    assert lib.litho_read_bin(p, b.ctypes.data, 14) == 0          # pads with zeros (file_io.cpp:251-258)
    assert np.array_equal(b, np.r_[a, np.zeros(4, np.float32)])
    c = np.zeros(6, np.float32)
    assert lib.litho_read_bin(p, c.ctypes.data, 6) == 0           # truncates
    assert np.array_equal(c, a[:6])
    assert lib.litho_read_bin(str(tmp_path / "missing.bin").encode(), c.ctypes.data, 6) == 6   # LITHO_ERR_IO


def test_kernel_info_roundtrip(lib, tmp_path):
    sc = np.array([5.75947, 2.47371, 0.0863987], np.float32)
    p = str(tmp_path / "kernel_info.txt").encode()
    assert lib.litho_write_kernel_info(p, 9, 9, 3, sc.ctypes.data) == 0
    txt = open(p.decode()).read()
    assert txt.startswith("# Kernel Information\n## Kernel Size and Count\n- Kernel Size: 9x9\n")
    kx, ky, nk = C.c_int(), C.c_int(), C.c_int()
    got = np.zeros(8, np.float32)
    assert lib.litho_read_kernel_info(p, C.addressof(kx), C.addressof(ky), C.addressof(nk), got.ctypes.data, 8) == 0
    assert (kx.value, ky.value, nk.value) == (9, 9, 3)
    np.testing.assert_allclose(got[:3], sc, rtol=1e-6)
