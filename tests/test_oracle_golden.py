"""Pin the FP64 oracle to the reference's own checked-in golden vectors.

The fixtures in tests/golden/ are copied from the reference by
tests/golden/make_golden.py (see its docstring for the source files).
"""
import numpy as np

from conftest import load_golden
from oracle import np_ref as R


def test_outer_sigma_and_nx(golden_optics):
    # tb_calc_tcc_correct.cpp:28-32: outerSigma 0.9, Nx = Ny = 4, tccSize 81
    assert abs(golden_optics["sigma"] - 0.9) < 1e-6
    assert golden_optics["Nx"] == 4
    assert golden_optics["tcc"].shape == (81, 81)


def test_tcc_matches_reference_golden(golden_optics):
    g = load_golden("tcc_golden.npz")
    ref = g["tcc_r"].astype(np.float64) + 1j * g["tcc_i"].astype(np.float64)
    tcc = golden_optics["tcc"]
    err = np.linalg.norm(tcc - ref) / np.linalg.norm(ref)
    assert err < 1e-7, err
    # Hermitian by construction (litho.cpp:510-515)
    assert np.array_equal(tcc, tcc.conj().T)


def test_eigenvalues_match_kernel_info(golden_optics):
    g = load_golden("tcc_golden.npz")
    _, scales, _ = R.calc_kernels(golden_optics["tcc"], 10)
    # kernel_info.txt prints 6 significant digits (std::cout default): rel rounding <= 5e-6
    np.testing.assert_allclose(scales, g["eigenvalues"], rtol=6e-6)


def _golden_mask512():
    ig = load_golden("image_golden.npz")
    m256 = np.unpackbits(ig["mask256_bits"]).reshape(256, 256).astype(np.float32)
    return R.create_mask(m256, 512, 512), ig["image512"]


def test_tcc_direct_image_matches_reference_golden(golden_optics):
    mask, ref = _golden_mask512()
    mskf = R.ft_r2c_padded(mask, 512, 512)
    nx = golden_optics["Nx"]
    img = R.ft_c2r_padded(R.calc_image(mskf, golden_optics["tcc"], nx, nx), 512, 512)
    assert R.rel_l2(img, ref) < 1e-7


def test_full_rank_socs_equals_tcc_direct_golden(golden_optics):
    """Full-rank SOCS + FI reproduces the TCC-direct golden for any conv grid / embed."""
    mask, ref = _golden_mask512()
    mskf = R.ft_r2c_padded(mask, 512, 512)
    nx = golden_optics["Nx"]
    krns, scales, _ = R.calc_kernels(golden_optics["tcc"], 81)
    for n, e in ((128, 94), (64, None), (32, None)):
        img, _ = R.calc_socs(mskf, 512, 512, krns, scales, 81, nx, nx, n, e)
        assert R.rel_l2(img, ref) < 1e-7, (n, e)


def test_socs_tmpimgp_matches_hls_golden(golden_optics):
    """source/SOCS_HLS/data/hls_output_full_32.bin: nk=4, 32x32 conv grid (FP32 HLS run)."""
    h = load_golden("hls_golden.npz")
    m = (h["mask512_u8"].astype(np.float32) / np.float32(255)).astype(np.float32)
    mskf = R.ft_r2c_padded(R.create_mask(m, 512, 512), 512, 512)
    nx = golden_optics["Nx"]
    krns, scales, _ = R.calc_kernels(golden_optics["tcc"], 4)
    t = R.socs_tmpimg(mskf, krns, scales, 4, nx, nx, 32, None)
    assert R.rel_l2(t, h["tmpimgp32"]) < 5e-6
    assert R.rel_l2(R.tmpimgp_center(t, nx, nx), h["center17"]) < 5e-6


def test_ft_r2c_padded_is_centred_fft():
    """litho.cpp:242-318 rebuild == fftshift(fft2(ifftshift(pad(m)))) / F^2 (even F)."""
    rng = np.random.default_rng(3)
    m = rng.random((24, 20)).astype(np.float32)
    out = R.ft_r2c_padded(m, 32, 32)
    ref = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(R.pad_centered(m, 32, 32).astype(np.float64)))) / 1024
    np.testing.assert_allclose(out, ref, atol=1e-14)


def test_immersion_extension_of_the_pupil():
    """n_medium = 1 is the reference formula; NA > 1 is NaN there and finite with n = 1.44."""
    from oracle import np_ref as R
    src = R.normalize_source(R.create_annular(21, 0.6, 0.9))
    sig = R.get_outer_sigma(src)
    a = R.calc_tcc(src, sig, 193.0, 0.8, 0.2, 256, 256, 2, 2)
    b = R.calc_tcc(src, sig, 193.0, 0.8, 0.2, 256, 256, 2, 2, n_medium=1.0)
    assert np.array_equal(a, b)
    nx = R.optics_nx(1.35, 128, sig, 193.0)
    with np.errstate(invalid="ignore"):
        c = R.calc_tcc(src, sig, 193.0, 1.35, 0.0, 128, 128, nx, nx)
    assert not np.isfinite(c).all()
    d = R.calc_tcc(src, sig, 193.0, 1.35, 0.0, 128, 128, nx, nx, n_medium=1.44)
    assert np.isfinite(d).all()
    assert np.allclose(d, d.conj().T)
