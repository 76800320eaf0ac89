"""Parity at the metric's geometry (1024^2, Nx = 8, tcc 289) against the reference itself.

Fixture: tests/golden/ref_litho_golden1024.npz, written by
tests/golden/make_golden_ref.py from the reference's own litho.cpp (built
unmodified by oracle/build_oracle.py) run on the reference's 1024^2
configuration (input/config/golden_1024.json: annular 0.6/0.9 on a 101^2 grid,
NA 0.8, lambda 193, defocus 0.2) with its mask input/mask/1024x1024.png, at
kernel.count 10 and 24.  Images are held as every 16th row plus whole-image
statistics (see the script's docstring).

Reference-held pins at the same configuration, checked here too:

* data/pc_cpp/run_log_10kernels.txt:43-47 -- mask-spectrum samples around DC;
  :56-59 -- TCC real-part statistics; :68-71 -- TCC-direct image statistics;
  :80-89 -- the ten scales.  Printed with six decimals (printStatistics,
  litho.cpp:1124-1145: population std over float data).
* data/matlab/out_validate/validation_metrics.csv:56-65 -- the ten largest
  eigenvalues in float64.  That MATLAB run formed its TCC with float64 pupil
  coordinates where litho.cpp:449-464 uses float32, which moves the spectrum
  by ~3e-8 relative; the bar is 5e-8.

The log's SOCS-image statistics (run_log_10kernels.txt:107-110) are NOT a pin:
kernel.count 10 cuts the degenerate pair 0.322799 (eigenvalues 9 and 10 of
data/pc_cpp/output_400kernels/kernels/kernel_info.txt), so the tenth kernel is
whichever member of that 2-D eigenspace the LAPACK build returns, and the
program built here prints max 0.379374 where the log has 0.380353.  At count 24
the cut falls in a gap (0.106370 vs 0.0870624) and the image is well defined;
the GPU chain is held to it.
"""
import numpy as np
import pytest

from conftest import load_golden
from oracle import np_ref as R

L = 1024
FP32_TOL = 1e-5     # plain GPU path vs the reference program (FP32 contract)
MIXED_TOL = 1e-4    # split-BF16 TCC / TF32 DFT path vs the reference program

RUN_LOG_MSKF = {(511, 511): 0.026167 - 0.002220j, (511, 512): 0.063272 + 0.000934j,
                (511, 513): 0.017988 - 0.001101j, (512, 511): 0.099257 + 0.036346j,
                (512, 512): 0.205368 + 0.0j}
RUN_LOG_TCC_REAL = (0.036434, 0.085118, 1.000000, 0.000000)           # mean, std, max, min
RUN_LOG_TCC_IMAGE = (0.094496, 0.099675, 0.385138, 0.004065)
RUN_LOG_SCALES = (23.010136, 9.634128, 9.634128, 2.661961, 2.638622, 1.067181, 1.067181, 0.554192,
                  0.553295, 0.322799)
MATLAB_EIG = (2.3010134993673475e+01, 9.6341274220890440e+00, 9.6341274220890369e+00, 2.6619608093681761e+00,
              2.6386217146783291e+00, 1.0671814937035911e+00, 1.0671814937035857e+00, 5.5419236896161039e-01,
              5.5329551323364901e-01, 3.2279851697088302e-01)
PRINT_ATOL = 6e-7   # "%f" rounding (5e-7) plus float32 storage


@pytest.fixture(scope="module")
def fx():
    d = load_golden("ref_litho_golden1024.npz")
    return {k: d[k] for k in d.files}


@pytest.fixture(scope="module")
def mask():
    d = load_golden("mask1024_t1.npz")
    return np.unpackbits(d["bits"]).reshape(tuple(d["shape"])).astype(np.float32)


@pytest.fixture(scope="module")
def optics(fx):
    src = R.normalize_source(R.create_annular(int(fx["gridSize"]), float(fx["inner"]), float(fx["outer"])))
    sig = min(R.get_outer_sigma(src), 1.0)
    return dict(src=src, sigma=sig, NA=float(fx["NA"]), wavelength=float(fx["wavelength"]),
                defocus=float(fx["defocus"]), Nx=int(fx["Nx"]))


@pytest.fixture(scope="module")
def oracle_tcc(optics):
    o = optics
    return R.calc_tcc(o["src"], o["sigma"], o["wavelength"], o["NA"], o["defocus"], L, L, o["Nx"], o["Nx"])


def _rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _rows(img, fx):
    return np.asarray(img)[::int(fx["row_stride"])]


def _window(spec, fx):
    w, F = int(fx["win"]), int(fx["F"])
    return np.asarray(spec)[F // 2 - w:F // 2 + w + 1, F // 2 - w:F // 2 + w + 1]


def _full_from_window(fx):
    """A full F x F spectrum that is the program's mask spectrum on the stored window and zero
    outside it.  calcSOCS and calcImage read only the (2Ny+1) x (2Nx+1) entries around DC
    (litho.cpp:888-911, 535-566), which the window covers."""
    w, F = int(fx["win"]), int(fx["F"])
    full = np.zeros((F, F), np.complex64)
    full[F // 2 - w:F // 2 + w + 1, F // 2 - w:F // 2 + w + 1] = fx["mskf_win"]
    return full.real.copy(), full.imag.copy()


def _stats(img):
    x = np.asarray(img, np.float64)
    return np.asarray([x.mean(), x.std(), x.max(), x.min()])


# --------------------------------------------------------------------------- CPU: the fixture and the oracle

def test_fixture_reproduces_run_log_pins(fx):
    """The program built here prints the reference's own 1024^2 log, to its printed digits."""
    for (y, x), v in RUN_LOG_MSKF.items():
        got = fx["mskf_win"][y - int(fx["F"]) // 2 + int(fx["win"]), x - int(fx["F"]) // 2 + int(fx["win"])]
        assert abs(got.real - v.real) < PRINT_ATOL and abs(got.imag - v.imag) < PRINT_ATOL, ((y, x), got, v)
    tr = fx["tcc"].real.astype(np.float32)
    np.testing.assert_allclose(_stats(tr), RUN_LOG_TCC_REAL, atol=PRINT_ATOL)
    np.testing.assert_allclose(fx["tcc_stats"], RUN_LOG_TCC_IMAGE, atol=PRINT_ATOL)
    np.testing.assert_allclose(fx["scales_10"], RUN_LOG_SCALES, atol=PRINT_ATOL)
    np.testing.assert_allclose(fx["scales_24"][:10], RUN_LOG_SCALES, atol=PRINT_ATOL)


def test_oracle_matches_program_at_1024(fx, mask, optics, oracle_tcc):
    assert R.optics_nx(optics["NA"], L, optics["sigma"], optics["wavelength"]) == int(fx["Nx"])
    mskf = R.ft_r2c_padded(mask, L, L)
    assert _rel(_window(mskf, fx), fx["mskf_win"]) < 1e-6
    assert _rel(oracle_tcc, fx["tcc"]) < 1e-6
    _, scales, _ = R.calc_kernels(oracle_tcc, 24)
    np.testing.assert_allclose(scales, fx["scales_24"], rtol=1e-6)
    nx = int(fx["Nx"])
    img_tcc = R.ft_c2r_padded(R.calc_image(mskf, oracle_tcc, nx, nx), L, L)
    assert R.rel_l2(_rows(img_tcc, fx), fx["tcc_rows"]) < 1e-6
    for nk in (10, 24):
        img, tmp = R.calc_socs(mskf, L, L, fx[f"krn_{nk}"].astype(np.complex128), fx[f"scales_{nk}"], nk,
                               nx, nx, 128, 94)
        assert R.rel_l2(_rows(img, fx), fx[f"socs_rows_{nk}"]) < 1e-6, nk
        assert R.rel_l2(tmp, fx[f"tmpimgp128_{nk}"]) < 1e-6, nk
        np.testing.assert_allclose(_stats(img), fx[f"socs_stats_{nk}"], rtol=1e-6, atol=1e-8)


def test_oracle_eigenvalues_match_matlab_fp64(oracle_tcc):
    w = np.linalg.eigvalsh(oracle_tcc)[::-1][:10]
    np.testing.assert_allclose(w, MATLAB_EIG, rtol=5e-8)


# --------------------------------------------------------------------------- GPU: the library against the program

@pytest.fixture(scope="module")
def ctx():
    import litho_gb300 as Lib
    c = Lib.Context(0)
    yield c
    c.close()


@pytest.mark.gpu
def test_gpu_fft_mask_and_tcc_match_program(ctx, fx, mask, optics):
    r, i = ctx.fft_mask(mask)
    spec = r + 1j * i
    assert _rel(_window(spec, fx), fx["mskf_win"]) < FP32_TOL
    for (y, x), v in RUN_LOG_MSKF.items():
        assert abs(spec[y, x] - v) < 2 * PRINT_ATOL, ((y, x), spec[y, x], v)
    o = optics
    tcc = ctx.calc_tcc(o["src"], o["sigma"], o["wavelength"], o["NA"], o["defocus"], L, L, o["Nx"], o["Nx"])
    assert _rel(tcc, fx["tcc"]) < 1e-6
    np.testing.assert_allclose(_stats(tcc.real.astype(np.float32)), RUN_LOG_TCC_REAL, atol=PRINT_ATOL)


@pytest.mark.gpu
def test_gpu_fp64_eigenvalues_match_matlab_and_program(ctx, fx, optics):
    o = optics
    tcc = ctx.calc_tcc(o["src"], o["sigma"], o["wavelength"], o["NA"], o["defocus"], L, L, o["Nx"], o["Nx"])
    _, s32, s64 = ctx.calc_kernels(tcc, 24)
    np.testing.assert_allclose(s64[:10], MATLAB_EIG, rtol=5e-8)
    np.testing.assert_allclose(s32, fx["scales_24"], rtol=1e-6)
    np.testing.assert_allclose(s32[:10], RUN_LOG_SCALES, atol=PRINT_ATOL)


@pytest.mark.gpu
@pytest.mark.parametrize("nk", [10, 24])
def test_gpu_calc_socs_with_program_kernels(ctx, fx, nk):
    """calcSOCS (Module 7) from the program's own mask spectrum, kernels and scales: at count 10
    the program's choice inside the degenerate pair is fixed by its kernels, so both counts pin."""
    mr, mi = _full_from_window(fx)
    nx = int(fx["Nx"])
    img, tmp = ctx.calc_socs(mr, mi, fx[f"krn_{nk}"], fx[f"scales_{nk}"], nx, nx, L, L, want_tmpimgp=True)
    assert R.rel_l2(_rows(img, fx), fx[f"socs_rows_{nk}"]) < FP32_TOL
    assert R.rel_l2(tmp, fx[f"tmpimgp128_{nk}"]) < FP32_TOL
    np.testing.assert_allclose(_stats(img), fx[f"socs_stats_{nk}"], rtol=FP32_TOL, atol=1e-7)


@pytest.mark.gpu
def test_gpu_calc_image_tcc_direct_matches_program(ctx, fx):
    """calcImage + FT_c2r_padded (Module 5) from the program's mask spectrum and TCC."""
    mr, mi = _full_from_window(fx)
    nx = int(fx["Nx"])
    img = ctx.calc_image(mr, mi, fx["tcc"].astype(np.complex128), nx, nx, L, L)
    assert R.rel_l2(_rows(img, fx), fx["tcc_rows"]) < FP32_TOL
    np.testing.assert_allclose(_stats(img), fx["tcc_stats"], rtol=FP32_TOL, atol=1e-7)
    np.testing.assert_allclose(_stats(img), RUN_LOG_TCC_IMAGE, atol=PRINT_ATOL)


@pytest.mark.gpu
def test_gpu_plain_chain_matches_program_k24(ctx, fx, mask, optics):
    """The whole GPU chain in FP64/FP32: TCC -> 24 kernels -> fused mask-to-image (plain form)."""
    import litho_gb300 as Lib
    o = optics
    tcc = ctx.calc_tcc(o["src"], o["sigma"], o["wavelength"], o["NA"], o["defocus"], L, L, o["Nx"], o["Nx"])
    krn, s32, _ = ctx.calc_kernels(tcc, 24)
    img = ctx.image(mask, krn, s32, o["Nx"], o["Nx"], precision=Lib.PREC_FP32)
    assert R.rel_l2(_rows(img, fx), fx["socs_rows_24"]) < FP32_TOL
    np.testing.assert_allclose(_stats(img), fx["socs_stats_24"], rtol=FP32_TOL, atol=1e-7)


@pytest.mark.gpu
def test_gpu_mixed_chain_matches_program_k24(ctx, fx, mask, optics):
    """Mixed form: split-BF16 TCC -> FP64 eigensolve -> split-TF32 tensor-core imaging, batched."""
    import litho_gb300 as Lib
    o = optics
    tcc = ctx.calc_tcc(o["src"], o["sigma"], o["wavelength"], o["NA"], o["defocus"], L, L, o["Nx"], o["Nx"],
                       precision=Lib.TCC_SPLIT_BF16)
    krn, s32, _ = ctx.calc_kernels(tcc, 24)
    ks = ctx.kernel_set(krn, s32, o["Nx"], o["Nx"])
    imgs = ctx.image_batch(ks, np.stack([mask, mask[::-1].copy()]), precision=Lib.PREC_MIXED)
    ks.close()
    assert R.rel_l2(_rows(imgs[0], fx), fx["socs_rows_24"]) < MIXED_TOL
    # the flipped mask's image is the flipped image of the same optics up to the source's symmetry;
    # it is checked against the plain GPU form instead
    plain = ctx.image(mask[::-1].copy(), krn, s32, o["Nx"], o["Nx"], precision=Lib.PREC_FP32)
    assert R.rel_l2(imgs[1], plain) < MIXED_TOL


@pytest.mark.gpu
def test_gpu_calc_image_matches_tcc_direct_golden_512(ctx, golden_optics):
    """litho_calc_image against the reference's checked-in TCC-direct golden
    (source/TCC_HLS/hls/tb/golden/image_expected_512x512.bin), GPU end to end:
    mask spectrum, TCC and TCC-direct image all from the library."""
    ig = load_golden("image_golden.npz")
    m256 = np.unpackbits(ig["mask256_bits"]).reshape(256, 256).astype(np.float32)
    m512 = R.create_mask(m256, 512, 512)
    g = golden_optics
    r, i = ctx.fft_mask(m512)
    tcc = ctx.calc_tcc(g["src"], g["sigma"], g["wavelength"], g["NA"], g["defocus"], 512, 512, g["Nx"], g["Nx"])
    img = ctx.calc_image(r, i, tcc, g["Nx"], g["Nx"], 512, 512)
    assert R.rel_l2(img, ig["image512"]) < FP32_TOL
