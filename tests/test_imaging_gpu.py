"""GPU parity of the imaging path (FT_r2c_padded, calcSOCS, FI) against the FP64 oracle.

Bar (stated by the path's contract): the FP32 GPU path matches the reference
algorithm within 1e-5 relative L2.
"""
import numpy as np
import pytest

from conftest import load_golden
from oracle import np_ref as R

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def L():
    import litho_gb300
    return litho_gb300


@pytest.fixture(scope="module")
def ctx(L):
    c = L.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def golden_kernels(golden_optics):
    krns, scales, _ = R.calc_kernels(golden_optics["tcc"], 10)
    return krns, scales


@pytest.fixture(scope="module")
def config2():
    """1024^2 Manhattan mask, quasar source (~2000 points), NA 0.8, lambda 193, K=24."""
    from litho_gb300 import synth
    src, S, n = synth.quasar_source(2000)
    sig = R.get_outer_sigma(src)
    nx = R.optics_nx(0.8, 1024, sig, 193.0)
    tcc = R.calc_tcc(src, sig, 193.0, 0.8, 0.0, 1024, 1024, nx, nx)
    krns, scales, _ = R.calc_kernels(tcc, 24)
    mask = synth.manhattan_mask(1024, seed=2)
    return dict(mask=mask, krns=krns, scales=scales, Nx=nx, tcc=tcc)


def _golden_mask512():
    ig = load_golden("image_golden.npz")
    m256 = np.unpackbits(ig["mask256_bits"]).reshape(256, 256).astype(np.float32)
    return R.create_mask(m256, 512, 512)


def test_fft_mask_matches_oracle(ctx):
    for shape in ((512, 512), (500, 500), (256, 384), (130, 70)):
        rng = np.random.default_rng(sum(shape))
        m = (rng.random(shape) > 0.5).astype(np.float32)
        r, i = ctx.fft_mask(m)
        ref = R.ft_r2c_padded(m, R.next_pow2(shape[1]), R.next_pow2(shape[0]))
        got = r.astype(np.float64) + 1j * i.astype(np.float64)
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < TOL, shape


def test_calc_socs_matches_oracle_128(ctx, golden_optics, golden_kernels):
    """litho.cpp calcSOCS: 128^2 conv grid, embed 94, tmpImgp + FI + crop."""
    mask = _golden_mask512()
    mskf = R.ft_r2c_padded(mask, 512, 512)
    krns, scales = golden_kernels
    nx = golden_optics["Nx"]
    ref_img, ref_tmp = R.calc_socs(mskf, 512, 512, krns, scales, 10, nx, nx, 128, 94)
    img, tmp = ctx.calc_socs(mskf.real.astype(np.float32), mskf.imag.astype(np.float32), krns, scales,
                             nx, nx, 512, 512, want_tmpimgp=True)
    assert R.rel_l2(img, ref_img) < TOL
    assert R.rel_l2(tmp, ref_tmp) < TOL


def test_calc_socs_tmpimgp_64(ctx, golden_optics, golden_kernels):
    """64^2 conv grid (eight-lane FFT kernel): tmpImgp and image against the oracle with the
    centred embedding (litho_thread.cpp:847)."""
    mask = _golden_mask512()
    mskf = R.ft_r2c_padded(mask, 512, 512)
    krns, scales = golden_kernels
    nx = golden_optics["Nx"]
    ref_img, ref_tmp = R.calc_socs(mskf, 512, 512, krns, scales, 10, nx, nx, 64, None)
    img, tmp = ctx.calc_socs(mskf.real.astype(np.float32), mskf.imag.astype(np.float32), krns, scales,
                             nx, nx, 512, 512, want_tmpimgp=True, conv_n=64)
    assert tmp.shape == (64, 64)
    assert R.rel_l2(tmp, ref_tmp) < TOL
    assert R.rel_l2(img, ref_img) < TOL


def test_calc_socs_matches_hls_golden_32(ctx, golden_optics):
    """source/SOCS_HLS/data/hls_output_full_32.bin: nk=4 on a 32^2 conv grid."""
    h = load_golden("hls_golden.npz")
    m = (h["mask512_u8"].astype(np.float32) / np.float32(255)).astype(np.float32)
    mskf = R.ft_r2c_padded(R.create_mask(m, 512, 512), 512, 512)
    krns, scales, _ = R.calc_kernels(golden_optics["tcc"], 4)
    nx = golden_optics["Nx"]
    _, tmp = ctx.calc_socs(mskf.real.astype(np.float32), mskf.imag.astype(np.float32), krns, scales,
                           nx, nx, 512, 512, want_tmpimgp=True, conv_n=32)
    assert R.rel_l2(tmp, h["tmpimgp32"]) < 5e-6


def test_full_rank_socs_reproduces_tcc_direct_golden(ctx, golden_optics):
    """All 81 kernels: SOCS == TCC-direct image golden (image_expected_512x512.bin)."""
    mask = _golden_mask512()
    krns, scales, _ = R.calc_kernels(golden_optics["tcc"], 81)
    nx = golden_optics["Nx"]
    img = ctx.image(mask, krns, scales, nx, nx)
    assert R.rel_l2(img, load_golden("image_golden.npz")["image512"]) < TOL


def test_image_fused_config1(ctx):
    """512^2, 40 rectangles, annular 0.6/0.9 on 21^2, NA 0.8, K=10 (defocus 0 and 0.2)."""
    from litho_gb300 import synth
    mask = synth.rect_mask(512, 40, 8, 64, seed=1)
    src = synth.annular_source(21, 0.6, 0.9)
    sig = R.get_outer_sigma(src)
    nx = R.optics_nx(0.8, 512, sig, 193.0)
    for defocus in (0.0, 0.2):
        tcc = R.calc_tcc(src, sig, 193.0, 0.8, defocus, 512, 512, nx, nx)
        krns, scales, _ = R.calc_kernels(tcc, 10)
        ref = R.mask_to_image(mask, krns, scales, nx, nx)
        img = ctx.image(mask, krns, scales, nx, nx)
        assert R.rel_l2(img, ref) < TOL, defocus


def test_image_fused_config2(ctx, config2):
    c = config2
    ref = R.mask_to_image(c["mask"], c["krns"], c["scales"], c["Nx"], c["Nx"])
    img = ctx.image(c["mask"], c["krns"], c["scales"], c["Nx"], c["Nx"])
    assert R.rel_l2(img, ref) < TOL


def test_batch_equals_single_and_device_path(ctx, config2, L):
    import torch
    from litho_gb300 import synth
    c = config2
    masks = np.stack([synth.density_rect_mask(1024, d, seed=s) for s, d in ((5, 0.2), (6, 0.4), (7, 0.6))])
    ks = ctx.kernel_set(c["krns"], c["scales"], c["Nx"], c["Nx"])
    out = ctx.image_batch(ks, masks)
    for b in range(3):
        single = ctx.image(masks[b], c["krns"], c["scales"], c["Nx"], c["Nx"])
        assert np.array_equal(out[b], single) or R.rel_l2(out[b], single) < 1e-6
    dm = torch.from_numpy(masks).cuda()
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    dout = ctx.image_batch(ks, dm)
    torch.cuda.synchronize()
    ctx.set_stream(None)
    assert R.rel_l2(dout.cpu().numpy(), out) < 1e-6
    ref0 = R.mask_to_image(masks[0], c["krns"], c["scales"], c["Nx"], c["Nx"])
    assert R.rel_l2(out[0], ref0) < TOL


def test_non_power_of_two_and_rectangular(ctx, golden_optics, golden_kernels):
    krns, scales = golden_kernels
    nx = golden_optics["Nx"]
    rng = np.random.default_rng(11)
    for Ly, Lx in ((500, 500), (256, 384), (300, 200)):
        m = (rng.random((Ly, Lx)) > 0.6).astype(np.float32)
        ref = R.mask_to_image(m, krns, scales, nx, nx)
        img = ctx.image(m, krns, scales, nx, nx)
        assert R.rel_l2(img, ref) < TOL, (Ly, Lx)


def test_odd_shapes(ctx, golden_optics, golden_kernels, L):
    """Odd mask sizes: rows and columns that are not 16-byte multiples (4-byte copies in the
    window ring), an odd row count in the FI kernel's row pairing (row +y' and -y' from one
    set of sums: the centre row y' = 0 and the unpaired edge row), and the mixed form with an
    odd row count."""
    krns, scales = golden_kernels
    nx = golden_optics["Nx"]
    rng = np.random.default_rng(13)
    for Ly, Lx in ((301, 257), (129, 255), (255, 130)):
        m = (rng.random((Ly, Lx)) > 0.6).astype(np.float32)
        ref = R.mask_to_image(m, krns, scales, nx, nx)
        assert R.rel_l2(ctx.image(m, krns, scales, nx, nx), ref) < TOL, (Ly, Lx)
    m = (rng.random((301, 256)) > 0.6).astype(np.float32)
    ref = R.mask_to_image(m, krns, scales, nx, nx)
    got = ctx.image(m, krns, scales, nx, nx, precision=L.PREC_MIXED)
    assert R.rel_l2(got, ref) < 1e-4


def test_edge_cases_report_status(ctx, golden_kernels, L):
    krns, scales = golden_kernels
    m = np.zeros((512, 512), np.float32)
    # an all-zero mask images to exactly zero
    assert not ctx.image(m, krns, scales, 4, 4).any()
    with pytest.raises(L.LithoError) as e:
        ctx.image(m, krns[:0], scales[:0], 4, 4)
    assert e.value.status == L.LITHO_ERR_ARG
    with pytest.raises(L.LithoError) as e:
        k = np.zeros((1, 41 * 41), np.complex128)
        ctx.image(m, k, np.ones(1, np.float32), 20, 20)
    assert e.value.status == L.LITHO_ERR_UNSUPPORTED
    mskf = R.ft_r2c_padded(m, 512, 512)
    with pytest.raises(L.LithoError) as e:   # 32 < 4*Nx+1 = 33 would alias
        ctx.calc_socs(mskf.real.astype(np.float32), mskf.imag.astype(np.float32),
                      np.zeros((1, 17 * 17), np.complex128), np.ones(1, np.float32), 8, 8, 512, 512, conv_n=32)
    assert e.value.status == L.LITHO_ERR_ARG
