"""Rectangular periods: Nx != Ny (litho.cpp:1300-1301 computes them from Lx and Ly separately).
1024 x 512 gives Nx = 8, Ny = 4 (64 x 64 conv grid); 2048 x 1024 gives Nx = 16, Ny = 8 (128 x 128
conv grid), so the eight- and sixteen-lane SOCS kernels run with KX != KY.  Plain and mixed images
are checked against the FP64 oracle, and the 64-grid tmpImgp against the oracle's centred embed."""
import numpy as np
import pytest

from oracle import np_ref as R

pytestmark = pytest.mark.gpu

NA, LAM = 0.8, 193.0
TOL_PLAIN, TOL_MIXED = 1e-5, 1e-4


@pytest.fixture(scope="module")
def ctx():
    import litho_gb300 as L
    c = L.Context(0)
    yield c
    c.close()


def _optics(Lx, Ly, nk):
    src = R.normalize_source(R.create_annular(21, 0.6, 0.9))
    sig = R.get_outer_sigma(src)
    nx, ny = R.optics_nx(NA, Lx, sig, LAM), R.optics_nx(NA, Ly, sig, LAM)
    tcc = R.calc_tcc(src, sig, LAM, NA, 0.0, Lx, Ly, nx, ny)
    krns, scales, _ = R.calc_kernels(tcc, nk)
    return krns, scales, nx, ny


@pytest.mark.parametrize("Lx,Ly,want", [(1024, 512, (8, 4)), (2048, 1024, (16, 8))])
def test_rect_period_images(ctx, Lx, Ly, want):
    import litho_gb300 as L
    from litho_gb300 import synth
    krns, scales, nx, ny = _optics(Lx, Ly, 16)
    assert (nx, ny) == want
    m = synth.density_rect_mask(max(Lx, Ly), 0.4, seed=21)[:Ly, :Lx].copy()
    ref = R.mask_to_image(m, krns, scales, nx, ny)
    plain = ctx.image(m, krns, scales, nx, ny)
    assert plain.shape == (Ly, Lx)
    assert R.rel_l2(plain, ref) < TOL_PLAIN
    ks = ctx.kernel_set(krns, scales, nx, ny)
    try:
        mixed = ctx.image_batch(ks, m[None], precision=L.PREC_MIXED)[0]
    finally:
        ks.close()
    assert R.rel_l2(mixed, ref) < TOL_MIXED


def test_rect_period_tmpimgp_64(ctx):
    krns, scales, nx, ny = _optics(1024, 512, 12)
    from litho_gb300 import synth
    m = synth.density_rect_mask(1024, 0.3, seed=22)[:512, :].copy()
    mskf = R.ft_r2c_padded(m, 1024, 512)
    ref_img, ref_tmp = R.calc_socs(mskf, 1024, 512, krns, scales, len(scales), nx, ny, 64, None)
    img, tmp = ctx.calc_socs(mskf.real.astype(np.float32), mskf.imag.astype(np.float32), krns, scales,
                             nx, ny, 1024, 512, want_tmpimgp=True, conv_n=64)
    assert R.rel_l2(tmp, ref_tmp) < TOL_PLAIN
    assert R.rel_l2(img, ref_img) < TOL_PLAIN
