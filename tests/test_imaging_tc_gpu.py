"""GPU parity of the mixed-precision (tcgen05 split-TF32) imaging path.

Bar (stated by the path's contract for the mixed-precision form): <= 1e-4
relative L2 against the FP64 oracle.  Shapes cover every tensor-core template:
Nx=4 (N=16, one K block), Nx=8 (N=32, two K blocks), Nx=16 (N=48, three K
blocks with 64-wide X tiles), and images that are not multiples of the tiles.
"""
import numpy as np
import pytest

from oracle import np_ref as R

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-4


@pytest.fixture(scope="module")
def L():
    import litho_gb300
    return litho_gb300


@pytest.fixture(scope="module")
def ctx(L):
    c = L.Context(0)
    yield c
    c.close()


def _kernels(Lp, src, K, defocus=0.0):
    sig = R.get_outer_sigma(src)
    nx = R.optics_nx(0.8, Lp, sig, 193.0)
    tcc = R.calc_tcc(src, sig, 193.0, 0.8, defocus, Lp, Lp, nx, nx)
    krns, scales, _ = R.calc_kernels(tcc, K)
    return krns, scales, nx


@pytest.fixture(scope="module")
def quasar():
    from litho_gb300 import synth
    return synth.quasar_source(2000)[0]


def _mixed(ctx, L, masks, krns, scales, nx):
    ks = ctx.kernel_set(krns, scales, nx, nx)
    try:
        return ctx.image_batch(ks, masks, precision=L.PREC_MIXED)
    finally:
        ks.close()


@pytest.mark.parametrize("Lp,K", [(512, 10), (1024, 24)])
def test_mixed_matches_oracle(ctx, L, quasar, Lp, K):
    from litho_gb300 import synth
    krns, scales, nx = _kernels(Lp, quasar, K)
    masks = np.stack([synth.manhattan_mask(Lp, seed=40 + i) for i in range(2)])
    out = _mixed(ctx, L, masks, krns, scales, nx)
    for i in range(2):
        ref = R.mask_to_image(masks[i], krns, scales, nx, nx)
        err = R.rel_l2(out[i], ref)
        assert err < TOL_MIXED, (Lp, i, err)


def test_mixed_nx16_2048(ctx, L, quasar):
    from litho_gb300 import synth
    krns, scales, nx = _kernels(2048, quasar, 24)
    assert nx == 16
    m = synth.density_rect_mask(2048, 0.4, seed=9)
    out = _mixed(ctx, L, m[None], krns, scales, nx)
    ref = R.mask_to_image(m, krns, scales, nx, nx)
    assert R.rel_l2(out[0], ref) < TOL_MIXED


def test_mixed_grey_mask_and_ragged_sizes(ctx, L):
    from litho_gb300 import synth
    src = synth.annular_source(21, 0.6, 0.9)
    rng = np.random.default_rng(5)
    for Ly, Lx in ((500, 500), (200, 300), (384, 256)):
        krns, scales, nx = _kernels(max(Lx, Ly), src, 8)
        m = (rng.integers(0, 256, size=(Ly, Lx)) / 255.0).astype(np.float32)   # grey levels, not TF32-exact
        out = _mixed(ctx, L, m[None], krns, scales, nx)
        ref = R.mask_to_image(m, krns, scales, nx, nx)
        assert R.rel_l2(out[0], ref) < TOL_MIXED, (Ly, Lx)


def test_mixed_batch_equals_single(ctx, L, quasar):
    from litho_gb300 import synth
    krns, scales, nx = _kernels(1024, quasar, 24)
    masks = np.stack([synth.density_rect_mask(1024, d, seed=s) for s, d in ((1, 0.2), (2, 0.5), (3, 0.6))])
    out = _mixed(ctx, L, masks, krns, scales, nx)
    for i in range(3):
        single = _mixed(ctx, L, masks[i:i + 1], krns, scales, nx)[0]
        assert R.rel_l2(out[i], single) < 1e-6


def test_mixed_unsupported_geometry(ctx, L):
    from litho_gb300 import synth
    src = synth.annular_source(21, 0.6, 0.9)
    krns, scales, nx = _kernels(256, src, 4)
    m = np.zeros((256, 258), np.float32)   # row pitch not a multiple of 16 bytes: no TMA
    with pytest.raises(L.LithoError) as e:
        _mixed(ctx, L, m[None], krns, scales, nx)
    assert e.value.status == L.LITHO_ERR_UNSUPPORTED



@pytest.mark.parametrize("prec,chunk", [("plain", 0), ("mixed", 0), ("mixed", 2 << 20), ("mixed", 1)])
def test_host_buffer_pipeline_matches_device_path(ctx, L, quasar, prec, chunk):
    """Host buffers of 20 masks of 1 MB move through the chunked copy/compute pipeline on
    three staging slots: by default ramped chunks of 1, 2, 3, 3, 3, 3, 2, 2, 1 masks (at
    least eight chunks), with a 2 MB chunk cap 1, 2 x 9, 1, with a 1-byte cap one mask per
    chunk.  The images equal the device-pointer path's."""
    import torch
    from litho_gb300 import synth
    p = L.PREC_MIXED if prec == "mixed" else L.PREC_FP32
    krns, scales, nx = _kernels(512, quasar, 10)
    masks = np.stack([synth.density_rect_mask(512, 0.2 + 0.02 * i, seed=90 + i) for i in range(20)])
    ks = ctx.kernel_set(krns, scales, nx, nx)
    try:
        ctx.set_host_chunk(chunk)
        host = ctx.image_batch(ks, masks, precision=p)          # numpy in, numpy out
        dm = torch.from_numpy(masks).cuda()
        torch.cuda.synchronize()  # the context images on its own stream
        dev = ctx.image_batch(ks, dm, precision=p)
        ctx.synchronize()
        dev = dev.cpu().numpy()
    finally:
        ctx.set_host_chunk(0)
        ks.close()
    for i in range(20):
        assert R.rel_l2(host[i], dev[i]) < 1e-6, i
    ref = R.mask_to_image(masks[17], krns, scales, nx, nx)
    assert R.rel_l2(host[17], ref) < (TOL_MIXED if prec == "mixed" else 1e-5)


@pytest.mark.parametrize("prec_name", ["mixed", "plain"])
def test_images_are_deterministic(L, quasar, prec_name):
    """A fresh context images 256 masks of 1024^2 (four masks repeated) in each form: every
    copy of a mask gives the same image bit for bit, within the first call and across calls.  (A DC row of
    the FI contraction's epilogue once raced with a warp two tiles ahead and corrupted a
    32 x 32 slab of the first call.)"""
    import torch
    from litho_gb300 import synth
    krns, scales, nx = _kernels(1024, quasar, 24)
    c = L.Context(0)
    try:
        ks = c.kernel_set(krns, scales, nx, nx)
        m = torch.from_numpy(np.stack([synth.density_rect_mask(1024, 0.3 + 0.001 * i, seed=200 + i)
                                       for i in range(4)]).astype(np.float32)).cuda().repeat(64, 1, 1)
        torch.cuda.synchronize()  # the context images on its own stream
        prec = L.PREC_MIXED if prec_name == "mixed" else L.PREC_FP32
        first = c.image_batch(ks, m, precision=prec)
        c.synchronize()
        for i in range(4, 256):
            assert torch.equal(first[i], first[i % 4]), i
        again = c.image_batch(ks, m, precision=prec)
        c.synchronize()
        assert torch.equal(first, again)
        ks.close()
    finally:
        c.close()
