"""The pipelined mixed-precision batch (litho_ctx_set_pipeline).

A LITHO_PREC_MIXED batch of device-resident masks of at least two chunks runs
as a two-stream pipeline: window DFT and interpolation contraction persistent on
a capped number of SMs, taking their tiles from a global counter, with each
chunk's SOCS and interpolation rows on a second stream.  Same bar as the mixed
form (<= 1e-4 relative L2 against the FP64 oracle); the pipelined and
unpipelined calls differ only in how partial sums are split, so they agree far
closer; repeated calls are bitwise identical (every tile is computed the same
way whichever CTA takes it, and the tile counters reset themselves).
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


def _kernels(Lp, K):
    from litho_gb300 import synth
    src = synth.quasar_source(2000)[0]
    sig = R.get_outer_sigma(src)
    nx = R.optics_nx(0.8, Lp, sig, 193.0)
    tcc = R.calc_tcc(src, sig, 193.0, 0.8, 0.0, Lp, Lp, nx, nx)
    krns, scales, _ = R.calc_kernels(tcc, K)
    return krns, scales, nx


def _masks(Lp, n, seed0):
    from litho_gb300 import synth
    base = [synth.manhattan_mask(Lp, seed=seed0 + i) for i in range(8)]
    return np.stack([base[i % 8] * np.float32(1 - 0.25 * (i // 8 % 2)) for i in range(n)])


@pytest.mark.parametrize("Lp,K,n,chunk,sms", [(512, 10, 160, 64, 0), (512, 10, 150, 48, 100), (1024, 24, 128, 64, 0)])
def test_pipelined_batch(L, Lp, K, n, chunk, sms):
    import torch
    krns, scales, nx = _kernels(Lp, K)
    masks = _masks(Lp, n, 60)
    dm = torch.from_numpy(masks).cuda()
    with L.Context(0) as ctx:
        ks = ctx.kernel_set(krns, scales, nx, nx)
        ctx.set_pipeline(chunk, sms)
        a = ctx.image_batch(ks, dm, precision=L.PREC_MIXED)
        b = ctx.image_batch(ks, dm, precision=L.PREC_MIXED)
        ctx.synchronize()
        a, b = a.cpu().numpy(), b.cpu().numpy()
        ctx.set_pipeline(0)
        c = ctx.image_batch(ks, dm, precision=L.PREC_MIXED)
        ctx.synchronize()
        c = c.cpu().numpy()
        ks.close()
    assert np.array_equal(a, b)
    for i in (0, chunk - 1, chunk, n // 2, n - 1):
        ref = R.mask_to_image(masks[i], krns, scales, nx, nx)
        assert R.rel_l2(a[i], ref) < TOL_MIXED, i
    assert max(R.rel_l2(a[i], c[i]) for i in range(n)) < 1e-5


def test_pipeline_knob_rejects_bad_values(L):
    with L.Context(0) as ctx:
        for chunk, sms in ((-1, 0), (64, -1), (64, 100000)):
            with pytest.raises(L.LithoError) as e:
                ctx.set_pipeline(chunk, sms)
            assert e.value.status == L.LITHO_ERR_ARG
