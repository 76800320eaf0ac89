"""Batched imaging of masks of uneven sizes in one CUDA graph (litho_batch_plan_*).

Each mask is imaged in the period of its size class; a mask smaller than the
period is centred in it (common/mask.cpp:31-60 createMask), so the oracle is
create_mask + FT_r2c_padded + calcSOCS on the padded mask.
"""
import numpy as np
import pytest

from oracle import np_ref as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L():
    import litho_gb300
    return litho_gb300


@pytest.fixture(scope="module")
def ctx(L):
    c = L.Context(0)
    yield c
    c.close()


def _kernels(Lp, src, K):
    sig = R.get_outer_sigma(src)
    nx = R.optics_nx(0.8, Lp, sig, 193.0)
    tcc = R.calc_tcc(src, sig, 193.0, 0.8, 0.0, Lp, Lp, nx, nx)
    krns, scales, _ = R.calc_kernels(tcc, K)
    return krns, scales, nx


@pytest.fixture(scope="module")
def classes():
    from litho_gb300 import synth
    k0 = _kernels(512, synth.annular_source(21, 0.6, 0.9), 8)
    k1 = _kernels(1024, synth.quasar_source(2000)[0], 12)
    return [(512, k0), (1024, k1)]


@pytest.mark.parametrize("prec_name,tol", [("fp32", 1e-5), ("mixed", 1e-4)])
def test_batch_plan_uneven_sizes(ctx, L, classes, prec_name, tol):
    import torch
    from litho_gb300 import synth
    prec = L.PREC_FP32 if prec_name == "fp32" else L.PREC_MIXED
    sets = [ctx.kernel_set(k[0], k[1], k[2], k[2]) for _, k in classes]
    periods = [p for p, _ in classes]
    # (class, Lx, Ly): several sizes per class, whose window DFTs run as parallel branches;
    # the rectangular ones share a row or column length (and so a twiddle table) with others
    items = [(0, 256, 256), (1, 512, 512), (0, 512, 512), (1, 1024, 1024), (1, 768, 768), (0, 256, 256),
             (1, 768, 1024), (0, 512, 256)]
    plan = L.BatchPlan(ctx, sets, periods, items, precision=prec)
    masks = [np.ascontiguousarray(synth.density_rect_mask(max(x, y), 0.2 + 0.06 * i, seed=60 + i)[:y, :x])
             for i, (_, x, y) in enumerate(items)]
    for i, m in enumerate(masks):
        plan.mask(i).copy_(torch.from_numpy(m))
    torch.cuda.synchronize()
    first = None
    for rep in range(2):   # the captured graph is replayed, to the same bits
        plan.run()
        ctx.synchronize()
        imgs = [plan.image(i).clone() for i in range(len(items))]
        if first is None:
            first = imgs
        else:
            assert all(torch.equal(a, b) for a, b in zip(first, imgs)), prec_name
        for i, (c, m, _) in enumerate(items):
            Lp = periods[c]
            krns, scales, nx = classes[c][1]
            ref = R.mask_to_image(R.create_mask(masks[i], Lp, Lp), krns, scales, nx, nx)
            got = plan.image(i).cpu().numpy()
            assert R.rel_l2(got, ref) < tol, (prec_name, rep, i)
    info = plan.describe()
    assert info["graph"] is True
    assert {c["period"] for c in info["classes"]} == {512, 1024}
    assert all(c["candidates"] >= 0 and (c["band"] == "tcc" or c["conv_n"] >= 32) for c in info["classes"])
    plan.close()
    for s in sets:
        s.close()


@pytest.mark.parametrize("prec_name,tol", [("fp32", 1e-5), ("mixed", 1e-4)])
def test_batch_plan_many_sizes_in_one_class(ctx, L, classes, prec_name, tol):
    """Six mask sizes in one class: the mixed window DFT takes up to four sizes per launch
    (a tensor map pair, row twiddles and a tile range each), so this class runs two launches
    (4 + 2 sizes) into the same partial array; the plain form runs six branches."""
    import torch
    from litho_gb300 import synth
    prec = L.PREC_FP32 if prec_name == "fp32" else L.PREC_MIXED
    Lp, k = classes[0]
    ks = ctx.kernel_set(k[0], k[1], k[2], k[2])
    items = [(0, 512, 512), (0, 64, 64), (0, 384, 384), (0, 128, 96), (0, 256, 256), (0, 192, 320), (0, 64, 64)]
    plan = L.BatchPlan(ctx, [ks], [Lp], items, precision=prec)
    masks = [np.ascontiguousarray(synth.density_rect_mask(max(x, y), 0.3 + 0.04 * i, seed=90 + i)[:y, :x])
             for i, (_, x, y) in enumerate(items)]
    for i, m in enumerate(masks):
        plan.mask(i).copy_(torch.from_numpy(m))
    torch.cuda.synchronize()
    plan.run()
    ctx.synchronize()
    krns, scales, nx = k
    for i in range(len(items)):
        ref = R.mask_to_image(R.create_mask(masks[i], Lp, Lp), krns, scales, nx, nx)
        assert R.rel_l2(plan.image(i).cpu().numpy(), ref) < tol, (prec_name, i)
    plan.close()
    ks.close()


def test_batch_plan_rejects_bad_items(ctx, L, classes):
    sets = [ctx.kernel_set(k[0], k[1], k[2], k[2]) for _, k in classes]
    with pytest.raises(L.LithoError):
        L.BatchPlan(ctx, sets, [512, 1024], [(0, 1024, 1024)])    # mask larger than its period
    with pytest.raises(L.LithoError):
        L.BatchPlan(ctx, sets, [500, 1024], [(0, 256, 256)])      # period not a power of two
    for s in sets:
        s.close()
