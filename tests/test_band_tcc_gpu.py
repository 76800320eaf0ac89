"""The SOCS band as the bilinear form of the rank-K TCC (LITHO_BAND_TCC) against the
per-kernel FFT form (LITHO_BAND_FFT) and the oracle.

calcSOCS (litho.cpp:795-1006) sums s_k |IFFT(K_k . M)|^2 on the conv grid; the
interpolation (litho.cpp:674-754) keeps the band |f| <= 2N of that intensity.  The TCC
form computes the same band as sum_{p-q=f} M(p) conj(M(q)) T(p, q) with
T = sum_k s_k K_k K_k^H, so both forms must give the oracle's image (FT_r2c_padded +
calcSOCS + FI in FP64) within the same tolerance, and each other to FP32 rounding.
"""
import numpy as np
import pytest

from oracle import np_ref as R

pytestmark = pytest.mark.gpu

PLAIN_TOL, MIXED_TOL, FORMS_TOL = 1e-5, 1e-4, 3e-6


def _kernels(src, Lx, Ly, K, NA=0.8, wl=193.0, defocus=0.0):
    sig = R.get_outer_sigma(src)
    nx, ny = R.optics_nx(NA, Lx, sig, wl), R.optics_nx(NA, Ly, sig, wl)
    tcc = R.calc_tcc(src, sig, wl, NA, defocus, Lx, Ly, nx, ny)
    krn, scales, _ = R.calc_kernels(tcc, K)
    return krn, scales, nx, ny


def _cases():
    from litho_gb300 import synth
    ann = R.normalize_source(R.create_annular(41, 0.6, 0.9))
    quasar = synth.quasar_source(2000)[0]
    return {
        # (Lx, Ly, source, K): the metric's optics (Nx = 8, K = 24), the golden-like
        # annular 512^2 (Nx = 4), a rectangular window (Nx != Ny) and the 256^2 Nx = 2 case
        "1024_quasar_k24": (1024, 1024, quasar, 24),
        "512_annular_k10": (512, 512, ann, 10),
        "512x256_annular_k12": (512, 256, ann, 12),
        "256_annular_k8": (256, 256, ann, 8),
        # Nx = 6: the kernel without a compile-time support size; Fx = 1024 > Lx
        "768_annular_k10": (768, 768, ann, 10),
        # Nx = 1: two lanes per image, sixteen images per warp
        "128_annular_k4": (128, 128, ann, 4),
        # Nx = 16: the table cut into row chunks (several partial groups)
        "2048_annular_k12": (2048, 2048, ann, 12),
    }


@pytest.fixture(scope="module", params=list(_cases().keys()))
def case(request):
    from litho_gb300 import synth
    Lx, Ly, src, K = _cases()[request.param]
    krn, scales, nx, ny = _kernels(src, Lx, Ly, K)
    seeds = ((0.3, 11), (0.5, 12), (0.45, 13)) if Lx * Ly <= 1024 * 1024 else ((0.4, 14),)
    masks = np.stack([synth.density_rect_mask(max(Lx, Ly), d, seed=s)[:Ly, :Lx]
                      for d, s in seeds]).astype(np.float32)
    masks = np.ascontiguousarray(masks)
    ref = [R.mask_to_image(m, krn, scales, nx, ny) for m in masks]
    return dict(name=request.param, krn=krn, scales=scales, nx=nx, ny=ny, masks=masks, ref=ref)


@pytest.fixture(scope="module")
def ctx():
    import litho_gb300 as L
    c = L.Context(0)
    yield c
    c.close()


def _run(ctx, case, method, prec):
    import litho_gb300 as L
    ctx.set_band_method(method)
    try:
        ks = ctx.kernel_set(case["krn"], case["scales"], case["nx"], case["ny"])
        out = ctx.image_batch(ks, case["masks"], precision=prec)
        ks.close()
    finally:
        ctx.set_band_method(L.BAND_AUTO)
    return out


def test_tcc_band_matches_fft_band_and_oracle(ctx, case):
    import litho_gb300 as L
    tcc = _run(ctx, case, L.BAND_TCC, L.PREC_FP32)
    fft = _run(ctx, case, L.BAND_FFT, L.PREC_FP32)
    for i, r in enumerate(case["ref"]):
        assert R.rel_l2(tcc[i], r) < PLAIN_TOL, (case["name"], i)
        assert R.rel_l2(fft[i], r) < PLAIN_TOL, (case["name"], i)
        assert R.rel_l2(tcc[i], fft[i]) < FORMS_TOL, (case["name"], i)


def test_tcc_band_mixed(ctx, case):
    import litho_gb300 as L
    if case["masks"].shape[2] % 32:
        pytest.skip("mixed form needs Lx % 32 == 0")
    got = _run(ctx, case, L.BAND_TCC, L.PREC_MIXED)
    for i, r in enumerate(case["ref"]):
        assert R.rel_l2(got[i], r) < MIXED_TOL, (case["name"], i)


def test_default_takes_one_of_the_two_forms(ctx, case):
    import litho_gb300 as L
    auto = _run(ctx, case, L.BAND_AUTO, L.PREC_FP32)
    tcc = _run(ctx, case, L.BAND_TCC, L.PREC_FP32)
    fft = _run(ctx, case, L.BAND_FFT, L.PREC_FP32)
    assert np.array_equal(auto, tcc) or np.array_equal(auto, fft)


def test_default_is_tcc_band_for_large_batches_at_nx8(ctx):
    # 256 masks of 1024^2 with the metric's Nx = 8, K = 24: the cost model takes the TCC form
    import torch
    import litho_gb300 as L
    from litho_gb300 import synth
    krn, scales, nx, ny = _kernels(synth.quasar_source(2000)[0], 1024, 1024, 24)
    assert nx == 8
    m = torch.from_numpy(np.stack([synth.density_rect_mask(1024, 0.3 + 0.001 * i, seed=200 + i)
                                   for i in range(4)]).astype(np.float32)).cuda().repeat(64, 1, 1)
    torch.cuda.synchronize()  # the context images on its own stream
    outs = {}
    ks = ctx.kernel_set(krn, scales, nx, ny)
    try:
        for name, meth in (("auto", L.BAND_AUTO), ("tcc", L.BAND_TCC)):
            ctx.set_band_method(meth)
            outs[name] = ctx.image_batch(ks, m, precision=L.PREC_MIXED)
            ctx.synchronize()
    finally:
        ctx.set_band_method(L.BAND_AUTO)
        ks.close()
    assert torch.equal(outs["auto"], outs["tcc"])


@pytest.mark.parametrize("prec_name,tol", [("fp32", PLAIN_TOL), ("mixed", MIXED_TOL)])
def test_batch_plan_under_each_band_method(ctx, prec_name, tol):
    import torch
    import litho_gb300 as L
    from litho_gb300 import synth
    Lx, Ly, src, K = _cases()["512_annular_k10"]
    krn, scales, nx, ny = _kernels(src, Lx, Ly, K)
    items = [(0, 512, 512), (0, 256, 256), (0, 384, 384)]
    masks = [synth.density_rect_mask(m, 0.35, seed=70 + i) for i, (_, m, _) in enumerate(items)]
    refs = [R.mask_to_image(R.create_mask(m, 512, 512), krn, scales, nx, ny) for m in masks]
    for method, name in ((L.BAND_FFT, "fft"), (L.BAND_TCC, "tcc")):
        ctx.set_band_method(method)
        try:
            ks = ctx.kernel_set(krn, scales, nx, ny)
            prec = L.PREC_FP32 if prec_name == "fp32" else L.PREC_MIXED
            plan = L.BatchPlan(ctx, [ks], [512], items, precision=prec)
            for i, m in enumerate(masks):
                plan.mask(i).copy_(torch.from_numpy(m))
            torch.cuda.synchronize()
            plan.run()
            ctx.synchronize()
            for i, r in enumerate(refs):
                assert R.rel_l2(plan.image(i).cpu().numpy(), r) < tol, (name, prec_name, i)
            assert [c["band"] for c in plan.describe()["classes"]] == [name]
            plan.close()
            ks.close()
        finally:
            ctx.set_band_method(L.BAND_AUTO)


def test_band_method_rejects_bad_values(ctx):
    import litho_gb300 as L
    with pytest.raises(L.LithoError) as ei:
        ctx.set_band_method(3)
    assert ei.value.status == L.LITHO_ERR_ARG
