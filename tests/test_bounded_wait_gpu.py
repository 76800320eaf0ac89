"""The bounded device-side waits give up, report, and leave the context usable.

Every mbarrier wait in the tensor-core kernels is bounded (about one second);
on expiry the kernel flags the error, drains what it issued, frees its tensor
memory and returns, and the host reports LITHO_ERR_TIMEOUT.  The reference has
no such path: its failure handling is assert and exit (common/file_io.cpp:
137-150, litho.cpp:246-248).

The failure is made on purpose and safely: litho_ctx_set_test_stall makes the
mixed window DFT's TMA producer stop issuing loads part-way through (a barrier
that nothing completes), so the consumers' waits run out.  No fault, trap or
unbounded loop is involved, and every load that was issued lands before the
kernel exits.
"""
import time

import numpy as np
import pytest

from oracle import np_ref as R

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-4


@pytest.fixture(scope="module")
def case(golden_optics):
    from litho_gb300 import synth
    g = golden_optics
    krn, scales, _ = R.calc_kernels(g["tcc"], 10)
    masks = np.stack([synth.rect_mask(512, 30, 8, 64, seed=s) for s in (3, 4, 5)])
    ref = [R.mask_to_image(m, krn, scales, g["Nx"], g["Nx"]) for m in masks]
    return dict(krn=krn, scales=scales, Nx=g["Nx"], masks=masks, ref=ref)


def _check(images, ref):
    for img, r in zip(images, ref):
        assert R.rel_l2(img, r) < MIXED_TOL


# chunk 0: the producer issues nothing; chunk 1: it issues one chunk's loads and stops, so the
# kernel must also wait for that load to land before it frees its shared memory (at 512^2 every
# CTA's tile spans two chunks, so both are reached)
@pytest.mark.parametrize("chunk", [0, 1])
def test_stalled_producer_times_out_and_context_recovers(case, chunk):
    import torch
    import litho_gb300 as Lib
    with Lib.Context(0) as ctx:
        ks = ctx.kernel_set(case["krn"], case["scales"], case["Nx"], case["Nx"])
        _check(ctx.image_batch(ks, case["masks"], precision=Lib.PREC_MIXED), case["ref"])
        ctx.set_test_stall(chunk)
        t0 = time.perf_counter()
        with pytest.raises(Lib.LithoError) as ei:
            ctx.image_batch(ks, case["masks"], precision=Lib.PREC_MIXED)
        elapsed = time.perf_counter() - t0
        assert ei.value.status == Lib.LITHO_ERR_TIMEOUT
        assert "wait gave up" in str(ei.value)
        # the waits are bounded at about a second each, and the stalled CTAs wait side by side
        assert elapsed < 20.0, elapsed
        ctx.set_test_stall(-1)
        # same context: host buffers, then device buffers with an explicit synchronise
        _check(ctx.image_batch(ks, case["masks"], precision=Lib.PREC_MIXED), case["ref"])
        dm = torch.from_numpy(case["masks"]).cuda()
        torch.cuda.synchronize()  # the context images on its own stream
        out = ctx.image_batch(ks, dm, precision=Lib.PREC_MIXED)
        ctx.synchronize()
        _check(out.cpu().numpy(), case["ref"])
        # the device itself is still usable by other work
        assert float(torch.ones(1024, device="cuda").sum().item()) == 1024.0


def test_stall_hook_rejects_bad_values():
    import litho_gb300 as Lib
    with Lib.Context(0) as ctx:
        with pytest.raises(Lib.LithoError) as ei:
            ctx.set_test_stall(-2)
        assert ei.value.status == Lib.LITHO_ERR_ARG
