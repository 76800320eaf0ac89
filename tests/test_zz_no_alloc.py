"""litho_image_noalloc: the imaging entry point for callers that cannot allocate.

Callers such as a latency-critical loop (cudaMalloc/cudaFree synchronise the
whole device) or a plugin whose host application owns the device memory budget
cannot let the library allocate.  litho_image_noalloc takes its intermediates
from a fixed array compiled into the library; this test calls it through the C
ABI twice in a row (the second call must not be disturbed by what the first left
in the shared array) and checks each image against the regular entry point,
litho_image_batch, within the imaging tolerance (1e-5 relative L2).

This file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import np_ref as R

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _kernels(L_, src):
    sig = R.get_outer_sigma(src)
    nx = R.optics_nx(0.8, L_, sig, 193.0)
    tcc = R.calc_tcc(src, sig, 193.0, 0.8, 0.0, L_, L_, nx, nx)
    krns, scales, _ = R.calc_kernels(tcc, 24)
    return krns, scales, nx


def test_noalloc_matches_image_batch_on_two_calls():
    import torch
    import litho_gb300 as L
    from litho_gb300 import synth

    fn = L.lib().litho_image_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                   C.c_void_p, C.c_void_p]

    krns, scales, nx = _kernels(1024, synth.quasar_source(2000)[0])
    masks = np.stack([synth.manhattan_mask(1024, seed=31), synth.density_rect_mask(1024, 0.35, seed=32)])
    kr = torch.from_numpy(np.ascontiguousarray(krns.real, np.float32)).cuda()
    ki = torch.from_numpy(np.ascontiguousarray(krns.imag, np.float32)).cuda()
    sc = torch.from_numpy(np.ascontiguousarray(scales, np.float32)).cuda()
    dm = torch.from_numpy(masks).cuda()

    with L.Context(0) as ctx:
        ks = ctx.kernel_set(krns, scales, nx, nx)
        expect = ctx.image_batch(ks, masks)
        ks.close()

    stream = torch.cuda.current_stream().cuda_stream
    for i in range(2):
        out = torch.full((1024, 1024), float("nan"), dtype=torch.float32, device="cuda")
        st = fn(C.c_void_p(dm[i].data_ptr()), 1024, 1024, C.c_void_p(kr.data_ptr()), C.c_void_p(ki.data_ptr()),
                C.c_void_p(sc.data_ptr()), 24, nx, nx, C.c_void_p(out.data_ptr()), C.c_void_p(stream))
        assert st == L.LITHO_OK
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert R.rel_l2(got, expect[i]) < TOL, i


def _noalloc_fn():
    import litho_gb300 as L
    fn = L.lib().litho_image_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                   C.c_void_p, C.c_void_p]
    return fn


# (Lx, Ly, wavelength): 250 x 300 at 55 nm gives Nx = 6, Ny = 8 (rectangular period, Lx % 4 != 0, the
# 64-point conv grid); 130 x 130 at 26 nm gives Nx = Ny = 7 (the 32-point conv grid, Lx % 4 != 0)
SHAPES = [(250, 300, 55.0), (130, 130, 26.0)]


@pytest.mark.parametrize("Lx,Ly,lam", SHAPES)
def test_noalloc_other_shapes_match_the_oracle(Lx, Ly, lam):
    import torch
    import litho_gb300 as L
    from litho_gb300 import synth
    fn = _noalloc_fn()
    src = synth.annular_source(21, 0.6, 0.9)
    sig = R.get_outer_sigma(src)
    nx, ny = R.optics_nx(0.8, Lx, sig, lam), R.optics_nx(0.8, Ly, sig, lam)
    tcc = R.calc_tcc(src, sig, lam, 0.8, 0.0, Lx, Ly, nx, ny)
    nk = 12
    krns, scales, _ = R.calc_kernels(tcc, nk)
    rng = np.random.default_rng(Lx + Ly)
    mask = (rng.random((Ly, Lx)) < 0.4).astype(np.float32)
    ref = R.mask_to_image(mask, krns, scales, nx, ny)
    kr = torch.from_numpy(np.ascontiguousarray(krns.real, np.float32)).cuda()
    ki = torch.from_numpy(np.ascontiguousarray(krns.imag, np.float32)).cuda()
    sc = torch.from_numpy(np.ascontiguousarray(scales, np.float32)).cuda()
    dm = torch.from_numpy(mask).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        out = torch.full((Ly, Lx), float("nan"), dtype=torch.float32, device="cuda")
        st = fn(C.c_void_p(dm.data_ptr()), Lx, Ly, C.c_void_p(kr.data_ptr()), C.c_void_p(ki.data_ptr()),
                C.c_void_p(sc.data_ptr()), nk, nx, ny, C.c_void_p(out.data_ptr()), C.c_void_p(stream))
        assert st == L.LITHO_OK
        torch.cuda.synchronize()
        assert R.rel_l2(out.cpu().numpy(), ref) < TOL, (Lx, Ly, nx, ny)


def test_noalloc_call_allocates_no_device_memory():
    """After a first call (which looks up the scratch array's address), further calls leave the
    device's free memory unchanged: nothing is allocated, by the library or for it."""
    import torch
    import litho_gb300 as L
    from litho_gb300 import synth
    fn = _noalloc_fn()
    krns, scales, nx = _kernels(1024, synth.quasar_source(2000)[0])
    kr = torch.from_numpy(np.ascontiguousarray(krns.real, np.float32)).cuda()
    ki = torch.from_numpy(np.ascontiguousarray(krns.imag, np.float32)).cuda()
    sc = torch.from_numpy(np.ascontiguousarray(scales, np.float32)).cuda()
    dm = torch.from_numpy(synth.manhattan_mask(1024, seed=33)).cuda()
    out = torch.empty((1024, 1024), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream

    def call():
        st = fn(C.c_void_p(dm.data_ptr()), 1024, 1024, C.c_void_p(kr.data_ptr()), C.c_void_p(ki.data_ptr()),
                C.c_void_p(sc.data_ptr()), 24, nx, nx, C.c_void_p(out.data_ptr()), C.c_void_p(stream))
        assert st == L.LITHO_OK

    call()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        call()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_sizes_beyond_its_limits():
    import litho_gb300 as L
    fn = L.lib().litho_image_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                   C.c_void_p, C.c_void_p]
    dummy = C.c_void_p(16)  # never dereferenced: the size checks come first
    assert fn(dummy, 8192, 8192, dummy, dummy, dummy, 24, 8, 8, dummy, None) == L.LITHO_ERR_ARG
    assert fn(dummy, 1024, 1024, dummy, dummy, dummy, 65, 8, 8, dummy, None) == L.LITHO_ERR_ARG
    assert fn(dummy, 1024, 1024, dummy, dummy, dummy, 24, 17, 8, dummy, None) == L.LITHO_ERR_ARG
