"""CPU checks of the surrogate's oracle (torch float64 autograd restatement of
FNO-2d): its gradient against central finite differences, its parameter layout
against the C ABI's, and the seeded rectangle stream."""
import numpy as np
import pytest

from oracle import fno_ref as F


def _params(rng, L):
    p = F.unpack(np.zeros(F.num_params()))
    th = []
    for name, shp in F.param_shapes():
        n = int(np.prod(shp))
        scale = {"R": 1.0 / 1024, "Pw": 1.0, "Pb": 1.0, "q2b": 0.1}.get(name, 1.0 / np.sqrt(32))
        th.append(scale * (rng.random(n) if name == "R" else rng.uniform(-1, 1, n)))
    return np.concatenate(th)


def test_layout_matches_c_abi():
    import ctypes
    import os
    lib = os.path.join(os.path.dirname(__file__), "..", "fpga-litho-accel_gb300", "litho_gb300",
                       "liblitho_gb300.so")
    if not os.path.exists(lib):
        pytest.skip("library not built")
    f = ctypes.CDLL(lib).litho_surrogate_num_params
    f.restype = ctypes.c_longlong
    assert f() == F.num_params() == 4202945


def test_gradient_matches_finite_differences():
    """Directional derivatives of the loss along random directions (float64)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    L, B = 32, 2
    th = _params(rng, L)
    masks = F.rect_masks(7, 0, B, L, wmin=4, wmax=12)
    tgt = 0.3 + 0.5 * np.roll(masks, 1, axis=2)
    loss, grad = F.loss_and_grad(th, masks, tgt)
    assert np.isfinite(loss) and np.all(np.isfinite(grad))
    m = torch.tensor(masks, dtype=torch.float64)
    t = torch.tensor(tgt, dtype=torch.float64)

    def f(x):
        return float(F.rel_l2_loss(F.forward(torch.tensor(x), m), t))

    for k in range(4):
        d = rng.standard_normal(th.shape[0])
        if k == 0:  # spectral weights only
            o = F.unpack(np.arange(th.shape[0]))["R"].ravel()
            d2 = np.zeros_like(d)
            d2[o] = d[o]
            d = d2
        d /= np.linalg.norm(d)
        h = 1e-5
        fd = (f(th + h * d) - f(th - h * d)) / (2 * h)
        an = float(grad @ d)
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)) + 1e-7, (k, fd, an)


def test_rect_stream_is_seeded_and_sliceable():
    a = F.rect_masks(11, 0, 6, 64, wmin=4, wmax=16)
    b = F.rect_masks(11, 3, 3, 64, wmin=4, wmax=16)
    assert np.array_equal(a[3:], b)
    assert set(np.unique(a)) <= {0.0, 1.0}
    assert 0.05 < a.mean() < 0.9
    assert not np.array_equal(a[0], a[1])
