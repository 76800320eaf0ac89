"""The learned surrogate: an FNO-2d of the SOCS map mask -> aerial image.

``Surrogate`` wraps the ``litho_surrogate_*`` C ABI (forward, loss/gradient,
Adam step; all on the GPU, on device tensors).  ``make_pairs`` builds training
pairs with the GPU SOCS path itself (seeded rectangle masks from
``litho_rect_masks`` imaged by ``litho_image_batch``), and ``train`` is the
training loop (Adam, step-decayed learning rate, mini-batches drawn from the
device-resident pair set).

Every call that takes or returns device tensors runs on torch's current
stream (the context is bound to it for the call), so the results are ordered
with the caller's torch work.
"""
from __future__ import annotations

import contextlib
import ctypes as C
import time

import numpy as np

from . import LITHO_OK, Context, KernelSet, LithoError, PREC_FP32, _lib, _ptr

WIDTH, MODES, HIDDEN, LAYERS = 32, 16, 128, 4

# rectangle statistics of the surrogate's mask family
RECT = dict(nmin=8, nmax=32, wmin=8, wmax=64)


@contextlib.contextmanager
def torch_stream(ctx: Context):
    """Bind the context to torch's current stream for the duration of a call."""
    import torch
    ctx.set_stream(torch.cuda.current_stream(ctx.device).cuda_stream)
    try:
        yield
    finally:
        ctx.set_stream(None)


def num_params() -> int:
    return int(_lib.litho_surrogate_num_params())


def rect_masks(ctx: Context, seed: int, first: int, count: int, L: int, out=None, **kw):
    """Masks first .. first+count-1 of the seeded rectangle stream, on the device."""
    import torch
    r = dict(RECT, **kw)
    out = out if out is not None else torch.empty((count, L, L), dtype=torch.float32, device=f"cuda:{ctx.device}")
    with torch_stream(ctx):
        ctx._check(_lib.litho_rect_masks(ctx.h, int(seed), int(first), int(count), int(L), r["nmin"], r["nmax"],
                                         r["wmin"], r["wmax"], _ptr(out)))
    return out


class Surrogate:
    def __init__(self, ctx: Context, L: int = 256, seed: int = 0):
        h = C.c_void_p()
        ctx._check(_lib.litho_surrogate_create(ctx.h, int(L), int(seed), C.byref(h)))
        self.ctx, self.h, self.L = ctx, h, L
        self.n = num_params()
        ctx._adopt(self)

    def close(self):
        if self.h:
            _lib.litho_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # parameters (flat float32, oracle layout)
    def params(self) -> np.ndarray:
        p = np.empty(self.n, np.float32)
        with torch_stream(self.ctx):
            self.ctx._check(_lib.litho_surrogate_get_params(self.h, _ptr(p), self.n))
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        assert p.shape == (self.n,)
        with torch_stream(self.ctx):
            self.ctx._check(_lib.litho_surrogate_set_params(self.h, _ptr(p), self.n))

    def forward(self, masks, out=None):
        import torch
        out = out if out is not None else torch.empty_like(masks)
        with torch_stream(self.ctx):
            self.ctx._check(_lib.litho_surrogate_forward(self.h, _ptr(masks), int(masks.shape[0]), _ptr(out)))
        return out

    def loss_grad(self, masks, targets, want_grad: bool = True):
        loss = C.c_float()
        g = np.empty(self.n, np.float32) if want_grad else None
        with torch_stream(self.ctx):
            self.ctx._check(_lib.litho_surrogate_loss_grad(self.h, _ptr(masks), _ptr(targets), int(masks.shape[0]),
                                                           C.byref(loss), _ptr(g) if want_grad else None))
        return float(loss.value), g

    def train_step(self, masks, targets, lr: float, weight_decay: float = 1e-4, want_loss: bool = True):
        loss = C.c_float()
        with torch_stream(self.ctx):
            self.ctx._check(_lib.litho_surrogate_train_step(self.h, _ptr(masks), _ptr(targets), int(masks.shape[0]),
                                                            float(lr), float(weight_decay),
                                                            C.byref(loss) if want_loss else None))
        return float(loss.value) if want_loss else None

    def set_alpha(self, alpha: float):
        self.ctx._check(_lib.litho_surrogate_set_alpha(self.h, float(alpha)))

    @property
    def alpha(self) -> float:
        return float(_lib.litho_surrogate_get_alpha(self.h))

    def project(self, images, Nx: int, Ny: int):
        """In-place band projection of device images; returns the device error estimates."""
        import torch
        est = torch.empty(images.shape[0], dtype=torch.float32, device=images.device)
        with torch_stream(self.ctx):
            self.ctx._check(_lib.litho_surrogate_project(self.h, int(Nx), int(Ny), _ptr(images),
                                                         int(images.shape[0]), _ptr(est)))
        return est

    def predict(self, ks: KernelSet, masks, out=None):
        """Network image (band-projected) and the low-frequency error estimate, both on the device."""
        import torch
        out = out if out is not None else torch.empty_like(masks)
        est = torch.empty(masks.shape[0], dtype=torch.float32, device=masks.device)
        with torch_stream(self.ctx):
            self.ctx._check(_lib.litho_surrogate_predict(self.h, ks.h, _ptr(masks), int(masks.shape[0]), _ptr(out),
                                                         _ptr(est)))
        return out, est

    def image(self, ks: KernelSet, masks, threshold: float, out=None):
        """Surrogate images with SOCS fallback: (images, estimates, used_socs) -- estimates and flags on the host."""
        import torch
        out = out if out is not None else torch.empty_like(masks)
        B = int(masks.shape[0])
        est = np.empty(B, np.float32)
        used = np.empty(B, np.int32)
        with torch_stream(self.ctx):
            self.ctx._check(_lib.litho_surrogate_image(self.h, ks.h, _ptr(masks), B, float(threshold), _ptr(out),
                                                       _ptr(est), _ptr(used)))
        return out, est, used.astype(bool)

    def save(self, path: str):
        np.save(path, self.params())

    def load(self, path: str):
        self.set_params(np.load(path))


# optics of the surrogate workload: the mixed-precision case's quasar source and
# lens (NA 0.8, 193 nm, in focus) on 256 x 256 masks, K = 24 kernels
C5 = dict(L=256, NA=0.8, wavelength=193.0, defocus=0.0, nk=24, n_src=2000)


def c5_kernel_set(ctx: Context, L: int = C5["L"]):
    """FP64 TCC + FP64 eigensolve on the GPU for the surrogate's optics -> (KernelSet, info)."""
    from . import optics_n, outer_sigma, synth
    src, S, npts = synth.quasar_source(C5["n_src"])
    sig = outer_sigma(src)
    nx = optics_n(C5["NA"], L, sig, C5["wavelength"])
    tcc = ctx.calc_tcc(src, sig, C5["wavelength"], C5["NA"], C5["defocus"], L, L, nx, nx)
    krn, s32, _ = ctx.calc_kernels(tcc, min(C5["nk"], tcc.shape[0]))
    ks = ctx.kernel_set(krn, s32, nx, nx)
    return ks, dict(Nx=nx, nk=int(krn.shape[0]), src_points=npts, src_grid=S, sigma=sig, krn=krn, scales=s32)


def make_pairs(ctx: Context, ks: KernelSet, seed: int, first: int, count: int, L: int, chunk: int = 512):
    """(masks, images) device tensors: seeded rectangle masks and their GPU SOCS images."""
    import torch
    dev = f"cuda:{ctx.device}"
    masks = torch.empty((count, L, L), dtype=torch.float32, device=dev)
    images = torch.empty_like(masks)
    for s in range(0, count, chunk):
        n = min(chunk, count - s)
        rect_masks(ctx, seed, first + s, n, L, out=masks[s:s + n])
        with torch_stream(ctx):
            ctx.image_batch(ks, masks[s:s + n], images[s:s + n], precision=PREC_FP32)
    return masks, images


def train(model: Surrogate, masks, images, epochs: int, batch: int = 32, lr: float = 1e-3,
          decay_every: int = 0, gamma: float = 0.5, weight_decay: float = 1e-4, seed: int = 0, log=None):
    """Adam over shuffled mini-batches; lr halves every ``decay_every`` epochs.  Returns per-epoch mean loss."""
    import torch
    n = masks.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    hist = []
    steps_per_epoch = n // batch
    for ep in range(epochs):
        cur = lr * (gamma ** (ep // decay_every) if decay_every else 1.0)
        perm = torch.randperm(n, generator=g).to(masks.device)
        tot = 0.0
        t0 = time.time()
        for s in range(steps_per_epoch):
            idx = perm[s * batch:(s + 1) * batch]
            tot += model.train_step(masks.index_select(0, idx), images.index_select(0, idx), cur, weight_decay)
        hist.append(tot / max(1, steps_per_epoch))
        if log:
            log(f"epoch {ep} lr {cur:.2e} loss {hist[-1]:.5f} ({time.time() - t0:.2f} s)")
    return hist


def rel_l2_per_image(a, b):
    import torch
    d = torch.linalg.vector_norm((a - b).reshape(a.shape[0], -1), dim=1)
    return d / torch.linalg.vector_norm(b.reshape(b.shape[0], -1), dim=1)
