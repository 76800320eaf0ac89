"""CPU oracle for the Fourier-neural-operator surrogate -- TEST INFRASTRUCTURE ONLY.

Nothing in the product imports this module: it is the oracle for the GPU
surrogate kernels (tests, ``__graft_entry__.smoke`` and ``bench.py``'s CPU leg).

The surrogate has no counterpart in the reference (the reference images every
mask with SOCS, litho.cpp:795-880).  Its architecture is the published FNO-2d
(Li et al., "Fourier Neural Operator for Parametric Partial Differential
Equations", ICLR 2021): a pointwise lift, four Fourier layers
``z = W v + b + irfft2(R . rfft2(v)|modes)`` with GELU between them (none after
the last), and a two-layer pointwise projection.  Here the input is the mask
alone (one channel): the Hopkins image of a periodic mask is shift-equivariant,
so the coordinate channels of the original FNO carry nothing.

The activation is GELU in its tanh form, 0.5 x (1 + tanh(sqrt(2/pi)(x + 0.044715 x^3)))
(Hendrycks & Gimpel 2016; torch ``gelu(approximate="tanh")``), which the GPU
kernels evaluate with the hardware tanh.

The restatement runs in float64 torch on the CPU so that autograd gives the
reference gradients the GPU backward kernels are checked against; the flat
parameter vector has exactly the layout the C ABI uses:

    Pw[32], Pb[32],
    W[l][o][c] (4 x 32 x 32), Wb[l][o] (4 x 32),
    R[l][j][kx][c][o][re,im] (4 x 32 x 16 x 32 x 32 x 2),  ky(j) = j (j<16), L-32+j (j>=16)
    Q1[h][c] (128 x 32), q1b[128], Q2[128], q2b[1]

The seeded rectangle generator below restates the device generator
(SplitMix64 counters, Steele/Lea/Flood 2014) bit for bit.
"""
from __future__ import annotations

import numpy as np

WIDTH = 32
MODES = 16
HIDDEN = 128
LAYERS = 4


def param_shapes(width=WIDTH, modes=MODES, hidden=HIDDEN, layers=LAYERS):
    shapes = [("Pw", (width,)), ("Pb", (width,))]
    shapes += [("W", (layers, width, width)), ("Wb", (layers, width))]
    shapes += [("R", (layers, 2 * modes, modes, width, width, 2))]
    shapes += [("Q1", (hidden, width)), ("q1b", (hidden,)), ("Q2", (hidden,)), ("q2b", (1,))]
    return shapes


def num_params(**kw):
    return int(sum(int(np.prod(s)) for _, s in param_shapes(**kw)))


def unpack(theta, **kw):
    """Split a flat vector (numpy or torch) into named views."""
    out, o = {}, 0
    for name, shp in param_shapes(**kw):
        n = int(np.prod(shp))
        out[name] = theta[o:o + n].reshape(shp)
        o += n
    assert o == theta.shape[0]
    return out


def ky_index(L, modes=MODES):
    return np.concatenate([np.arange(modes), np.arange(L - modes, L)])


def forward(theta, masks, modes=MODES):
    """theta: torch float64 [P]; masks: torch float64 [B, L, L] -> images [B, L, L]."""
    import torch
    import torch.nn.functional as F
    p = unpack(theta)
    B, L, _ = masks.shape
    v = masks[..., None] * p["Pw"] + p["Pb"]                       # [B, y, x, C]
    kyi = torch.as_tensor(ky_index(L, modes))
    for l in range(LAYERS):
        zw = v @ p["W"][l].T + p["Wb"][l]
        vf = torch.fft.rfft2(v, dim=(1, 2))                          # [B, L, L/2+1, C]
        R = torch.complex(p["R"][l][..., 0], p["R"][l][..., 1])     # [2m, m, C, C]
        sel = vf[:, kyi, :modes, :]                                  # [B, 2m, m, C]
        mixed = torch.einsum("bjkc,jkco->bjko", sel, R)
        oft = torch.zeros(B, L, L // 2 + 1, v.shape[-1], dtype=vf.dtype)
        oft[:, kyi, :modes, :] = mixed
        zs = torch.fft.irfft2(oft, s=(L, L), dim=(1, 2))
        z = zw + zs
        v = F.gelu(z, approximate="tanh") if l < LAYERS - 1 else z
    h = F.gelu(v @ p["Q1"].T + p["q1b"], approximate="tanh")
    return h @ p["Q2"] + p["q2b"][0]


def rel_l2_loss(out, target):
    """Mean over the batch of ||out - target|| / ||target|| (the FNO paper's loss)."""
    import torch
    d = torch.linalg.vector_norm((out - target).reshape(out.shape[0], -1), dim=1)
    n = torch.linalg.vector_norm(target.reshape(target.shape[0], -1), dim=1)
    return (d / n).mean()


def loss_and_grad(theta_np, masks_np, targets_np):
    """float64 loss and d loss / d theta by torch CPU autograd."""
    import torch
    th = torch.tensor(np.asarray(theta_np, np.float64), requires_grad=True)
    m = torch.tensor(np.asarray(masks_np, np.float64))
    t = torch.tensor(np.asarray(targets_np, np.float64))
    loss = rel_l2_loss(forward(th, m), t)
    loss.backward()
    return float(loss.detach()), th.grad.numpy().copy()


def predict(theta_np, masks_np):
    import torch
    with torch.no_grad():
        return forward(torch.tensor(np.asarray(theta_np, np.float64)),
                       torch.tensor(np.asarray(masks_np, np.float64))).numpy()


# --------------------------------------------------------------------------- masks
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix(x):
    """SplitMix64 output function on uint64 arrays (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def _h(seed, idx, k):
    with np.errstate(over="ignore"):
        base = np.uint64(seed) * np.uint64(0xD1B54A32D192ED03) + np.asarray(idx, np.uint64) * np.uint64(
            0x9E3779B97F4A7C15)
        return _splitmix(base + np.uint64(k))


def rect_masks(seed, first, count, L, nmin=8, nmax=32, wmin=8, wmax=64):
    """Masks ``first .. first+count-1`` of the seeded stream: nrect in [nmin, nmax]
    axis-aligned rectangles with sides in [wmin, wmax] on a 0 background."""
    out = np.zeros((count, L, L), np.float32)
    for b in range(count):
        i = np.uint64(first + b)
        n = nmin + int(_h(seed, i, 0) % np.uint64(nmax - nmin + 1))
        for r in range(n):
            w = wmin + int(_h(seed, i, 1 + 4 * r) % np.uint64(wmax - wmin + 1))
            hh = wmin + int(_h(seed, i, 2 + 4 * r) % np.uint64(wmax - wmin + 1))
            x0 = int(_h(seed, i, 3 + 4 * r) % np.uint64(L - w + 1))
            y0 = int(_h(seed, i, 4 + 4 * r) % np.uint64(L - hh + 1))
            out[b, y0:y0 + hh, x0:x0 + w] = 1.0
    return out
