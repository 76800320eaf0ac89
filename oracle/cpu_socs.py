"""Multi-threaded CPU restatement of litho.cpp Modules 3 + 7 (the timed CPU baseline).

TEST INFRASTRUCTURE ONLY (and the bench's CPU leg): imported by ``bench.py`` for its
``cpu_baseline`` leg and for ``--impl reference`` (the reference's CPU path timed
on the host cores), never by the product.

For one mask it runs, in FP64 exactly as the reference orders the work:

* ``FT_r2c_padded`` (litho.cpp:242-318): centre-pad, roll, r2c over the full
  F x F grid (half spectrum [F][F/2+1]), rebuild the centred full spectrum from
  it by Hermitian symmetry (``rebuild_centred``), divide by F^2;
* ``calcSOCS`` (litho.cpp:795-1006): for each of the K kernels, embed K_k*M in a
  128 x 128 grid at offset 94, unnormalised backward c2c, accumulate
  s_k |E|^2; fftshift;
* ``FI`` (litho.cpp:674-754): r2c of the 128^2 intensity, zero-pad into the
  F x F half spectrum, c2r, roll; ``crop2DCentered``.

The K inverse FFTs are batched into one call and every transform uses
``scipy.fft`` with ``workers`` threads (pocketfft), so all host cores work on
each image, as litho_thread.cpp's OpenMP build would.
"""
from __future__ import annotations

import os
import time

import numpy as np
import scipy.fft as sfft

from . import np_ref as R


def rebuild_centred(half: np.ndarray, Fx: int, Fy: int) -> np.ndarray:
    """The full centred spectrum from an r2c half spectrum, as litho.cpp:264-312 does:
    R = the half spectrum with its rows rolled so DC lands at row Fy/2; the left half
    mirrors R by Hermitian symmetry; the right half is R itself from column Fx/2 on."""
    wt = Fx // 2 + 1
    ay = (Fy + 1) // 2
    r = np.concatenate([half[ay:], half[:ay]], axis=0)
    left = np.empty_like(r)
    if Fy % 2 == 0:
        left[0] = np.conj(r[0, ::-1])
        left[1:] = np.conj(r[:0:-1, ::-1])
    else:
        left[:] = np.conj(r[::-1, ::-1])
    out = np.empty((Fy, Fx), np.complex128)
    out[:, :wt] = left
    out[:, Fx // 2:] = r[:, :Fx - Fx // 2]
    return out


def socs_image(mask: np.ndarray, krns: np.ndarray, scales: np.ndarray, Nx: int, Ny: int,
               conv_n: int = 128, embed: int = 94, workers: int | None = None) -> np.ndarray:
    workers = workers or os.cpu_count() or 1
    Ly, Lx = mask.shape
    Fx, Fy = R.next_pow2(Lx), R.next_pow2(Ly)
    padded = R.pad_centered(mask.astype(np.float32), Fx, Fy)
    shifted = R.my_shift(padded, False, False).astype(np.float64)
    half = sfft.rfft2(shifted, workers=workers)
    mskf = rebuild_centred(half, Fx, Fy) / (Fx * Fy)
    K = len(scales)
    kx_, ky_ = 2 * Nx + 1, 2 * Ny + 1
    win = mskf[Fy // 2 - Ny:Fy // 2 + Ny + 1, Fx // 2 - Nx:Fx // 2 + Nx + 1]
    B = np.zeros((K, conv_n, conv_n), np.complex128)
    B[:, embed:embed + ky_, embed:embed + kx_] = krns.reshape(K, ky_, kx_) * win[None]
    E = sfft.ifft2(B, axes=(1, 2), workers=workers) * (conv_n * conv_n)
    acc = np.einsum("k,kyx->yx", scales.astype(np.float32).astype(np.float64), E.real ** 2 + E.imag ** 2)
    tmpimgp = R.my_shift(acc, True, True)
    sh = R.my_shift(tmpimgp, False, False)
    s = sfft.rfft2(sh, workers=workers) / (conv_n * conv_n)
    out = np.zeros((Fy, Fx // 2 + 1), np.complex128)
    pos = conv_n // 2 + 1
    w = min(conv_n // 2 + 1, Fx // 2 + 1)
    out[:pos, :w] = s[:pos, :w]
    out[pos + Fy - conv_n:, :w] = s[pos:, :w]
    real = sfft.irfft2(out, s=(Fy, Fx), workers=workers) * (Fx * Fy)
    img = R.my_shift(real, False, False).astype(np.float32)
    return R.crop_centered(img, Lx, Ly)


def time_images(masks, krns, scales, Nx, Ny, budget_s: float = 15.0, min_images: int = 2,
                workers: int | None = None):
    """Image masks cyclically until ``budget_s`` has elapsed (at least ``min_images``).

    Returns (images_per_s, n_images, elapsed_s, images of the first pass over ``masks``).
    """
    workers = workers or os.cpu_count() or 1
    socs_image(masks[0], krns, scales, Nx, Ny, workers=workers)   # warm the FFT plan caches
    out = []
    n = 0
    t0 = time.perf_counter()
    while True:
        img = socs_image(masks[n % len(masks)], krns, scales, Nx, Ny, workers=workers)
        if n < len(masks):
            out.append(img)
        n += 1
        el = time.perf_counter() - t0
        if n >= min_images and el >= budget_s:
            break
    el = time.perf_counter() - t0
    return n / el, n, el, out
