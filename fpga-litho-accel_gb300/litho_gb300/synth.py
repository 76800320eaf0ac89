"""Seeded synthetic masks and sources for the benchmark workloads.

The reference's own mask suite is only present as PNG renderings, so seeded
generators with the shapes and value distributions of the benchmark
configurations stand in for it:

* ``rect_mask``       -- L x L float32 0/1 mask of random axis-aligned rectangles
                         (512^2, 40 rectangles of width 8-64 px for the plain case).
* ``manhattan_mask``  -- L x L float32 0/1 Manhattan layout: tiles of line/space
                         gratings and contact arrays, about 50 % pattern density.
* ``density_rect_mask`` -- random rectangles until a target density is reached
                         (the batched case's 20-60 % masks).
* ``annular_source``  -- common/source.cpp:5-23 createAnnular + normalizeMatrix.
* ``quasar_source``   -- four poles at 45/135/225/315 degrees, radial band
                         [sigma_in, sigma_out], 30-degree opening; the grid size is
                         chosen so that about ``n_points`` pixels are lit.  Not a
                         reference source type (the reference imports such sources
                         from a file, litho.cpp:1100-1103 cannot parse one).
"""
from __future__ import annotations

import math

import numpy as np


def rect_mask(L: int = 512, n_rect: int = 40, wmin: int = 8, wmax: int = 64, seed: int = 1) -> np.ndarray:
    rng = np.random.default_rng(seed)
    m = np.zeros((L, L), np.float32)
    for _ in range(n_rect):
        w = int(rng.integers(wmin, wmax + 1))
        h = int(rng.integers(wmin, wmax + 1))
        x = int(rng.integers(0, L - w + 1))
        y = int(rng.integers(0, L - h + 1))
        m[y:y + h, x:x + w] = 1.0
    return m


def density_rect_mask(L: int, density: float, seed: int, wmin: int = 8, wmax: int = 96) -> np.ndarray:
    rng = np.random.default_rng(seed)
    m = np.zeros((L, L), np.float32)
    target = density * L * L
    while m.sum() < target:
        w = int(rng.integers(wmin, min(wmax, L) + 1))
        h = int(rng.integers(wmin, min(wmax, L) + 1))
        x = int(rng.integers(0, L - w + 1))
        y = int(rng.integers(0, L - h + 1))
        m[y:y + h, x:x + w] = 1.0
    return m


def manhattan_mask(L: int = 1024, seed: int = 2, tile: int = 128) -> np.ndarray:
    """Tiles of L/S gratings (50 % duty) and contact arrays (50 % area fill)."""
    rng = np.random.default_rng(seed)
    m = np.zeros((L, L), np.float32)
    for ty in range(0, L, tile):
        for tx in range(0, L, tile):
            h, w = min(tile, L - ty), min(tile, L - tx)
            kind = rng.integers(0, 3)
            pitch = int(rng.choice([16, 24, 32, 48, 64]))
            yy, xx = np.mgrid[0:h, 0:w]
            if kind == 0:      # vertical lines
                t = (xx % pitch) < pitch // 2
            elif kind == 1:    # horizontal lines
                t = (yy % pitch) < pitch // 2
            else:              # contacts: square side pitch/sqrt(2) -> 50 % area
                s = max(1, int(round(pitch / math.sqrt(2.0))))
                t = ((xx % pitch) < s) & ((yy % pitch) < s)
            m[ty:ty + h, tx:tx + w] = t.astype(np.float32)
    return m


def normalize(src: np.ndarray) -> np.ndarray:
    """common/source.cpp:89-103: sequential float32 sum, divide."""
    flat = src.astype(np.float32).ravel()
    s = np.cumsum(flat, dtype=np.float32)[-1]
    if s != 0:
        flat = (flat / np.float32(s)).astype(np.float32)
    return flat.reshape(src.shape)


def annular_source(S: int, inner: float, outer: float) -> np.ndarray:
    c = (S - 1) // 2
    ri = int(np.float32(inner) * np.float32(c))
    ro = int(np.float32(outer) * np.float32(c))
    y, x = np.mgrid[0:S, 0:S]
    d = np.sqrt((x - c).astype(np.float64) ** 2 + (y - c).astype(np.float64) ** 2)
    return normalize(((d >= ri) & (d <= ro)).astype(np.float32))


def _quasar(S: int, s_in: float, s_out: float, opening_deg: float) -> np.ndarray:
    c = (S - 1) // 2
    y, x = np.mgrid[0:S, 0:S]
    dx, dy = (x - c).astype(np.float64), (y - c).astype(np.float64)
    r = np.sqrt(dx * dx + dy * dy) / c
    ang = np.degrees(np.arctan2(dy, dx)) % 360.0
    half = opening_deg / 2
    lit = np.zeros((S, S), bool)
    for a0 in (45.0, 135.0, 225.0, 315.0):
        da = np.abs((ang - a0 + 180.0) % 360.0 - 180.0)
        lit |= (r >= s_in) & (r <= s_out) & (da <= half)
    return lit.astype(np.float32)


def quasar_source(n_points: int = 2000, s_in: float = 0.7, s_out: float = 0.9, opening_deg: float = 30.0):
    """Returns (normalised source, grid size S, lit count) with lit count closest to n_points."""
    best = None
    for S in range(21, 401, 2):
        q = _quasar(S, s_in, s_out, opening_deg)
        n = int(q.sum())
        if best is None or abs(n - n_points) < abs(best[2] - n_points):
            best = (q, S, n)
        if n > n_points * 1.2:
            break
    q, S, n = best
    return normalize(q), S, n
