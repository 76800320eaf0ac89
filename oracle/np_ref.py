"""FP64 numpy restatement of the reference's Hopkins/SOCS aerial-image path.

TEST INFRASTRUCTURE ONLY.  This module is the oracle that the GPU library is
checked against.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs
of ``bench.py`` may import it, and only to check results or as the timed CPU
baseline; the product (``liblitho_gb300.so`` and the ``litho_gb300`` Python
binding) never calls into it.

Every function restates one function of the reference program
``validation/golden/src/litho.cpp`` (cited as ``litho.cpp:LINE``) or of its
``validation/golden/src/common/`` helpers.  The third-party arithmetic the
reference links (FFTW 3.x for the transforms, LAPACK ``zheevr`` for the
eigensolve; neither is vendored, versions unpinned) is replaced by numpy's
pocketfft and LAPACK ``zheevd``; their results at the boundary are pinned by the
reference's own checked-in goldens (``tests/test_oracle_golden.py``):

* ``source/TCC_HLS/hls/tb/golden/tcc_expected_{r,i}.bin``  -> calc_tcc
* ``source/TCC_HLS/hls/tb/golden/image_expected_512x512.bin`` -> ft_r2c_padded,
  calc_image, ft_c2r_padded, and (full rank) calc_kernels + calc_socs + fi
* ``source/TCC_HLS/hls/tb/golden/kernels/kernel_info.txt`` -> calc_kernels scales
* ``source/SOCS_HLS/data/hls_output_full_32.bin`` -> calc_socs tmpImgp

Floating-point types follow the reference where they matter for parity: the
pupil phase is evaluated in float32 exactly as litho.cpp:449-464 does, and all
accumulation is float64 (``std::complex<double>`` in the reference).
"""
from __future__ import annotations

import math

import numpy as np

f32 = np.float32


# ---------------------------------------------------------------------------
# small helpers (litho.cpp:116-177)
# ---------------------------------------------------------------------------

def next_pow2(x: int) -> int:
    """litho.cpp:120-125 ``nextPowerOfTwo``."""
    assert x > 0
    p = 1
    while p < x:
        p <<= 1
    return p


def my_shift(a: np.ndarray, shift_x: bool, shift_y: bool) -> np.ndarray:
    """litho.cpp:134-146 ``myShift``: out[(y+yh)%Y][(x+xh)%X] = in[y][x].

    ``True`` rolls by floor(N/2) (fftshift), ``False`` by ceil(N/2) (ifftshift).
    """
    Y, X = a.shape
    xh = X // 2 if shift_x else (X + 1) // 2
    yh = Y // 2 if shift_y else (Y + 1) // 2
    return np.roll(a, (yh, xh), axis=(0, 1))


def pad_centered(src: np.ndarray, dst_x: int, dst_y: int) -> np.ndarray:
    """litho.cpp:148-162 ``pad2DCentered`` (offset (dst-src)/2, zero fill)."""
    sy, sx = src.shape
    out = np.zeros((dst_y, dst_x), dtype=src.dtype)
    oy, ox = (dst_y - sy) // 2, (dst_x - sx) // 2
    out[oy:oy + sy, ox:ox + sx] = src
    return out


def crop_centered(src: np.ndarray, dst_x: int, dst_y: int) -> np.ndarray:
    """litho.cpp:164-177 ``crop2DCentered`` (offset (src-dst)/2)."""
    sy, sx = src.shape
    oy, ox = (sy - dst_y) // 2, (sx - dst_x) // 2
    return src[oy:oy + dst_y, ox:ox + dst_x].copy()


# ---------------------------------------------------------------------------
# source and mask (common/source.cpp, common/mask.cpp)
# ---------------------------------------------------------------------------

def create_annular(S: int, inner: float, outer: float) -> np.ndarray:
    """common/source.cpp:5-23 ``createAnnular`` (radii truncated to int pixels)."""
    c = (S - 1) // 2
    ri = int(f32(inner) * f32(c))
    ro = int(f32(outer) * f32(c))
    y, x = np.mgrid[0:S, 0:S]
    d = np.sqrt((x - c).astype(np.float64) ** 2 + (y - c).astype(np.float64) ** 2)
    return ((d >= ri) & (d <= ro)).astype(np.float32)


def create_cross_quadrupole(S: int, radius: float, offset: float) -> np.ndarray:
    """common/source.cpp:25-56 ``createCrossQuadrupole``."""
    c = (S - 1) // 2
    off = int(f32(offset) * f32(c))
    rad = int(f32(radius) * f32(c))
    y, x = np.mgrid[0:S, 0:S]
    out = np.zeros((S, S), dtype=bool)
    for cx, cy in ((c, c + off), (c, c - off), (c + off, c), (c - off, c)):
        out |= np.sqrt((x - cx) ** 2.0 + (y - cy) ** 2.0) <= rad
    return out.astype(np.float32)


def create_dipole(S: int, radius: float, offset: float, on_x_axis: bool) -> np.ndarray:
    """common/source.cpp:58-87 ``createDipole`` (note: centre is S/2, not (S-1)/2)."""
    off = int(f32(offset) * f32((S - 1) // 2))
    rad = int(f32(radius) * f32((S - 1) // 2))
    c = S // 2
    y, x = np.mgrid[0:S, 0:S]
    out = np.zeros((S, S), dtype=bool)
    for sgn in (1, -1):
        cx = c + sgn * (off if on_x_axis else 0)
        cy = c + sgn * (0 if on_x_axis else off)
        out |= np.sqrt((x - cx) ** 2.0 + (y - cy) ** 2.0) <= rad
    return out.astype(np.float32)


def normalize_source(src: np.ndarray) -> np.ndarray:
    """common/source.cpp:89-103 ``normalizeMatrix``: sequential float32 sum, then divide."""
    flat = src.astype(np.float32).ravel()
    s = np.cumsum(flat, dtype=np.float32)[-1] if flat.size else f32(0)
    if s != 0:
        flat = (flat / f32(s)).astype(np.float32)
    return flat.reshape(src.shape)


def create_mask(in_mask: np.ndarray, Lx: int, Ly: int, dose: float = 1.0) -> np.ndarray:
    """common/mask.cpp:31-60 ``createMask``: centre ``in_mask`` in an Ly x Lx period, times dose."""
    my, mx = in_mask.shape
    out = np.zeros((Ly, Lx), dtype=np.float32)
    oy, ox = (Ly - my) // 2, (Lx - mx) // 2
    out[oy:oy + my, ox:ox + mx] = (in_mask.astype(np.float32) * f32(dose)).astype(np.float32)
    return out


def line_space(sx: int, sy: int, line: int, space: int, horizontal: bool) -> np.ndarray:
    """common/mask.cpp:5-29 ``generateLineSpace``."""
    period = line + space
    if horizontal:
        col = (np.arange(sy) % period) < line
        return np.repeat(col[:, None], sx, axis=1).astype(np.float32)
    row = (np.arange(sx) % period) < line
    return np.repeat(row[None, :], sy, axis=0).astype(np.float32)


def get_outer_sigma(src: np.ndarray) -> float:
    """litho.cpp:414-426 ``getOuterSigma``: max lit radius / centre, float32."""
    S = src.shape[0]
    c = (S - 1) // 2
    ys, xs = np.nonzero(src != 0)
    if ys.size == 0 or c == 0:
        return 0.0
    d2 = (ys - c) ** 2 + (xs - c) ** 2
    md = f32(np.sqrt(np.float64(d2.max())))
    return float(f32(md / f32(c)))


def optics_nx(NA: float, L: int, outer_sigma: float, wavelength: float) -> int:
    """litho.cpp:1297-1301: sigma clamped to 1, Nx = floor(NA*L*(1+sigma)/lambda) in float32."""
    s = min(f32(outer_sigma), f32(1.0))
    v = f32(f32(f32(NA) * f32(L)) * f32(f32(1) + s)) / f32(wavelength)
    return int(math.floor(float(f32(v))))


# ---------------------------------------------------------------------------
# FFT wrappers (litho.cpp:242-408)
# ---------------------------------------------------------------------------

def ft_r2c_padded(mask: np.ndarray, fft_x: int, fft_y: int) -> np.ndarray:
    """litho.cpp:242-318 ``FT_r2c_padded``.

    Centre-pad, roll by ceil(F/2), r2c, rebuild the full spectrum with DC at
    (F_y/2, F_x/2) exactly as the reference's half-spectrum reconstruction,
    divide by F_x*F_y.  Returns complex128 of shape (F_y, F_x).
    """
    Ly, Lx = mask.shape
    padded = pad_centered(mask.astype(np.float32), fft_x, fft_y)
    shifted = my_shift(padded, False, False).astype(np.float64)
    half = np.fft.rfft2(shifted)                       # (F_y, F_x//2+1)
    wt = fft_x // 2 + 1
    AY = (fft_y + 1) // 2
    BY = fft_y - AY
    R = np.empty_like(half)
    R[:BY] = half[AY:AY + BY]
    R[BY:] = half[:fft_y - BY]
    L = np.empty_like(half)
    xr = np.arange(wt)[::-1]
    if fft_y % 2 == 0:
        L[0] = np.conj(R[0, xr])
        L[1:] = np.conj(R[::-1][:-1][:, xr])
    else:
        L[:] = np.conj(R[::-1][:, xr])
    out = np.zeros((fft_y, fft_x), dtype=np.complex128)
    out[:, :wt] = L
    out[:, fft_x // 2:] = R[:, :fft_x - fft_x // 2]
    return out / (fft_x * fft_y)


def ft_c2r_padded(spec: np.ndarray, out_x: int, out_y: int) -> np.ndarray:
    """litho.cpp:358-408 ``FT_c2r_padded``: full centred spectrum -> cropped float32 image."""
    Fy, Fx = spec.shape
    wt = Fx // 2 + 1
    xh = (Fx + 1) // 2
    yh = (Fy + 1) // 2
    datac = np.zeros((Fy, wt), dtype=np.complex128)
    xs = np.arange(xh - 1, Fx)
    sx = (xs + xh) % Fx
    keep = sx < wt
    xs, sx = xs[keep], sx[keep]
    sy = (np.arange(Fy) + yh) % Fy
    datac[np.ix_(sy, sx)] = spec[:, xs]
    if Fx % 2 == 0:
        R = np.empty(Fy, dtype=np.complex128)
        R[0] = np.conj(spec[0, 0])
        R[1:] = np.conj(spec[::-1, 0][:-1])
        datac[:, wt - 1] = R
    real = np.fft.irfft2(datac, s=(Fy, Fx)) * (Fx * Fy)
    shifted = my_shift(real, False, False)
    return crop_centered(shifted.astype(np.float32), out_x, out_y)


# ---------------------------------------------------------------------------
# TCC (litho.cpp:428-516)
# ---------------------------------------------------------------------------

def pupil_matrix(src: np.ndarray, outer_sigma: float, wavelength: float, NA: float,
                 defocus: float, Lx: int, Ly: int, Nx: int, Ny: int, n_medium: float = 1.0):
    """The pupil table of litho.cpp:437-471 restricted to lit source points.

    Returns (P, J, ids): P is complex128 (tccSize, n_lit) with the float32
    cos/sin of the float32 phase, J the float32 source weights, ids the source
    pixel indices in the reference's (q, p) loop order.  n_medium != 1 is the
    immersion extension of the phase, sqrt(n^2 - rho^2 NA^2) (the reference's
    sqrt(1 - rho^2 NA^2) is NaN wherever rho NA > 1).
    """
    S = src.shape[0]
    srcf = src.astype(np.float32).ravel()
    sh = int((S - 1) / 2.0)
    oSgm = int(math.ceil(float(f32(f32(sh) * f32(outer_sigma)))))
    NAf, lamf = f32(NA), f32(wavelength)
    dz = f32(f32(defocus) / f32(f32(NAf * NAf) / lamf))
    k = f32(2 * math.pi / float(lamf))
    Lx_norm = f32(f32(f32(Lx) * NAf) / lamf)
    Ly_norm = f32(f32(f32(Ly) * NAf) / lamf)
    tcc = (2 * Nx + 1) * (2 * Ny + 1)
    cols, J, ids = [], [], []
    for q in range(-oSgm, oSgm + 1):
        for p in range(-oSgm, oSgm + 1):
            sid = (q + sh) * S + p + sh
            if srcf[sid] == 0 or p * p + q * q > sh * sh:
                continue
            sx = f32(f32(p) / f32(sh))
            sy = f32(f32(q) / f32(sh))
            nxmin = int(f32(f32(-1 - sx) * Lx_norm))
            nxmax = int(f32(f32(1 - sx) * Lx_norm))
            nymin = int(f32(f32(-1 - sy) * Ly_norm))
            nymax = int(f32(f32(1 - sy) * Ly_norm))
            col = np.zeros(tcc, dtype=np.complex128)
            nys = np.arange(nymin, nymax + 1)
            nxs = np.arange(nxmin, nxmax + 1)
            fy = (nys.astype(np.float32) / Ly_norm + sy).astype(np.float32)
            fx = (nxs.astype(np.float32) / Lx_norm + sx).astype(np.float32)
            FY, FX = np.meshgrid(fy, fx, indexing="ij")
            NY, NX = np.meshgrid(nys, nxs, indexing="ij")
            rho2 = (FX * FX + FY * FY).astype(np.float32)
            ok = ((FY * FY) <= 1) & (rho2.astype(np.float64) <= 1.0)
            r = (rho2 * NAf).astype(np.float32) * NAf
            with np.errstate(invalid="ignore"):
                nm2 = float(n_medium) * float(n_medium)
                val = np.float64(f32(dz * k)) * np.sqrt(nm2 - r.astype(np.float32).astype(np.float64))
            phase = val.astype(np.float32)
            idx = (NY + Ny) * (2 * Nx + 1) + NX + Nx
            if ok.any():
                ii = idx[ok]
                if ii.min() < 0 or ii.max() >= tcc:
                    raise ValueError("pupil support exceeds the (2Nx+1)(2Ny+1) grid")
                ph = phase[ok]
                col[ii] = np.cos(ph).astype(np.float64) + 1j * np.sin(ph).astype(np.float64)
            cols.append(col)
            J.append(srcf[sid])
            ids.append(sid)
    if not cols:
        return np.zeros((tcc, 0), np.complex128), np.zeros(0, np.float32), np.zeros(0, np.int64)
    return np.stack(cols, axis=1), np.asarray(J, np.float32), np.asarray(ids)


def calc_tcc(src: np.ndarray, outer_sigma: float, wavelength: float, NA: float, defocus: float,
             Lx: int, Ly: int, Nx: int, Ny: int, n_medium: float = 1.0) -> np.ndarray:
    """litho.cpp:428-516 ``calcTCC``: TCC = sum_s J_s p_s p_s^H, upper triangle then conj mirror."""
    P, J, _ = pupil_matrix(src, outer_sigma, wavelength, NA, defocus, Lx, Ly, Nx, Ny, n_medium)
    T = (P * J.astype(np.float64)[None, :]) @ P.conj().T
    up = np.triu(T)
    return up + np.conj(np.triu(T, 1)).T


# ---------------------------------------------------------------------------
# TCC-direct image (litho.cpp:522-566)
# ---------------------------------------------------------------------------

def calc_image(mskf: np.ndarray, tcc: np.ndarray, Nx: int, Ny: int) -> np.ndarray:
    """litho.cpp:522-566 ``calcImage``: imgf on nx2 >= 0 only (C2R completes the rest)."""
    Fy, Fx = mskf.shape
    n = tcc.shape[0]
    th = (n - 1) // 2
    imgf = np.zeros((Fy, Fx), dtype=np.complex128)
    cy, cx = Fy // 2, Fx // 2
    ny1, nx1 = np.meshgrid(np.arange(-Ny, Ny + 1), np.arange(-Nx, Nx + 1), indexing="ij")
    ny1, nx1 = ny1.ravel(), nx1.ravel()
    b = mskf[ny1 + cy, nx1 + cx]
    row = ny1 * (2 * Nx + 1) + nx1 + th
    for ny2 in range(-2 * Ny, 2 * Ny + 1):
        for nx2 in range(0, 2 * Nx + 1):
            ok = (np.abs(nx2 + nx1) <= Nx) & (np.abs(ny2 + ny1) <= Ny)
            a = mskf[ny2 + ny1[ok] + cy, nx2 + nx1[ok] + cx]
            col = (ny2 + ny1[ok]) * (2 * Nx + 1) + (nx2 + nx1[ok]) + th
            imgf[ny2 + cy, nx2 + cx] = np.sum(a * np.conj(b[ok]) * tcc[row[ok], col])
    return imgf


# ---------------------------------------------------------------------------
# kernels (litho.cpp:579-645)
# ---------------------------------------------------------------------------

def calc_kernels(tcc: np.ndarray, nk: int):
    """litho.cpp:579-645 ``calcKernels``.

    Top-nk eigenpairs of the Hermitian TCC (upper triangle, as zheevr 'U'),
    scales descending, each eigenvector stored reversed (krn[i][j] = v_i[n-1-j]).
    Returns (krns complex128 (nk, n), scales float32 (nk,), w float64 (nk,)).
    """
    n = tcc.shape[0]
    w, V = np.linalg.eigh(tcc, UPLO="U")
    order = np.arange(n - 1, n - 1 - nk, -1)
    w_top = w[order]
    krns = V[:, order].T[:, ::-1].copy()
    return krns, w_top.astype(np.float32), w_top


# ---------------------------------------------------------------------------
# SOCS + Fourier interpolation (litho.cpp:674-754, 795-1006)
# ---------------------------------------------------------------------------

def fi(tmp_imgp: np.ndarray, out_x: int, out_y: int) -> np.ndarray:
    """litho.cpp:674-754 ``FI``: zero-pad spectral interpolation N^2 -> F^2 (float64 out)."""
    Ny_, Nx_ = tmp_imgp.shape
    shifted = my_shift(tmp_imgp.astype(np.float64), False, False)
    spec = np.fft.rfft2(shifted) / (Nx_ * Ny_)
    in_wt = Nx_ // 2 + 1
    out_wt = out_x // 2 + 1
    out = np.zeros((out_y, out_wt), dtype=np.complex128)
    pos = Ny_ // 2 + 1
    w = min(in_wt, out_wt)
    out[:pos, :w] = spec[:pos, :w]
    dif = out_y - Ny_
    rows = np.arange(pos, Ny_)
    orow = rows + dif
    ok = orow < out_y
    out[orow[ok], :w] = spec[rows[ok], :w]
    real = np.fft.irfft2(out, s=(out_y, out_x)) * (out_x * out_y)
    return my_shift(real, False, False)


def socs_tmpimg(mskf: np.ndarray, krns: np.ndarray, scales: np.ndarray, nk: int, Nx: int, Ny: int,
                conv_n: int = 128, embed: int | None = 94) -> np.ndarray:
    """litho.cpp:879-934: sum_k s_k |IFFT(embed(K_k * M))|^2 on the conv grid, then fftshift.

    ``embed=None`` centres the kernel (litho_thread.cpp:847); 94 is litho.cpp's
    HLS-matched offset (litho.cpp:826-827).  Returns tmpImgp (float64).
    """
    Fy, Fx = mskf.shape
    kx_, ky_ = 2 * Nx + 1, 2 * Ny + 1
    ex = (conv_n - kx_) // 2 if embed is None else embed
    ey = (conv_n - ky_) // 2 if embed is None else embed
    win = mskf[Fy // 2 - Ny:Fy // 2 + Ny + 1, Fx // 2 - Nx:Fx // 2 + Nx + 1]
    acc = np.zeros((conv_n, conv_n))
    for k in range(nk):
        B = np.zeros((conv_n, conv_n), dtype=np.complex128)
        kk = krns[k].reshape(ky_, kx_)
        # litho.cpp:905-912 skips products whose grid index falls outside the conv grid
        y0, x0 = max(ey, 0), max(ex, 0)
        y1, x1 = min(ey + ky_, conv_n), min(ex + kx_, conv_n)
        if y1 > y0 and x1 > x0:
            B[y0:y1, x0:x1] = (kk * win)[y0 - ey:y1 - ey, x0 - ex:x1 - ex]
        E = np.fft.ifft2(B) * (conv_n * conv_n)
        acc += np.float64(np.float32(scales[k])) * (E.real ** 2 + E.imag ** 2)
    return my_shift(acc, True, True)


def calc_socs(mskf: np.ndarray, phys_x: int, phys_y: int, krns: np.ndarray, scales: np.ndarray,
              nk: int, Nx: int, Ny: int, conv_n: int = 128, embed: int | None = 94):
    """litho.cpp:795-1006 ``calcSOCS``: returns (image float32 (phys_y, phys_x), tmpImgp float64)."""
    Fy, Fx = mskf.shape
    tmpimgp = socs_tmpimg(mskf, krns, scales, nk, Nx, Ny, conv_n, embed)
    padded = fi(tmpimgp, Fx, Fy).astype(np.float32)
    return crop_centered(padded, phys_x, phys_y), tmpimgp


def tmpimgp_center(tmpimgp: np.ndarray, Nx: int, Ny: int) -> np.ndarray:
    """litho.cpp:950-963: centre (4Nx+1)x(4Ny+1) of tmpImgp (``tmpImgp_pad{N}.bin``)."""
    N = tmpimgp.shape[0]
    cx, cy = 4 * Nx + 1, 4 * Ny + 1
    ox, oy = (N - cx) // 2, (N - cy) // 2
    return tmpimgp[oy:oy + cy, ox:ox + cx].astype(np.float32)


# ---------------------------------------------------------------------------
# whole-path convenience (litho.cpp:1193-1486 module order)
# ---------------------------------------------------------------------------

def mask_to_image(mask: np.ndarray, krns: np.ndarray, scales: np.ndarray, Nx: int, Ny: int,
                  conv_n: int = 128, embed: int | None = 94) -> np.ndarray:
    """Modules 3 + 7 of litho.cpp: FT_r2c_padded then calcSOCS (with FI and crop)."""
    Ly, Lx = mask.shape
    mskf = ft_r2c_padded(mask, next_pow2(Lx), next_pow2(Ly))
    img, _ = calc_socs(mskf, Lx, Ly, krns, scales, len(scales), Nx, Ny, conv_n, embed)
    return img


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    """Relative L2 error ||a-b|| / ||b|| in float64."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (nb if nb > 0 else 1.0))
