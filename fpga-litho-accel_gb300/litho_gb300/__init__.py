"""Python binding of liblitho_gb300.so (ctypes over the C ABI in include/litho_gb300.h).

The names and argument meanings follow the reference program
``validation/golden/src/litho.cpp``: ``fft_mask`` is FT_r2c_padded
(litho.cpp:242-318), ``calc_socs`` is calcSOCS (litho.cpp:795-1006),
``calc_tcc`` is calcTCC (litho.cpp:428-516), ``calc_kernels`` is calcKernels
(litho.cpp:579-645).  Arrays may be numpy arrays (host; the library stages them)
or CUDA tensors exposing ``data_ptr()`` (device; work is queued on the context's
stream).

The shared library is required: importing this module raises ImportError when
it has not been built, and every call runs on the GPU -- there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liblitho_gb300.so")

LITHO_OK = 0
LITHO_ERR_ARG = 1
LITHO_ERR_CUDA = 2
LITHO_ERR_NOCONVERGE = 3
LITHO_ERR_NAN = 4
LITHO_ERR_NOMEM = 5
LITHO_ERR_IO = 6
LITHO_ERR_UNSUPPORTED = 7
LITHO_ERR_TIMEOUT = 8
MEM_HOST = 0
MEM_DEVICE = 1
PREC_FP32 = 0
PREC_MIXED = 1
# how the SOCS band is formed (litho_ctx_set_band_method)
BAND_AUTO = 0
BAND_FFT = 1
BAND_TCC = 2
TCC_FP64 = 0
TCC_SPLIT_BF16 = 1

if not os.path.exists(LIB_PATH):
    raise ImportError(f"{LIB_PATH} is missing: build it with `python fpga-litho-accel_gb300/build.py` "
                      "(or __graft_entry__.build()); there is no CPU fallback")

_lib = C.CDLL(LIB_PATH)

_p = C.c_void_p
_i = C.c_int
_f = C.c_float

_SIGS = {
    "litho_ctx_create": (_i, [_i, C.POINTER(_p)]),
    "litho_ctx_destroy": (_i, [_p]),
    "litho_ctx_set_stream": (_i, [_p, _p]),
    "litho_ctx_get_stream": (_p, [_p]),
    "litho_ctx_synchronize": (_i, [_p]),
    "litho_last_error": (C.c_char_p, [_p]),
    "litho_status_string": (C.c_char_p, [_i]),
    "litho_version": (_i, []),
    "litho_outer_sigma": (_f, [_p, _i]),
    "litho_optics_n": (_i, [_f, _i, _f, _f]),
    "litho_fft_mask": (_i, [_p, _p, _i, _i, _p, _p, _i]),
    "litho_calc_socs": (_i, [_p, _p, _p, _i, _i, _p, _p, _p, _i, _i, _i, _i, _i, _p, _p, _i, _i]),
    "litho_image": (_i, [_p, _p, _i, _i, _p, _p, _p, _i, _i, _i, _p, _i, _i]),
    "litho_kernel_set_create": (_i, [_p, _p, _p, _p, _i, _i, _i, _i, C.POINTER(_p)]),
    "litho_kernel_set_destroy": (_i, [_p]),
    "litho_image_batch": (_i, [_p, _p, _p, _i, _i, _i, _p, _i, _i]),
    "litho_calc_tcc": (_i, [_p, _p, _i, _f, _f, _f, _f, _i, _i, _i, _i, _p, _i, _i]),
    "litho_calc_kernels": (_i, [_p, _p, _i, _i, _p, _p, _p, _p, _p, _i]),
    "litho_calc_tcc_medium": (_i, [_p, _p, _i, _f, _f, _f, _f, _f, _i, _i, _i, _i, _p, _i, _i]),
    "litho_calc_image": (_i, [_p, _p, _p, _i, _i, _p, _i, _i, _i, _i, _i, _p, _i]),
    "litho_ctx_enable_timing": (_i, [_p, _i]),
    "litho_ctx_stage_times": (_i, [_p, _p, _p, _i]),
    "litho_ctx_set_test_stall": (_i, [_p, _i]),
    "litho_ctx_set_band_method": (_i, [_p, _i]),
    "litho_ctx_set_host_chunk": (_i, [_p, C.c_size_t]),
    "litho_tcc_gemm_shape": (_i, [_p, _i, _i, _i]),
    "litho_tcc_gemm_describe": (_i, [_p, C.c_char_p, _i]),
    "litho_batch_plan_create": (_i, [_p, _p, _p, _i, _p, _i, _i, _i, C.POINTER(_p)]),
    "litho_batch_plan_mask": (_p, [_p, _i]),
    "litho_batch_plan_image": (_p, [_p, _i]),
    "litho_batch_plan_run": (_i, [_p]),
    "litho_batch_plan_describe": (_i, [_p, C.c_char_p, _i]),
    "litho_batch_plan_destroy": (_i, [_p]),
    "litho_surrogate_num_params": (C.c_longlong, []),
    "litho_surrogate_create": (_i, [_p, _i, C.c_ulonglong, C.POINTER(_p)]),
    "litho_surrogate_destroy": (None, [_p]),
    "litho_surrogate_get_params": (_i, [_p, _p, C.c_longlong]),
    "litho_surrogate_set_params": (_i, [_p, _p, C.c_longlong]),
    "litho_surrogate_forward": (_i, [_p, _p, _i, _p]),
    "litho_surrogate_loss_grad": (_i, [_p, _p, _p, _i, _p, _p]),
    "litho_surrogate_train_step": (_i, [_p, _p, _p, _i, _f, _f, _p]),
    "litho_rect_masks": (_i, [_p, C.c_ulonglong, C.c_longlong, _i, _i, _i, _i, _i, _i, _p]),
    "litho_surrogate_set_alpha": (_i, [_p, _f]),
    "litho_surrogate_get_alpha": (_f, [_p]),
    "litho_surrogate_project": (_i, [_p, _i, _i, _p, _i, _p]),
    "litho_surrogate_predict": (_i, [_p, _p, _p, _i, _p, _p]),
    "litho_surrogate_image": (_i, [_p, _p, _p, _i, _f, _p, _p, _p]),
}
BATCH_AUTOTUNE = 1
_CUDA_STREAM_LEGACY = 0x1  # cudaStreamLegacy
BATCH_GRAPH = 2


class _BatchItem(C.Structure):
    _fields_ = [("cls", C.c_int), ("mLx", C.c_int), ("mLy", C.c_int)]


class _DevArray:
    """A raw device buffer exposed through __cuda_array_interface__ (float32, C order)."""

    def __init__(self, ptr: int, shape):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": "<f4", "data": (int(ptr), False),
                                         "version": 3, "strides": None}
STAGES = ("win_dft", "socs", "fi_prep", "fi_out", "fft_mask", "tcc", "eig", "upload", "surrogate")
for _name, (_res, _args) in _SIGS.items():
    _fn = getattr(_lib, _name)
    _fn.restype = _res
    _fn.argtypes = _args


def lib() -> C.CDLL:
    return _lib


class LithoError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


def _is_dev(a) -> bool:
    return hasattr(a, "data_ptr") and getattr(a, "is_cuda", False)


def _ptr(a):
    if a is None:
        return None
    if _is_dev(a):
        return C.c_void_p(a.data_ptr())
    return a.ctypes.data_as(C.c_void_p)


def _host_f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def outer_sigma(src: np.ndarray) -> float:
    """getOuterSigma (litho.cpp:414-426) clamped to 1 (litho.cpp:1298)."""
    s = _host_f32(src)
    return float(_lib.litho_outer_sigma(_ptr(s), int(s.shape[0])))


def optics_n(NA: float, L: int, outer_sigma_: float, wavelength: float) -> int:
    """Nx = floor(NA*L*(1+sigma)/lambda) in float32 (litho.cpp:1300)."""
    return int(_lib.litho_optics_n(NA, int(L), outer_sigma_, wavelength))


def next_pow2(x: int) -> int:
    p = 1
    while p < x:
        p <<= 1
    return p


class KernelSet:
    """SOCS kernels uploaded once (k-major (nk, 2Ny+1, 2Nx+1) complex) + scales."""

    def __init__(self, ctx: "Context", krn: np.ndarray, scales: np.ndarray, Nx: int, Ny: int):
        self.ctx = ctx
        k = np.asarray(krn)
        kr = np.ascontiguousarray(k.real, dtype=np.float32)
        ki = np.ascontiguousarray(k.imag, dtype=np.float32)
        s = _host_f32(scales)
        self.nk, self.Nx, self.Ny = int(s.shape[0]), int(Nx), int(Ny)
        h = C.c_void_p()
        ctx._check(_lib.litho_kernel_set_create(ctx.h, _ptr(kr), _ptr(ki), _ptr(s), self.nk, self.Nx, self.Ny,
                                                MEM_HOST, C.byref(h)))
        self.h = h
        ctx._adopt(self)

    def close(self):
        if self.h:
            _lib.litho_kernel_set_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchPlan:
    """Masks of uneven sizes imaged per size class in one CUDA graph (litho_batch_plan_*).

    ``sets``/``periods``: one KernelSet and power-of-two period per size class;
    ``items``: (cls, mLx, mLy) per mask.  ``mask(i)``/``image(i)`` return torch
    views of the plan's device slots.
    """

    def __init__(self, ctx: "Context", sets, periods, items, precision: int = PREC_FP32,
                 flags: int = BATCH_AUTOTUNE | BATCH_GRAPH):
        self.ctx = ctx
        self.items = [tuple(int(v) for v in it) for it in items]
        self.periods = [int(p) for p in periods]
        hs = (C.c_void_p * len(sets))(*[s.h for s in sets])
        ps = (C.c_int * len(periods))(*self.periods)
        arr = (_BatchItem * len(items))(*[_BatchItem(c, x, y) for c, x, y in self.items])
        h = C.c_void_p()
        ctx._check(_lib.litho_batch_plan_create(ctx.h, C.cast(hs, C.c_void_p), C.cast(ps, C.c_void_p), len(sets),
                                                C.cast(arr, C.c_void_p), len(items), precision, flags, C.byref(h)))
        self.h = h
        ctx._adopt(self)

    def mask(self, i: int):
        import torch
        c, x, y = self.items[i]
        return torch.as_tensor(_DevArray(_lib.litho_batch_plan_mask(self.h, i), (y, x)), device="cuda")

    def image(self, i: int):
        import torch
        L_ = self.periods[self.items[i][0]]
        return torch.as_tensor(_DevArray(_lib.litho_batch_plan_image(self.h, i), (L_, L_)), device="cuda")

    def run(self):
        self.ctx._check(_lib.litho_batch_plan_run(self.h))

    def describe(self) -> dict:
        import json
        buf = C.create_string_buffer(1 << 16)
        _lib.litho_batch_plan_describe(self.h, buf, len(buf))
        return json.loads(buf.value.decode())

    def close(self):
        if self.h:
            _lib.litho_batch_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """A litho_ctx: one CUDA device, one stream, grow-only workspaces."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        st = _lib.litho_ctx_create(int(device), C.byref(h))
        if st != LITHO_OK:
            raise LithoError(st, f"litho_ctx_create(device={device}) failed")
        self.h = h
        self.device = device
        self._children = weakref.WeakSet()

    def _adopt(self, obj):
        """Objects made on this context (kernel sets, batch plans, surrogates) are closed with it."""
        self._children.add(obj)

    def close(self):
        if self.h:
            kids = list(self._children)
            for k in kids:  # plans and surrogates before the kernel sets they may use
                if not isinstance(k, KernelSet):
                    k.close()
            for k in kids:
                if isinstance(k, KernelSet):
                    k.close()
            _lib.litho_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, st: int):
        if st != LITHO_OK:
            msg = _lib.litho_last_error(self.h).decode(errors="replace")
            raise LithoError(st, msg or _lib.litho_status_string(st).decode())

    def set_stream(self, stream_handle: Optional[int]):
        """Queue work on a caller's stream (``torch.cuda.Stream.cuda_stream``); None restores the
        context's own stream.  Handle 0 (torch's default stream) is the legacy default stream,
        passed as cudaStreamLegacy since a NULL handle means the context's own stream."""
        if stream_handle is None:
            h = None
        else:
            h = C.c_void_p(int(stream_handle) if int(stream_handle) != 0 else _CUDA_STREAM_LEGACY)
        self._check(_lib.litho_ctx_set_stream(self.h, h))

    def synchronize(self):
        self._check(_lib.litho_ctx_synchronize(self.h))

    def enable_timing(self, on: bool = True):
        self._check(_lib.litho_ctx_enable_timing(self.h, 1 if on else 0))

    def set_test_stall(self, chunk: int):
        """Error-path test hook (litho_ctx_set_test_stall): chunk >= 0 makes the mixed window
        DFT's TMA producer stop at that chunk, so the call returns LITHO_ERR_TIMEOUT; -1 = off."""
        self._check(_lib.litho_ctx_set_test_stall(self.h, int(chunk)))

    def set_band_method(self, method: int):
        """BAND_AUTO (default: per batch, the form a cost model fitted on GB300 expects to be
        faster), BAND_FFT (per kernel FFTs on the conv grid) or BAND_TCC (the TCC bilinear form
        wherever the kernel set has its table) (litho_ctx_set_band_method)."""
        self._check(_lib.litho_ctx_set_band_method(self.h, int(method)))

    def set_host_chunk(self, nbytes: int = 0):
        """Mask bytes per chunk of image_batch on host arrays (litho_ctx_set_host_chunk);
        0 restores the default (128 MB)."""
        self._check(_lib.litho_ctx_set_host_chunk(self.h, int(nbytes)))

    def stage_times(self, reset: bool = True):
        """{stage: (device ms, kernel launches)} since the last reset (synchronises the stream)."""
        ms = (C.c_double * len(STAGES))()
        n = (C.c_longlong * len(STAGES))()
        self._check(_lib.litho_ctx_stage_times(self.h, C.cast(ms, C.c_void_p), C.cast(n, C.c_void_p),
                                               1 if reset else 0))
        return {s: (ms[i], n[i]) for i, s in enumerate(STAGES)}

    @property
    def stream(self) -> int:
        return int(_lib.litho_ctx_get_stream(self.h) or 0)

    # -- FT_r2c_padded -------------------------------------------------------
    def fft_mask(self, mask, out_r=None, out_i=None):
        """Centred, normalised mask spectrum (litho.cpp:242-318). Returns (mskf_r, mskf_i)."""
        Ly, Lx = mask.shape
        Fx, Fy = next_pow2(Lx), next_pow2(Ly)
        if _is_dev(mask):
            import torch
            out_r = out_r if out_r is not None else torch.empty((Fy, Fx), dtype=torch.float32, device=mask.device)
            out_i = out_i if out_i is not None else torch.empty((Fy, Fx), dtype=torch.float32, device=mask.device)
            self._check(_lib.litho_fft_mask(self.h, _ptr(mask), Lx, Ly, _ptr(out_r), _ptr(out_i), MEM_DEVICE))
            return out_r, out_i
        m = _host_f32(mask)
        out_r = np.empty((Fy, Fx), np.float32)
        out_i = np.empty((Fy, Fx), np.float32)
        self._check(_lib.litho_fft_mask(self.h, _ptr(m), Lx, Ly, _ptr(out_r), _ptr(out_i), MEM_HOST))
        return out_r, out_i

    # -- calcSOCS --------------------------------------------------------------
    def calc_socs(self, mskf_r, mskf_i, krn, scales, Nx: int, Ny: int, phys_x: int, phys_y: int,
                  want_tmpimgp: bool = False, conv_n: int = 0):
        """calcSOCS (litho.cpp:795-1006) from a full spectrum. Returns image or (image, tmpImgp)."""
        Fy, Fx = mskf_r.shape
        k = np.asarray(krn)
        kr = np.ascontiguousarray(k.real, dtype=np.float32).reshape(-1)
        ki = np.ascontiguousarray(k.imag, dtype=np.float32).reshape(-1)
        s = _host_f32(scales)
        nk = int(s.shape[0])
        n = conv_n or 128
        image = np.empty((phys_y, phys_x), np.float32)
        tmp = np.empty((n, n), np.float32) if want_tmpimgp else None
        self._check(_lib.litho_calc_socs(self.h, _ptr(_host_f32(mskf_r)), _ptr(_host_f32(mskf_i)), Fx, Fy,
                                         _ptr(kr), _ptr(ki), _ptr(s), nk, Nx, Ny, phys_x, phys_y,
                                         _ptr(image), _ptr(tmp), conv_n, MEM_HOST))
        return (image, tmp) if want_tmpimgp else image

    # -- calcImage (TCC-direct) ------------------------------------------------
    def calc_image(self, mskf_r, mskf_i, tcc, Nx: int, Ny: int, phys_x: int, phys_y: int):
        """calcImage + FT_c2r_padded (litho.cpp:522-566, 358-408): TCC-direct image."""
        Fy, Fx = mskf_r.shape
        t = np.ascontiguousarray(tcc, dtype=np.complex128)
        out = np.empty((phys_y, phys_x), np.float32)
        self._check(_lib.litho_calc_image(self.h, _ptr(_host_f32(mskf_r)), _ptr(_host_f32(mskf_i)), Fx, Fy,
                                          _ptr(t), t.shape[0], Nx, Ny, phys_x, phys_y, _ptr(out), MEM_HOST))
        return out

    # -- fused mask -> image ---------------------------------------------------
    def image(self, mask, krn, scales, Nx: int, Ny: int, precision: int = PREC_FP32):
        """FT_r2c_padded + calcSOCS for one mask (host arrays)."""
        Ly, Lx = mask.shape
        k = np.asarray(krn)
        kr = np.ascontiguousarray(k.real, dtype=np.float32).reshape(-1)
        ki = np.ascontiguousarray(k.imag, dtype=np.float32).reshape(-1)
        s = _host_f32(scales)
        out = np.empty((Ly, Lx), np.float32)
        self._check(_lib.litho_image(self.h, _ptr(_host_f32(mask)), Lx, Ly, _ptr(kr), _ptr(ki), _ptr(s),
                                     int(s.shape[0]), Nx, Ny, _ptr(out), precision, MEM_HOST))
        return out

    def kernel_set(self, krn, scales, Nx: int, Ny: int) -> KernelSet:
        return KernelSet(self, krn, scales, Nx, Ny)

    def image_batch(self, ks: KernelSet, masks, images=None, precision: int = PREC_FP32):
        """Image a batch of equal-size masks (B, Ly, Lx).  Device tensors stay on the device; the
        work is queued on the context's stream (its own non-blocking stream unless set_stream
        chose another), so the tensors' producers on other streams must be ordered before the
        call (torch.cuda.synchronize(), or set_stream(torch.cuda.current_stream().cuda_stream))."""
        B, Ly, Lx = masks.shape
        if _is_dev(masks):
            import torch
            images = images if images is not None else torch.empty_like(masks)
            self._check(_lib.litho_image_batch(self.h, ks.h, _ptr(masks), B, Lx, Ly, _ptr(images), precision,
                                               MEM_DEVICE))
            return images
        m = _host_f32(masks)
        out = np.empty_like(m) if images is None else images
        self._check(_lib.litho_image_batch(self.h, ks.h, _ptr(m), B, Lx, Ly, _ptr(out), precision, MEM_HOST))
        return out

    # -- calcTCC ---------------------------------------------------------------
    def calc_tcc(self, src, outer_sigma_: float, wavelength: float, NA: float, defocus: float,
                 Lx: int, Ly: int, Nx: int, Ny: int, precision: int = TCC_FP64, n_medium: float = 1.0) -> np.ndarray:
        """calcTCC (litho.cpp:428-516). Returns complex128 (tcc, tcc).  n_medium != 1 uses the
        immersion form of the pupil phase (litho_calc_tcc_medium)."""
        s = _host_f32(src)
        n = (2 * Nx + 1) * (2 * Ny + 1)
        out = np.empty((n, n), np.complex128)
        if n_medium == 1.0:
            self._check(_lib.litho_calc_tcc(self.h, _ptr(s), int(s.shape[0]), outer_sigma_, wavelength, NA, defocus,
                                            Lx, Ly, Nx, Ny, _ptr(out), precision, MEM_HOST))
        else:
            self._check(_lib.litho_calc_tcc_medium(self.h, _ptr(s), int(s.shape[0]), outer_sigma_, wavelength, NA,
                                                   defocus, n_medium, Lx, Ly, Nx, Ny, _ptr(out), precision, MEM_HOST))
        return out

    GEMM_SHAPES = ((64, 64), (128, 64), (256, 64), (128, 32), (256, 32))

    def tcc_gemm_shape(self, bn: int = 0, bk: int = 64, sched: int = 0):
        """Fix the split-BF16 TCC GEMM's column tile width bn and K slice bk (one of GEMM_SHAPES)
        and its schedule (0 whole tiles, 1 last one or two rounds split along K, 2 last partial
        round split); bn = 0 restores the on-device autotuner (litho_tcc_gemm_shape)."""
        self._check(_lib.litho_tcc_gemm_shape(self.h, int(bn), int(bk), int(sched)))

    def tcc_gemm_tuning(self) -> list:
        """The autotuner's cached choices with every candidate's time (litho_tcc_gemm_describe)."""
        import json
        buf = C.create_string_buffer(1 << 16)
        _lib.litho_tcc_gemm_describe(self.h, buf, len(buf))
        return json.loads(buf.value.decode())

    # -- calcKernels -----------------------------------------------------------
    def calc_kernels(self, tcc: np.ndarray, nk: int):
        """calcKernels (litho.cpp:579-645). Returns (krn complex128 (nk, n), scales f32, scales f64)."""
        t = np.ascontiguousarray(tcc, dtype=np.complex128)
        n = t.shape[0]
        kr = np.empty((nk, n), np.float32)
        ki = np.empty((nk, n), np.float32)
        sc = np.empty(nk, np.float32)
        k64 = np.empty((nk, n), np.complex128)
        s64 = np.empty(nk, np.float64)
        self._check(_lib.litho_calc_kernels(self.h, _ptr(t), n, nk, _ptr(kr), _ptr(ki), _ptr(sc), _ptr(k64),
                                            _ptr(s64), MEM_HOST))
        return k64, sc, s64
