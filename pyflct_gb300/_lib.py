"""ctypes binding of libflctgpu.so (the C ABI declared in include/flct_gpu.h).

The library is built in-tree (``python -m pyflct_gb300.build``).  Loading
fails loudly when it is missing or when no sm_103 GPU is present: there is no
CPU fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libflctgpu.so")

# flct_status (include/flct_gpu.h)
OK = 0
ERR_ARG = 1
ERR_SKIP_NONPOSITIVE = 2
ERR_SKIP_OFFSET = 3
ERR_SKIP_TOO_BIG = 4
ERR_BOX_SIZE = 5
ERR_GRID_TOO_SMALL = 6
ERR_NO_DEVICE = 7
ERR_CUDA = 8
ERR_ALLOC = 9
ERR_UNSUPPORTED = 10
ERR_WARP_DIMS = 11
ERR_TIMEOUT = 12

FORMS = {"fp32": 0, "tc_fp16": 1, "tc_bf16": 2, "auto": 3}


class Params(C.Structure):
    _fields_ = [
        ("deltat", C.c_double), ("deltas", C.c_double), ("sigma", C.c_double),
        ("thresh", C.c_double), ("thresh_abs", C.c_int), ("skip", C.c_int),
        ("poffset", C.c_int), ("qoffset", C.c_int), ("interpolate", C.c_int),
        ("filter", C.c_int), ("kr", C.c_double), ("hires", C.c_int), ("quiet", C.c_int),
        ("form", C.c_int),
    ]


class Timing(C.Structure):
    _fields_ = [
        ("ms_total", C.c_float), ("ms_window", C.c_float), ("ms_prepass", C.c_float),
        ("ms_interp", C.c_float), ("ms_h2d", C.c_float), ("ms_d2h", C.c_float),
        ("windows", C.c_longlong), ("launches", C.c_int), ("box", C.c_int), ("form", C.c_int),
        ("ms_fit", C.c_float),
    ]


class Pair(C.Structure):
    _fields_ = [
        ("f1", C.c_void_p), ("f2", C.c_void_p), ("nx", C.c_int), ("ny", C.c_int),
        ("params", Params), ("vx", C.c_void_p), ("vy", C.c_void_p), ("vm", C.c_void_p),
    ]


class FlctError(RuntimeError):
    """A non-OK flct_status, with the library's message."""

    def __init__(self, code: int, message: str = ""):
        super().__init__(f"flct status {code}: {message}")
        self.code = code
        self.message = message


# every symbol include/flct_gpu.h declares, with (restype, argtypes)
_dp = C.POINTER(C.c_double)
_vp = C.c_void_p
SIGNATURES = {
    "flct_gpu_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "flct_gpu_destroy": (None, [_vp]),
    "flct_gpu_last_error": (C.c_char_p, [_vp]),
    "flct_gpu_status_string": (C.c_char_p, [C.c_int]),
    "flct_gpu_last_timing": (C.c_int, [_vp, C.POINTER(Timing)]),
    "flct_gpu_version": (C.c_char_p, []),
    "flct_gpu_output_len": (C.c_longlong, [C.POINTER(Params), C.c_int, C.c_int]),
    "flct_gpu_velocity": (C.c_int, [_vp, C.POINTER(Params), _dp, _dp, C.c_int, C.c_int, _dp, _dp, _dp]),
    "flct_gpu_velocity_device": (C.c_int, [_vp, C.POINTER(Params), _vp, _vp, C.c_int, C.c_int,
                                           _vp, _vp, _vp, _vp]),
    "flct_gpu_velocity_batch": (C.c_int, [_vp, C.c_int, C.POINTER(Pair), _vp]),
    "flct_gpu_cross_cor_batch": (C.c_int, [_vp, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_double,
                                           C.c_int, _dp, _dp]),
    "flct_gpu_interpcc2d": (C.c_int, [_vp, _dp, C.c_double, C.c_int, C.c_int, _dp, C.c_int, _dp,
                                      C.c_int, _dp]),
    "flct_gpu_shift_frac2d": (C.c_int, [_vp, _dp, C.c_double, C.c_double, _dp, C.c_int, C.c_int,
                                        C.c_int]),
    "flct_gpu_warp_frac2d": (C.c_int, [_vp, _dp, _dp, _dp, _dp, C.c_int, C.c_int, C.c_int]),
    "flct_gpu_interpcc2d_noalloc": (C.c_int, [_vp, C.c_double, C.c_int, C.c_int, _vp, C.c_int, _vp,
                                              C.c_int, _vp, _vp]),
}

_lock = threading.Lock()
_lib = None


def load(path: str | None = None):
    """Load libflctgpu.so and declare every ABI symbol (raises if missing)."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise FlctError(ERR_NO_DEVICE, f"{p} is not built; run python -m pyflct_gb300.build")
        L = C.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = L
        return L


class Context:
    """One library context (device workspace + stream) on a CUDA device."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.flct_gpu_create(device, C.byref(h))
        if rc != OK:
            raise FlctError(rc, self.lib.flct_gpu_status_string(rc).decode()
                            + " (an sm_103 GPU is required; there is no CPU path)")
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.lib.flct_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc: int):
        if rc != OK:
            msg = self.lib.flct_gpu_last_error(self.h)
            raise FlctError(rc, msg.decode() if msg else "")

    def timing(self) -> Timing:
        t = Timing()
        self.check(self.lib.flct_gpu_last_timing(self.h, C.byref(t)))
        return t


_contexts: dict[int, Context] = {}


def context(device: int = 0) -> Context:
    with _lock:
        c = _contexts.get(device)
    if c is None:
        c = Context(device)
        with _lock:
            _contexts[device] = c
    return c
