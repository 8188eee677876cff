"""ctypes front end to the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module: it is the checker for the GPU path, never the product.

* ``liboracle.so`` -- the project's C restatement of FLCT 1.01's hot path
  (flct_oracle.c) over its own double-precision FFT.
* ``_ref/``        -- the unmodified reference sources compiled in place
  against the project FFTW-API shim (``make ref``); present only where the
  reference tree is available, so every user of it must cope with absence.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
XMISS = -999999.0
VCID = 2136967593

_lock = threading.Lock()
_lib = None


class OParams(C.Structure):
    _fields_ = [
        ("deltat", C.c_double), ("deltas", C.c_double), ("sigma", C.c_double),
        ("thresh", C.c_double), ("thresh_abs", C.c_int), ("skip", C.c_int),
        ("poffset", C.c_int), ("qoffset", C.c_int), ("interpolate", C.c_int),
        ("filter", C.c_int), ("kr", C.c_double), ("hires", C.c_int),
    ]


class ODerived(C.Structure):
    _fields_ = [("nsize", C.c_int), ("thresh_abs_value", C.c_double),
                ("xoffset", C.c_int), ("yoffset", C.c_int),
                ("global_mode", C.c_int)]


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (gcc only)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB_PATH


def reference_source() -> str:
    """The reference's source/ directory: $FLCT_REFERENCE_SOURCE, else
    source/ of a checkout named `reference` beside this repository, else ''."""
    env = os.environ.get("FLCT_REFERENCE_SOURCE", "")
    if env:
        return env
    sib = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference", "source")
    return sib if os.path.isdir(sib) else ""


def build_ref() -> bool:
    """Compile the reference in place into _ref/ when its sources exist."""
    src = reference_source()
    if not src or not os.path.exists(os.path.join(src, "flct.c")):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + src], check=True)
    return True


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(LIB_PATH)
            dp = C.POINTER(C.c_double)
            L.oflct_velocity.argtypes = [C.POINTER(OParams), dp, dp, C.c_int, C.c_int,
                                         dp, dp, dp, C.c_int]
            L.oflct_derive.argtypes = [C.POINTER(OParams), dp, dp, C.c_int, C.c_int,
                                       C.POINTER(ODerived)]
            L.oflct_cross_cor.argtypes = [dp, dp, C.c_int, C.c_int, C.c_int, C.c_double,
                                          C.c_int, dp, dp, dp]
            L.oflct_cross_cor_batch.argtypes = [dp, dp, C.c_int, C.c_int, C.c_int,
                                                C.c_double, dp, dp, C.c_int]
            L.oflct_extract_window.argtypes = [C.POINTER(OParams), dp, dp, C.c_int, C.c_int,
                                               C.c_int, C.c_int, dp, dp, C.POINTER(C.c_int)]
            L.oflct_peak_fit.argtypes = [dp, C.c_int, C.c_int, C.POINTER(C.c_int),
                                         C.POINTER(C.c_int), dp, dp]
            L.oflct_peak_fit.restype = None
            L.oflct_interpcc2d.argtypes = [dp, C.c_double, C.c_int, C.c_int, dp, C.c_int,
                                           dp, C.c_int, dp]
            L.oflct_shift_frac2d.argtypes = [dp, C.c_double, C.c_double, dp, C.c_int,
                                             C.c_int, C.c_int]
            L.oflct_warp_frac2d.argtypes = [dp, dp, dp, dp, C.c_int, C.c_int, C.c_int,
                                            C.c_int]
            _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _c(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def make_params(deltat=1.0, deltas=1.0, sigma=4.0, thresh=0.0, thresh_abs=False,
                skip=0, poffset=0, qoffset=0, interpolate=False, kr=None,
                hires=False) -> OParams:
    return OParams(deltat, deltas, sigma, thresh, int(bool(thresh_abs)), skip, poffset,
                   qoffset, int(bool(interpolate)), 0 if kr is None else 1,
                   0.0 if kr is None else float(kr), int(bool(hires)))


class OracleError(RuntimeError):
    def __init__(self, code):
        super().__init__(f"oracle status {code}")
        self.code = code


def derive(f1, f2, **kw):
    f1, f2 = _c(f1), _c(f2)
    d = ODerived()
    p = make_params(**kw)
    rc = lib().oflct_derive(C.byref(p), _p(f1), _p(f2), f1.shape[0], f1.shape[1],
                            C.byref(d))
    if rc:
        raise OracleError(rc)
    return d


def velocity(f1, f2, nthreads=None, **kw):
    """FLCT velocity (vx, vy, vm) of C-order images f1, f2 [nx][ny]."""
    f1, f2 = _c(f1), _c(f2)
    nx, ny = f1.shape
    p = make_params(**kw)
    out = [np.empty((nx, ny)) for _ in range(3)]
    nt = nthreads or os.cpu_count() or 1
    rc = lib().oflct_velocity(C.byref(p), _p(f1), _p(f2), nx, ny, *[_p(o) for o in out], nt)
    if rc:
        raise OracleError(rc)
    if p.sigma <= 0:
        return tuple(o.reshape(-1)[:1].reshape(1, 1).copy() for o in out)
    return tuple(out)


def extract_window(f1, f2, i, j, **kw):
    """The windowed sub-images (g1, g2) the velocity loop uses at (i, j)."""
    f1, f2 = _c(f1), _c(f2)
    p = make_params(**kw)
    d = derive(f1, f2, **kw)
    n = 2 * d.nsize
    g1, g2 = np.empty((n, n)), np.empty((n, n))
    nn = C.c_int()
    rc = lib().oflct_extract_window(C.byref(p), _p(f1), _p(f2), f1.shape[0], f1.shape[1],
                                    int(i), int(j), _p(g1), _p(g2), C.byref(nn))
    if rc:
        raise OracleError(rc)
    return g1, g2


def cross_cor(g1, g2, kr=None, hires=False, want_abs=False):
    g1, g2 = _c(g1), _c(g2)
    n0, n1 = g1.shape
    sx, sy = C.c_double(), C.c_double()
    ab = np.empty((n0, n1)) if want_abs else None
    rc = lib().oflct_cross_cor(_p(g1), _p(g2), n0, n1, 0 if kr is None else 1,
                               0.0 if kr is None else float(kr), int(bool(hires)),
                               C.byref(sx), C.byref(sy),
                               _p(ab) if want_abs else None)
    if rc:
        raise OracleError(rc)
    return (sx.value, sy.value, ab) if want_abs else (sx.value, sy.value)


def cross_cor_batch(g1, g2, kr=None, nthreads=None):
    """Shifts of nwin windows g1[w], g2[w] (arrays of shape (nwin, n, n))."""
    g1, g2 = _c(g1), _c(g2)
    nwin, n, _ = g1.shape
    sx, sy = np.empty(nwin), np.empty(nwin)
    rc = lib().oflct_cross_cor_batch(_p(g1), _p(g2), n, nwin, 0 if kr is None else 1,
                                     0.0 if kr is None else float(kr), _p(sx), _p(sy),
                                     nthreads or os.cpu_count() or 1)
    if rc:
        raise OracleError(rc)
    return sx, sy


def peak_fit(absccor):
    a = _c(absccor)
    ix, iy = C.c_int(), C.c_int()
    sx, sy = C.c_double(), C.c_double()
    lib().oflct_peak_fit(_p(a), a.shape[0], a.shape[1], C.byref(ix), C.byref(iy),
                         C.byref(sx), C.byref(sy))
    return ix.value, iy.value, sx.value, sy.value


def interpcc2d(fdata, xmiss, xwant, ywant):
    f = _c(fdata)
    xw, yw = _c(xwant), _c(ywant)
    out = np.empty((xw.size, yw.size))
    rc = lib().oflct_interpcc2d(_p(f), xmiss, f.shape[0], f.shape[1], _p(xw), xw.size,
                                _p(yw), yw.size, _p(out))
    if rc:
        raise OracleError(rc)
    return out


def shift_frac2d(arr, delx, dely, transp=1):
    a = _c(arr)
    out = np.empty_like(a)
    rc = lib().oflct_shift_frac2d(_p(a), float(delx), float(dely), _p(out), a.shape[0],
                                  a.shape[1], transp)
    if rc:
        raise OracleError(rc)
    return out


def warp_frac2d(arr, delx, dely, transp=1, nthreads=None):
    a, dx, dy = _c(arr), _c(delx), _c(dely)
    out = np.empty_like(a)
    rc = lib().oflct_warp_frac2d(_p(a), _p(dx), _p(dy), _p(out), a.shape[0], a.shape[1],
                                 transp, nthreads or os.cpu_count() or 1)
    if rc:
        raise OracleError(rc)
    return out


# ------------------------------------------------ vel_ccor files (oracle) --

def write_vc(path, *arrays):
    """vel_ccor file: big-endian magic, IDL dims (fast, slow), float32 arrays
    (flct.c:1182-1259, 2016-2109).  Arrays are C-order [nx][ny]."""
    nx, ny = arrays[0].shape
    with open(path, "wb") as fh:
        fh.write(np.array([VCID, ny, nx], dtype=">i4").tobytes())
        for a in arrays:
            fh.write(np.ascontiguousarray(a, dtype=">f4").tobytes())


def read_vc(path, count):
    b = open(path, "rb").read()
    magic, ny, nx = np.frombuffer(b[:12], ">i4")
    if magic != VCID:
        raise ValueError("not a vel_ccor file")
    a = np.frombuffer(b[12:12 + 4 * count * nx * ny], ">f4").astype(np.float64)
    return [x.reshape(nx, ny) for x in a.reshape(count, nx * ny)]


def ref_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "flct")) and os.path.exists(
        os.path.join(REF_DIR, "warp"))


def ref_flct(f1, f2, workdir, args):
    """Run the compiled reference flct CLI on float32-rounded images."""
    inp = os.path.join(workdir, "ref_in.dat")
    outp = os.path.join(workdir, "ref_out.dat")
    write_vc(inp, f1, f2)
    cmd = [os.path.join(REF_DIR, "flct"), inp, outp] + [str(a) for a in args] + ["-q"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r, (read_vc(outp, 3) if r.returncode == 0 else None)
