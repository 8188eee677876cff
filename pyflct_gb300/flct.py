"""Python front end mirroring the reference's flct / warp interface.

The reference exposes two programs (source/flct.c main, source/warp.c main)
whose arguments are ``flct ifile ofile deltat deltas sigma [-t thr[a]]
[-k kr] [-s N[pP][qQ][i]] [-h] [-q]`` and ``warp ifile sfile ofile [-q]``.
These functions take the same parameters with the same meaning, on numpy
arrays in the reference's C order ([nx][ny], nx = slow axis = IDL y), and run
them on the GPU through the C ABI.  Fatal argument errors of the reference
(exit 1 with a message) raise FlctError with the matching status code.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import FlctError, Params

__all__ = ["flct", "make_params", "parse_skip", "parse_thresh", "cross_cor", "interpcc2d",
           "shift_frac2d", "warp_frac2d", "warp", "FlctBatch", "flct_batch", "FlctError"]


def parse_thresh(thresh) -> tuple[float, bool]:
    """'-t' value: a number, or a string whose 'a' forces absolute units
    (flct.c:384-397)."""
    if thresh is None:
        return 0.0, False
    if isinstance(thresh, str):
        s = thresh
        absolute = "a" in s
        if absolute:
            s = s[: s.index("a")]
        return _atof(s), absolute
    return float(thresh), False


def _atof(s: str) -> float:
    """C atof: the longest leading number, 0.0 when there is none."""
    s = s.strip()
    best = 0.0
    for k in range(len(s), 0, -1):
        try:
            best = float(s[:k])
            break
        except ValueError:
            continue
    return best


def _atoi(s: str) -> int:
    s = s.strip()
    k = 0
    if k < len(s) and s[k] in "+-":
        k += 1
    while k < len(s) and s[k].isdigit():
        k += 1
    try:
        return int(s[:k])
    except ValueError:
        return 0


def parse_skip(skip) -> tuple[int, int, int, bool]:
    """'-s N[pP][qQ][i]' (flct.c:398-453) -> (N, p, q, interpolate).  An int
    means N alone.  N <= 0 is returned as -1 (the reference's fatal
    "skip is zero or negative")."""
    if skip is None:
        return 0, 0, 0, False
    if not isinstance(skip, str):
        n = int(skip)
        return (n if n > 0 else -1), 0, 0, False
    s = skip
    interp = "i" in s
    if interp:
        s = s[: s.index("i")]
    q = p = 0
    if "q" in s:
        k = s.index("q")
        q = _atoi(s[k + 1:])
        s = s[:k]
    if "p" in s:
        k = s.index("p")
        p = _atoi(s[k + 1:])
        s = s[:k]
    n = _atoi(s)
    return (n if n > 0 else -1), p, q, interp


def make_params(deltat, deltas, sigma, thresh=None, kr=None, skip=None, hires=False,
                quiet=True, form="fp32") -> Params:
    t, tabs = parse_thresh(thresh)
    n, p, q, interp = parse_skip(skip)
    return Params(float(deltat), float(deltas), float(sigma), t, int(tabs), n, p, q, int(interp),
                  0 if kr is None else 1, 0.0 if kr is None else float(kr), int(bool(hires)),
                  int(bool(quiet)), _lib.FORMS[form] if isinstance(form, str) else int(form))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def flct(f1, f2, deltat, deltas, sigma, thresh=None, kr=None, skip=None, hires=False,
         quiet=True, form="fp32", device=0):
    """Velocity field (vx, vy, vm) from two frames, like ``flct``.

    f1, f2: 2-D arrays [nx][ny].  Returns three float64 arrays of the same
    shape (1x1 in the global-shift mode sigma <= 0)."""
    f1, f2 = _f64(f1), _f64(f2)
    if f1.ndim != 2 or f1.shape != f2.shape:
        raise FlctError(_lib.ERR_ARG, "f1 and f2 must be 2-D arrays of one shape")
    ctx = _lib.context(device)
    p = make_params(deltat, deltas, sigma, thresh, kr, skip, hires, quiet, form)
    nx, ny = f1.shape
    nout = ctx.lib.flct_gpu_output_len(C.byref(p), nx, ny)
    shape = (nx, ny) if nout == nx * ny else (1, 1)
    out = [np.empty(shape) for _ in range(3)]
    ctx.check(ctx.lib.flct_gpu_velocity(ctx.h, C.byref(p), _dp(f1), _dp(f2), nx, ny,
                                        *[_dp(o) for o in out]))
    return tuple(out)


def cross_cor(g1, g2, kr=None, form="fp32", device=0):
    """Shifts (shiftx, shifty) of stacks of n x n windows, like cross_cor.

    g1, g2: arrays (nwin, n, n) or (n, n)."""
    g1, g2 = _f64(g1), _f64(g2)
    single = g1.ndim == 2
    if single:
        g1, g2 = g1[None], g2[None]
    if g1.ndim != 3 or g1.shape != g2.shape or g1.shape[1] != g1.shape[2]:
        raise FlctError(_lib.ERR_ARG, "windows must be square and of one shape")
    nwin, n, _ = g1.shape
    sx, sy = np.empty(nwin), np.empty(nwin)
    ctx = _lib.context(device)
    ctx.check(ctx.lib.flct_gpu_cross_cor_batch(
        ctx.h, _dp(g1), _dp(g2), n, nwin, 0 if kr is None else 1,
        0.0 if kr is None else float(kr), _lib.FORMS[form] if isinstance(form, str) else int(form),
        _dp(sx), _dp(sy)))
    return (sx[0], sy[0]) if single else (sx, sy)


def interpcc2d(fdata, xmiss, xwant, ywant, device=0):
    """Cubic-convolution interpolation of fdata at (xwant x ywant)."""
    f = _f64(fdata)
    xw, yw = _f64(xwant).ravel(), _f64(ywant).ravel()
    out = np.empty((xw.size, yw.size))
    ctx = _lib.context(device)
    ctx.check(ctx.lib.flct_gpu_interpcc2d(ctx.h, _dp(f), float(xmiss), f.shape[0], f.shape[1],
                                          _dp(xw), xw.size, _dp(yw), yw.size, _dp(out)))
    return out


def shift_frac2d(arr, delx, dely, transp=1, device=0):
    a = _f64(arr)
    out = np.empty_like(a)
    ctx = _lib.context(device)
    ctx.check(ctx.lib.flct_gpu_shift_frac2d(ctx.h, _dp(a), float(delx), float(dely), _dp(out),
                                            a.shape[0], a.shape[1], int(transp)))
    return out


def warp_frac2d(arr, delx, dely, transp=1, device=0):
    a, dx, dy = _f64(arr), _f64(delx), _f64(dely)
    out = np.empty_like(a)
    ctx = _lib.context(device)
    ctx.check(ctx.lib.flct_gpu_warp_frac2d(ctx.h, _dp(a), _dp(dx), _dp(dy), _dp(out),
                                           a.shape[0], a.shape[1], int(transp)))
    return out


def warp(arr, delx, dely, device=0):
    """The warp program's dispatch (warp.c:163-188): shift arrays of the
    image's shape warp non-uniformly, 1x1 arrays shift uniformly, anything
    else is an error."""
    a = _f64(arr)
    dx, dy = np.atleast_2d(_f64(delx)), np.atleast_2d(_f64(dely))
    if dx.shape == a.shape and dy.shape == a.shape:
        return warp_frac2d(a, dx, dy, 1, device)
    if dx.shape == (1, 1) and dy.shape == (1, 1):
        return shift_frac2d(a, dx[0, 0], dy[0, 0], 1, device)
    raise FlctError(_lib.ERR_WARP_DIMS,
                    f"warp: bad shift arrays: nx={a.shape[0]}, nxdel={dx.shape[0]}, "
                    f"ny={a.shape[1]}, nydel={dx.shape[1]}")


class FlctBatch:
    """Many frame pairs of uneven sizes and sigmas in one batched GPU call
    (flct_gpu_velocity_batch): device-resident inputs and outputs, so that
    repeated runs replay the library's captured CUDA graph.

    shapes: sequence of (nx, ny); params: one flct_params per pair (from
    make_params).  f1[k], f2[k] are float64 CUDA tensors [nx][ny] to fill;
    run() computes vx[k], vy[k], vm[k] on the current torch stream."""

    def __init__(self, shapes, params, device=0):
        import torch
        if len(shapes) != len(params):
            raise FlctError(_lib.ERR_ARG, "one params entry per pair is required")
        # a context of its own: the captured graph and its workspace stay
        # valid while other calls use the shared context
        self.ctx = _lib.Context(device)
        dev = torch.device("cuda", device)
        self.device = dev
        z = lambda s: torch.zeros(s, dtype=torch.float64, device=dev)
        self.f1 = [z(tuple(s)) for s in shapes]
        self.f2 = [z(tuple(s)) for s in shapes]
        self.vx = [z(tuple(s)) for s in shapes]
        self.vy = [z(tuple(s)) for s in shapes]
        self.vm = [z(tuple(s)) for s in shapes]
        self.pairs = (_lib.Pair * max(1, len(shapes)))()
        for k, ((nx, ny), p) in enumerate(zip(shapes, params)):
            q = self.pairs[k]
            q.f1, q.f2 = self.f1[k].data_ptr(), self.f2[k].data_ptr()
            q.nx, q.ny = int(nx), int(ny)
            q.params = p
            q.vx, q.vy, q.vm = self.vx[k].data_ptr(), self.vy[k].data_ptr(), self.vm[k].data_ptr()
        self.npairs = len(shapes)

    def load(self, frames):
        """Copy (f1, f2) arrays of each pair into the device inputs."""
        import torch
        for k, (a, b) in enumerate(frames):
            self.f1[k].copy_(torch.as_tensor(_f64(a)), non_blocking=False)
            self.f2[k].copy_(torch.as_tensor(_f64(b)), non_blocking=False)
        return self

    def run(self, stream=None):
        import torch
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        self.ctx.check(self.ctx.lib.flct_gpu_velocity_batch(self.ctx.h, self.npairs, self.pairs,
                                                             C.c_void_p(st.cuda_stream)))

    def timing(self):
        return self.ctx.timing()


def flct_batch(frames, params, device=0):
    """Velocity fields of many pairs [(f1, f2), ...] (numpy arrays [nx][ny])
    with one params per pair, in one batched GPU call.  Returns a list of
    (vx, vy, vm) numpy arrays."""
    shapes = [np.shape(a) for a, _ in frames]
    b = FlctBatch(shapes, params, device)
    b.load(frames)
    b.run()
    import torch
    torch.cuda.synchronize(b.device)
    return [(b.vx[k].cpu().numpy(), b.vy[k].cpu().numpy(), b.vm[k].cpu().numpy())
            for k in range(len(frames))]
