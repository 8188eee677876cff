"""Comparison of GPU velocities with the FP64 oracle, with tie handling.

The GPU computes |c| in FP32 (or split precision), the oracle in FP64.  The
integer peak must be identical except at documented ties: windows whose FP64
|c| has another value within TIE_REL of the maximum at the GPU's peak.  Those
windows are reported, not failed, and the interpolated pixels whose stencil
touches them are excluded from the interpolated comparison.
"""
import numpy as np

import pyoracle as po

TOL = 1e-3        # max |dv| in px/frame against the FP64 oracle
TIE_REL = 2e-4    # relative |c| gap below which two maxima count as a tie


def classify_ties(f1, f2, vx_g, vy_g, vx_o, vy_o, bad, kw):
    """For each bad computed pixel, decide whether it is an argmax tie."""
    d = po.derive(f1, f2, **kw)
    n = 2 * d.nsize
    deltinv_ds = kw.get("deltas", 1.0) / kw.get("deltat", 1.0)
    ties, real = [], []
    for (i, j) in zip(*np.nonzero(bad)):
        g1, g2 = po.extract_window(f1, f2, i, j, **kw)
        _, _, ab = po.cross_cor(g1, g2, kr=kw.get("kr"), want_abs=True)
        # GPU's integer peak: shift + n/2 rounded (sub-pixel part is < 1)
        I = int(np.floor(vy_g[i, j] / deltinv_ds + n // 2 + 0.5))
        J = int(np.floor(vx_g[i, j] / deltinv_ds + n // 2 + 0.5))
        m = ab.max()
        near = False
        for di in (-1, 0, 1):
            for dj in (-1, 0, 1):
                a, b = I + di, J + dj
                if 0 <= a < n and 0 <= b < n and ab[a, b] >= (1 - TIE_REL) * m:
                    near = True
        (ties if near else real).append((int(i), int(j)))
    return ties, real


def compare(f1, f2, got, ref, kw, tol=TOL):
    """Return a report dict; raises AssertionError on a parity failure."""
    vx_g, vy_g, vm_g = got
    vx_o, vy_o, vm_o = ref
    assert np.array_equal(vm_g, vm_o), f"mask differs at {np.argwhere(vm_g != vm_o)[:5]}"
    comp = vm_o == 1.0
    nanmask = np.isnan(vx_o) | np.isnan(vy_o)
    assert np.array_equal(np.isnan(vx_g), np.isnan(vx_o))
    assert np.array_equal(np.isnan(vy_g), np.isnan(vy_o))
    dx = np.where(nanmask, 0.0, np.abs(vx_g - vx_o))
    dy = np.where(nanmask, 0.0, np.abs(vy_g - vy_o))
    bad = comp & ((dx > tol) | (dy > tol))
    ties, real = classify_ties(f1, f2, vx_g, vy_g, vx_o, vy_o, bad, kw) if bad.any() else ([], [])
    assert not real, f"{len(real)} non-tie velocity mismatches, e.g. {real[:5]}"
    ok = comp & ~bad
    rep = {
        "computed": int(comp.sum()),
        "ties": len(ties),
        "max_dv": float(max(dx[ok].max(initial=0.0), dy[ok].max(initial=0.0))),
        "rms_dv": float(np.sqrt(np.mean(np.concatenate([dx[ok], dy[ok]]) ** 2))) if ok.any() else 0.0,
    }
    interp = vm_o == 0.5
    if interp.any():
        excl = np.zeros_like(interp)
        skip = kw.get("skip", 0)
        for (i, j) in ties:
            excl[max(0, i - 3 * skip):i + 3 * skip + 1, max(0, j - 3 * skip):j + 3 * skip + 1] = True
        sel = interp & ~excl
        di = np.maximum(dx, dy)[sel]
        assert di.max(initial=0.0) <= tol, f"interpolated max |dv| {di.max()}"
        rep["interp_max_dv"] = float(di.max(initial=0.0))
    return rep
