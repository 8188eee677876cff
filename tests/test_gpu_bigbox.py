"""GPU parity of boxes above 64 (sigma >= 16) against the FP64 oracle.

The reference derives the box from sigma without an upper limit
(flct.c:567-580); boxes above 64 run the big-box FP32 kernel (one window
per CTA in shared memory, direct DFTs).  Tolerance: max |dv| <= 1e-3
px/frame, bit-exact mask, integer peaks identical except at documented ties.
"""
import numpy as np
import pytest

import pyoracle as po
from _compare import TIE_REL, TOL, compare
from _golden import parse_cli_args

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def gpu():
    from pyflct_gb300 import _lib, build
    build.build()
    return _lib.context(0)


@pytest.mark.parametrize("n", [68, 84, 100, 128])
def test_direct_windows_big(n):
    from pyflct_gb300 import synth
    from pyflct_gb300.flct import cross_cor
    rng = np.random.default_rng(3000 + n)
    g1 = np.empty((12, n, n))
    g2 = np.empty((12, n, n))
    for k in range(12):
        f = synth.kfield((n + 8, n + 8), rng)
        s = synth.fourier_shift(f, *rng.uniform(-2, 2, 2))
        g1[k], g2[k] = f[4:4 + n, 4:4 + n], s[4:4 + n, 4:4 + n]
    for kr in (None, 0.5):
        ox, oy = po.cross_cor_batch(g1, g2, kr=kr)
        gx, gy = cross_cor(g1, g2, kr=kr, form="fp32")
        d = np.maximum(np.abs(gx - ox), np.abs(gy - oy))
        for k in np.nonzero(d > TOL)[0]:
            _, _, ab = po.cross_cor(g1[k], g2[k], kr=kr, want_abs=True)
            I = int(np.floor(gx[k] + n // 2 + 0.5))
            J = int(np.floor(gy[k] + n // 2 + 0.5))
            near = any(0 <= I + a < n and 0 <= J + b < n and ab[I + a, J + b] >= (1 - TIE_REL) * ab.max()
                       for a in (-1, 0, 1) for b in (-1, 0, 1))
            assert near, (n, kr, int(k), float(d[k]))
        print(n, kr, "max |d|", float(d.max()))


@pytest.mark.parametrize("sigma,shape,extra", [
    (16.0, (210, 220), {}), (16.0, (214, 208), {"kr": 0.5, "skip": "3i"}),
    (20.0, (260, 256), {"skip": "2", "hires": True}), (24.0, (310, 304), {"skip": "3i", "thresh": 0.2}),
])
def test_velocity_big_boxes(sigma, shape, extra):
    from pyflct_gb300 import synth
    from pyflct_gb300.flct import flct
    rng = np.random.default_rng(int(sigma) * 7)
    f1 = synth.kfield(shape, rng)
    f2 = synth.fourier_shift(f1, *rng.uniform(-1.5, 1.5, 2))
    args = [1, 1, sigma]
    for k, v in extra.items():
        args += {"kr": ["-k", v], "skip": ["-s", v], "thresh": ["-t", v], "hires": ["-h"]}[k]
    kw = parse_cli_args(args)
    assert 2 * po.derive(f1, f2, **kw).nsize > 64
    ref = po.velocity(f1, f2, **kw)
    for form in ("fp32", "auto"):
        got = flct(f1, f2, 1.0, 1.0, sigma, form=form, **extra)
        rep = compare(f1, f2, got, ref, kw)
        print(form, sigma, extra, rep)


def test_big_box_in_batch_and_tc_refused():
    from pyflct_gb300 import _lib, synth
    from pyflct_gb300.flct import FlctError, flct, flct_batch, make_params
    rng = np.random.default_rng(77)
    frames, params = [], []
    for shape, sigma in (((210, 215), 16.0), ((96, 100), 8.0), ((220, 212), 16.0)):
        f1 = synth.kfield(shape, rng)
        frames.append((f1, synth.fourier_shift(f1, *rng.uniform(-1, 1, 2))))
        params.append(make_params(1.0, 1.0, sigma))
    out = flct_batch(frames, params)
    for (f1, f2), p, got in zip(frames, params, out):
        want = flct(f1, f2, 1.0, 1.0, p.sigma)
        for x, y in zip(got, want):
            assert np.array_equal(x, y)
    f1, f2 = frames[0]
    with pytest.raises(FlctError) as e:
        flct(f1, f2, 1.0, 1.0, 16.0, form="tc_fp16")
    assert e.value.code == _lib.ERR_UNSUPPORTED
