"""Pin the CPU oracle (C restatement) to the reference's golden vectors.

The oracle is only trusted as a checker once it reproduces (a) the fixture
the reference ships (tests/testgaussvel.dat: flct hashgauss.dat 1 1 5 -k 0.5)
and (b) outputs of the unmodified reference compiled here, recorded under
tests/golden/ by make_golden.py.
"""
import numpy as np
import pytest

import pyoracle as po
from _golden import cli_cases, load, parse_cli_args, window_cases


def test_reference_shipped_fixture():
    z = load("reference_tests.npz")
    f1, f2 = z["f1"].astype(np.float64), z["f2"].astype(np.float64)
    vx, vy, vm = po.velocity(f1, f2, nthreads=4, deltat=1, deltas=1, sigma=5, kr=0.5)
    # the fixture is float32; the reference's float64 results round to it
    assert np.abs(vx - z["vx"]).max() < 2e-6
    assert np.abs(vy - z["vy"]).max() < 2e-6
    assert np.array_equal(vm, z["vm"].astype(np.float64))
    # physics sanity: the recovered field follows the applied shifts
    assert np.sqrt(np.mean((vx - z["deltax"]) ** 2)) < 0.08
    assert np.sqrt(np.mean((vy - z["deltay"]) ** 2)) < 0.08


@pytest.mark.parametrize("case", cli_cases(), ids=lambda c: c[0])
def test_cli_case(case):
    name, args, rc, f1, f2, ref = case
    kw = parse_cli_args(args)
    if rc != 0:
        with pytest.raises(po.OracleError):
            po.velocity(f1, f2, nthreads=2, **kw)
        return
    got = po.velocity(f1, f2, nthreads=2, **kw)
    for g, r in zip(got, ref):
        g32 = g.astype(np.float32).astype(np.float64)
        r = r.reshape(g32.shape) if r.size == g32.size else r[: g32.shape[0], : g32.shape[1]]
        # bit-identical after the file format's float32 rounding (NaN == NaN)
        assert np.array_equal(g32, r, equal_nan=True), name


@pytest.mark.parametrize("wc", window_cases(), ids=lambda w: f"n{w[0]}_kr{w[1]}")
def test_window_case(wc):
    n, kr, g1, g2, sx, sy = wc
    for w in range(g1.shape[0]):
        a, b = po.cross_cor(g1[w], g2[w], kr=kr)
        assert a == sx[w] and b == sy[w]
    bx, by = po.cross_cor_batch(g1, g2, kr=kr, nthreads=3)
    assert np.array_equal(bx, sx) and np.array_equal(by, sy)


def test_interp_cases():
    z = load("ref_interp_cases.npz")
    for q in range(int(z["count"])):
        out = po.interpcc2d(z[f"i{q}_f"], float(z[f"i{q}_xmiss"]), z[f"i{q}_xw"], z[f"i{q}_yw"])
        assert np.array_equal(out, z[f"i{q}_out"])


def test_warp_cases():
    z = load("ref_warp_cases.npz")
    img = z["warp_img"].astype(np.float64)
    out = po.warp_frac2d(img, z["warp_dx"].astype(np.float64), z["warp_dy"].astype(np.float64),
                         nthreads=2)
    assert np.array_equal(out.astype(np.float32), z["warp_out"])
    sx, sy = (float(v) for v in z["shift_xy"])
    out = po.shift_frac2d(img, sx, sy)
    assert np.array_equal(out.astype(np.float32), z["shift_out"])


def test_warp_shift_equivalence():
    """A constant field through the non-uniform warp equals the uniform shift
    (the reference CLI picks one or the other by the shift-file size)."""
    rng = np.random.default_rng(5)
    img = rng.standard_normal((12, 10))
    dx, dy = np.full((12, 10), 0.3), np.full((12, 10), -0.8)
    a = po.warp_frac2d(img, dx, dy, nthreads=1)
    b = po.shift_frac2d(img, 0.3, -0.8)
    assert np.abs(a - b).max() < 1e-12


def test_status_codes_match_product_header():
    import os, re
    hdr = open(os.path.join(os.path.dirname(__file__), "..", "include", "flct_gpu.h")).read()
    orc = open(os.path.join(os.path.dirname(po.__file__), "flct_oracle.h")).read()
    for name in ("ARG", "SKIP_NONPOSITIVE", "SKIP_OFFSET", "SKIP_TOO_BIG", "BOX_SIZE",
                 "GRID_TOO_SMALL", "ALLOC", "WARP_DIMS"):
        a = re.search(r"FLCT_ERR_%s\s*=\s*(\d+)" % name, hdr)
        b = re.search(r"OFLCT_ERR_%s\s+(\d+)" % name, orc)
        assert a and b and a.group(1) == b.group(1), name
