"""The flct / warp drop-in programs end to end on the GPU: vel_ccor files in,
vel_ccor files out, checked against the reference's shipped test
(hashgauss.dat -> testgaussvel.dat), the golden command-line cases and the
golden warp cases.  The files hold float32, so outputs are compared after
the same rounding."""
import os
import subprocess

import numpy as np
import pytest

import pyoracle as po
from _compare import TOL
from _golden import cli_cases, load

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "pyflct_gb300", "bin")


@pytest.fixture(scope="module", autouse=True)
def built():
    from pyflct_gb300 import build
    build.build()


def run(prog, *args):
    return subprocess.run([os.path.join(BIN, prog)] + [str(a) for a in args], capture_output=True, text=True)


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def test_reference_shipped_test(tmp_path):
    """flct hashgauss.dat testgaussvel.dat 1 1 5 -k 0.5 (the reference's README test)."""
    z = load("reference_tests.npz")
    inp, out = tmp_path / "hashgauss.dat", tmp_path / "testgaussvel.dat"
    po.write_vc(inp, z["f1"], z["f2"])
    r = run("flct", inp, out, 1, 1, 5, "-k", 0.5, "-q")
    assert r.returncode == 0, r.stdout
    vx, vy, vm = po.read_vc(out, 3)
    assert np.array_equal(vm, f32(z["vm"]))
    ok = vm == 1
    assert np.abs(vx - f32(z["vx"]))[ok].max() <= TOL + 1e-6
    assert np.abs(vy - f32(z["vy"]))[ok].max() <= TOL + 1e-6
    # verbose run prints the banner and finishes
    r = run("flct", inp, out, 1, 1, 5, "-k", 0.5)
    assert r.returncode == 0 and "flct: finished" in r.stdout


@pytest.mark.parametrize("case", cli_cases(), ids=lambda c: c[0])
def test_golden_cli_case(tmp_path, case):
    name, args, rc, f1, f2, golden = case
    inp, out = tmp_path / "in.dat", tmp_path / "out.dat"
    po.write_vc(inp, f1, f2)
    r = run("flct", inp, out, *args, "-q")
    assert r.returncode == rc, (name, r.stdout)
    if rc != 0:
        return
    got = po.read_vc(out, 3)
    assert got[0].shape == golden[0].shape
    assert np.array_equal(got[2], f32(golden[2])), name
    ok = got[2] == 1
    for g, ref in zip(got[:2], golden[:2]):
        assert np.array_equal(np.isnan(g), np.isnan(ref))
        d = np.abs(g - f32(ref))[ok & ~np.isnan(g)]
        assert d.size == 0 or d.max() <= TOL + 1e-5, (name, d.max())


def test_golden_warp_and_shift(tmp_path):
    z = load("ref_warp_cases.npz")
    img, sh, out = tmp_path / "img.dat", tmp_path / "sh.dat", tmp_path / "out.dat"
    po.write_vc(img, z["warp_img"])
    po.write_vc(sh, z["warp_dx"], z["warp_dy"])
    r = run("warp", img, sh, out, "-q")
    assert r.returncode == 0, r.stdout
    (w,) = po.read_vc(out, 1)
    ref = f32(z["warp_out"])
    assert np.abs(w - ref).max() <= 2e-5 * np.abs(ref).max() + 1e-6
    dx, dy = z["shift_xy"][0], z["shift_xy"][1]
    po.write_vc(sh, np.full((1, 1), dx), np.full((1, 1), dy))
    r = run("warp", img, sh, out)
    assert r.returncode == 0 and "warp: finished" in r.stdout
    (s,) = po.read_vc(out, 1)
    ref = f32(z["shift_out"])
    assert np.abs(s - ref).max() <= 2e-5 * np.abs(ref).max() + 1e-6
