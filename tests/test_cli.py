"""The flct / warp drop-in programs on the CPU side: command-line handling
and vel_ccor file errors, which the programs finish before touching the
GPU.  Where the reference's own programs are built (oracle/_ref), the
messages and exit codes are compared with theirs."""
import os
import subprocess

import numpy as np
import pytest

import pyoracle as po

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "pyflct_gb300", "bin")


@pytest.fixture(scope="module", autouse=True)
def built():
    from pyflct_gb300 import build
    build.build()


def run(prog, *args, cwd=None):
    return subprocess.run([os.path.join(BIN, prog)] + [str(a) for a in args], capture_output=True, text=True,
                          cwd=cwd)


def test_usage_exits_1():
    for prog, args in (("flct", ()), ("flct", ("a",) * 14), ("warp", ("a", "b")), ("warp", ("a",) * 6)):
        r = run(prog, *args)
        assert r.returncode == 1 and "Syntax:" in r.stdout


@pytest.mark.parametrize("args,msg", [
    (["-s", "0"], "flct: skip =0 is zero or negative, fatal"),
    (["-s", "-3"], "flct: skip =-3 is zero or negative, fatal"),
    (["-s", "3p3"], "flct: p=3,q=0, abs(p) or abs(q) >= skip=3"),
    (["-s", "4q-4i"], "flct: p=0,q=-4, abs(p) or abs(q) >= skip=4"),
])
def test_skip_errors_before_reading(tmp_path, args, msg):
    r = run("flct", tmp_path / "missing.dat", tmp_path / "out.dat", 1, 1, 4, *args)
    assert r.returncode == 1 and r.stdout.strip().splitlines()[-1] == msg
    if po.ref_available():
        ref = subprocess.run([os.path.join(po.REF_DIR, "flct"), str(tmp_path / "missing.dat"),
                              str(tmp_path / "out.dat"), "1", "1", "4"] + args, capture_output=True, text=True)
        assert ref.returncode == 1 and ref.stdout.strip().splitlines()[-1] == msg


def test_file_errors(tmp_path):
    r = run("flct", tmp_path / "missing.dat", tmp_path / "o.dat", 1, 1, 4, "-q")
    assert r.returncode == 1 and "read2images: cannot open file" in r.stdout
    bad = tmp_path / "bad.dat"
    bad.write_bytes(b"\x00" * 64)
    r = run("flct", bad, tmp_path / "o.dat", 1, 1, 4, "-q")
    assert r.returncode == 1 and "read2images: input file is not a vel_ccor i/o file" in r.stdout
    r = run("warp", bad, bad, tmp_path / "o.dat", "-q")
    assert r.returncode == 1 and "readimage: input file is not a vel_ccor i/o file" in r.stdout
    # a truncated file
    short = tmp_path / "short.dat"
    po.write_vc(short, np.ones((8, 9)))
    r = run("flct", short, tmp_path / "o.dat", 1, 1, 4, "-q")
    assert r.returncode == 1 and "fewer than 2 arrays" in r.stdout


def test_bad_shift_arrays(tmp_path):
    img, sh = tmp_path / "img.dat", tmp_path / "sh.dat"
    po.write_vc(img, np.ones((10, 12)))
    po.write_vc(sh, np.zeros((3, 4)), np.zeros((3, 4)))
    r = run("warp", img, sh, tmp_path / "o.dat", "-q")
    assert r.returncode == 1
    assert r.stdout.strip() == "warp: bad shift arrays: nx=10, nxdel=3, ny=12, nydel=4"


def test_no_cpu_path(tmp_path):
    """Without a GPU a valid run fails loudly instead of computing on the CPU."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    inp = tmp_path / "in.dat"
    po.write_vc(inp, np.ones((20, 20)), np.ones((20, 20)))
    r = run("flct", inp, tmp_path / "o.dat", 1, 1, 3, "-q")
    assert r.returncode == 1 and "no CPU path" in r.stdout
    assert not (tmp_path / "o.dat").exists()
