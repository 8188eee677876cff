"""Regenerate the golden fixtures in this directory from the reference.

Run in an environment that has the reference tree (FLCT 1.01) and gcc:

    python tests/golden/make_golden.py [REFERENCE_ROOT]

It compiles the unmodified reference sources in place against the project's
FFTW-API shim (``make -C oracle ref``) and records:

* ``reference_tests.npz``   the reference's own fixtures (tests/hashgauss.dat,
                            tests/deltaxygauss.dat, tests/testgaussvel.dat).
* ``ref_cli_cases.npz``     inputs, argv and outputs of the reference ``flct``
                            CLI on small synthetic cases covering every option
                            (-t relative/absolute, -k, -s N[pP][qQ][i], -h,
                            sigma=0, NaN and constant regions), plus error
                            cases with their exit status.
* ``ref_window_cases.npz``  per-window ``cross_cor`` shifts (double) for
                            box sizes 12, 20, 32, 48, with and without -k.
* ``ref_interp_cases.npz``  ``interpcc2d`` outputs (double) on grids with
                            missing values and out-of-range targets.
* ``ref_warp_cases.npz``    ``warp`` outputs for a non-uniform field and a
                            uniform shift.

Inputs are float32-rounded, as the vel_ccor file format stores them.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import pyoracle as po  # noqa: E402
from pyflct_gb300 import synth  # noqa: E402


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def main(refroot=""):
    """refroot: the reference checkout (holding source/ and tests/); default
    $FLCT_REFERENCE_ROOT, else a checkout named `reference` beside this
    repository."""
    refroot = refroot or os.environ.get("FLCT_REFERENCE_ROOT", "") or \
        os.path.join(os.path.dirname(ROOT), "reference")
    os.environ["FLCT_REFERENCE_SOURCE"] = os.path.join(refroot, "source")
    if not po.build_ref():
        raise SystemExit("reference sources not found under " + refroot)
    tmp = tempfile.mkdtemp()

    # -- the reference's own fixtures -------------------------------------
    t = os.path.join(refroot, "tests")
    f1, f2 = po.read_vc(os.path.join(t, "hashgauss.dat"), 2)
    dx, dy = po.read_vc(os.path.join(t, "deltaxygauss.dat"), 2)
    vx, vy, vm = po.read_vc(os.path.join(t, "testgaussvel.dat"), 3)
    np.savez_compressed(os.path.join(HERE, "reference_tests.npz"),
                        f1=f1.astype(np.float32), f2=f2.astype(np.float32),
                        deltax=dx.astype(np.float32), deltay=dy.astype(np.float32),
                        vx=vx.astype(np.float32), vy=vy.astype(np.float32),
                        vm=vm.astype(np.float32),
                        args=json.dumps([1, 1, 5, "-k", 0.5]))

    # -- CLI cases ----------------------------------------------------------
    rng = np.random.default_rng(777)
    cases = []

    def add(name, a, b, args, expect_rc=0):
        a, b = f32(a), f32(b)
        r, out = po.ref_flct(a, b, tmp, args)
        assert r.returncode == expect_rc, (name, r.returncode, r.stdout)
        cases.append((name, a, b, args, r.returncode, out))

    c1, c2, _ = synth.config1()
    add("config1_128_sigma4", c1, c2, [1, 1, 4])
    k = synth.kfield((48, 64), rng)
    add("sig3_threl", k, synth.fourier_shift(k, 0.4, -0.7), [1, 1, 3, "-t", 0.3])
    add("sig5_thabs_kr", k, synth.fourier_shift(k, -1.2, 0.25), [1, 1, 5, "-t", "0.25a", "-k", 0.5])
    k2 = synth.kfield((60, 52), rng)
    s2 = synth.fourier_shift(k2, 0.6, 0.3)
    add("sig4_skip3_pq_interp_thr", k2, s2, [2, 0.5, 4, "-s", "3p1q-2i", "-t", 0.2])
    add("sig4_skip4_p2_nointerp", k2, s2, [1, 1, 4, "-s", "4p2"])
    k3 = synth.kfield((64, 64), rng)
    add("sig8_skip4_interp", k3, synth.fourier_shift(k3, -0.35, 0.8), [1, 1, 8, "-s", "4i"])
    k4 = synth.kfield((40, 44), rng)
    k4b = synth.fourier_shift(k4, 0.2, 0.2)
    k4[5:12, 20:30] = 1.5
    k4b[5:12, 20:30] = 1.5
    k4[30, 3] = np.nan
    add("sig3_nan_const", k4, k4b, [1, 1, 3])
    k5 = synth.kfield((50, 40), rng)
    add("sigma0_global", k5, synth.fourier_shift(k5, 1.3, -0.6), [1, 1, 0])
    add("sigma0_global_kr", k5, synth.fourier_shift(k5, -0.4, 2.2), [1, 1, 0, "-k", 0.4])
    k6 = synth.kfield((40, 40), rng)
    add("sig3_hires", k6, synth.fourier_shift(k6, 0.45, -0.15), [1, 1, 3, "-h"])
    k7 = synth.kfield((70, 72), rng)
    add("sig11_box44", k7, synth.fourier_shift(k7, 0.1, 0.9), [1, 1, 11, "-k", 0.7])
    add("sig6_box24_skip2i", k7, synth.fourier_shift(k7, -0.5, 0.5), [1, 1, 6, "-s", "2i"])
    k8 = synth.kfield((100, 104), rng)
    add("sig15_box64", k8, synth.fourier_shift(k8, 0.7, -0.3), [1, 1, 15])
    k9 = synth.kfield((33, 35), rng)
    add("sig2_box4", k9, synth.fourier_shift(k9, 0.3, 0.1), [1, 1, 2])
    # fatal argument errors: the reference prints and exits 1
    add("err_skip_zero", k9, k9, [1, 1, 3, "-s", "0"], expect_rc=1)
    add("err_skip_offset", k9, k9, [1, 1, 3, "-s", "3p3"], expect_rc=1)
    add("err_skip_too_big", k9, k9, [1, 1, 3, "-s", "33"], expect_rc=1)
    add("err_box_size", k9, k9, [1, 1, 0.5], expect_rc=1)

    blob = {}
    for idx, (name, a, b, args, rc, out) in enumerate(cases):
        blob[f"c{idx}_f1"] = a.astype(np.float32)
        blob[f"c{idx}_f2"] = b.astype(np.float32)
        if out is not None:
            for nm, arr in zip(("vx", "vy", "vm"), out):
                blob[f"c{idx}_{nm}"] = arr.astype(np.float32)
    blob["index"] = json.dumps([[name, args, rc] for name, _, _, args, rc, _ in cases])
    np.savez_compressed(os.path.join(HERE, "ref_cli_cases.npz"), **blob)

    # -- per-window cross_cor through the reference shared object -----------
    L = C.CDLL(os.path.join(po.REF_DIR, "libflctref.so"))
    dp = C.POINTER(C.c_double)
    L.cross_cor.argtypes = [C.c_int, C.c_int, C.c_int, dp, dp, C.POINTER(dp), C.c_int,
                            C.c_int, dp, dp, C.c_int, C.c_double]
    L.interpcc2d.argtypes = [dp, C.c_double, C.c_int, C.c_int, dp, C.c_int, dp, C.c_int,
                             C.POINTER(dp)]
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    win = {}
    wrng = np.random.default_rng(4242)
    gidx = 0
    for n in (12, 20, 32, 48):
        for kr in (None, 0.5):
            base = synth.kfield((n + 8, n + 8), wrng)
            sh = synth.fourier_shift(base, *wrng.uniform(-2, 2, 2))
            g1s, g2s, sxs, sys_ = [], [], [], []
            for w in range(8):
                oi, oj = wrng.integers(0, 8, 2)
                ii, jj = np.meshgrid(np.arange(n) - n / 2 + 0.5, np.arange(n) - n / 2 + 0.5,
                                     indexing="ij")
                gw = np.exp(-(ii ** 2 + jj ** 2) / (n / 2.2) ** 2)
                a = base[oi:oi + n, oj:oj + n]
                b = sh[oi:oi + n, oj:oj + n]
                g1 = f32(gw * (a - a.mean()))
                g2 = f32(gw * (b - b.mean()))
                sx, sy = C.c_double(), C.c_double()
                ab = dp()
                g1c, g2c = np.ascontiguousarray(g1), np.ascontiguousarray(g2)
                L.cross_cor(2, -1, 1, g1c.ctypes.data_as(dp), g2c.ctypes.data_as(dp),
                            C.byref(ab), n, n, C.byref(sx), C.byref(sy),
                            0 if kr is None else 1, 0.0 if kr is None else kr)
                libc.free(C.cast(ab, C.c_void_p))
                g1s.append(g1)
                g2s.append(g2)
                sxs.append(sx.value)
                sys_.append(sy.value)
            win[f"w{gidx}_g1"] = np.array(g1s, dtype=np.float32)
            win[f"w{gidx}_g2"] = np.array(g2s, dtype=np.float32)
            win[f"w{gidx}_sx"] = np.array(sxs)
            win[f"w{gidx}_sy"] = np.array(sys_)
            win[f"w{gidx}_meta"] = json.dumps({"n": n, "kr": kr})
            gidx += 1
    win["count"] = gidx
    np.savez_compressed(os.path.join(HERE, "ref_window_cases.npz"), **win)

    # -- interpcc2d --------------------------------------------------------
    it = {}
    irng = np.random.default_rng(99)
    icases = [(7, 9, -999999.0, 3), (5, 4, -999999.0, 2), (12, 10, 0.0, 4)]
    for q, (gx, gy, xm, skip) in enumerate(icases):
        fd = irng.standard_normal((gx, gy))
        holes = irng.random((gx, gy)) < 0.12
        fd[holes] = xm
        xo, yo = int(irng.integers(0, skip)), int(irng.integers(0, skip))
        nxo, nyo = gx * skip + 2, gy * skip + 1
        xw = (np.arange(nxo) - xo) / skip
        yw = (np.arange(nyo) - yo) / skip
        fdc = np.ascontiguousarray(fd)
        out = dp()
        L.interpcc2d(fdc.ctypes.data_as(dp), xm, gx, gy, np.ascontiguousarray(xw).ctypes.data_as(dp),
                     nxo, np.ascontiguousarray(yw).ctypes.data_as(dp), nyo, C.byref(out))
        res = np.ctypeslib.as_array(out, shape=(nxo * nyo,)).copy().reshape(nxo, nyo)
        libc.free(C.cast(out, C.c_void_p))
        it[f"i{q}_f"] = fd
        it[f"i{q}_xw"] = xw
        it[f"i{q}_yw"] = yw
        it[f"i{q}_xmiss"] = xm
        it[f"i{q}_out"] = res
    it["count"] = len(icases)
    np.savez_compressed(os.path.join(HERE, "ref_interp_cases.npz"), **it)

    # -- warp ----------------------------------------------------------------
    wr = {}
    img = f32(f1[:40, :60])
    ddx, ddy = f32(dx[:40, :60]), f32(dy[:40, :60])
    po.write_vc(os.path.join(tmp, "wi.dat"), img)
    po.write_vc(os.path.join(tmp, "ws.dat"), ddx, ddy)
    subprocess.run([os.path.join(po.REF_DIR, "warp"), os.path.join(tmp, "wi.dat"),
                    os.path.join(tmp, "ws.dat"), os.path.join(tmp, "wo.dat"), "-q"], check=True)
    wr["warp_img"] = img.astype(np.float32)
    wr["warp_dx"] = ddx.astype(np.float32)
    wr["warp_dy"] = ddy.astype(np.float32)
    wr["warp_out"] = po.read_vc(os.path.join(tmp, "wo.dat"), 1)[0].astype(np.float32)
    shx, shy = np.float32(0.37), np.float32(-1.3)
    po.write_vc(os.path.join(tmp, "ss.dat"), np.array([[shx]]), np.array([[shy]]))
    subprocess.run([os.path.join(po.REF_DIR, "warp"), os.path.join(tmp, "wi.dat"),
                    os.path.join(tmp, "ss.dat"), os.path.join(tmp, "so.dat"), "-q"], check=True)
    wr["shift_xy"] = np.array([shx, shy], dtype=np.float32)
    wr["shift_out"] = po.read_vc(os.path.join(tmp, "so.dat"), 1)[0].astype(np.float32)
    np.savez_compressed(os.path.join(HERE, "ref_warp_cases.npz"), **wr)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main(*sys.argv[1:])
