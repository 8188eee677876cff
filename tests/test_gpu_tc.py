"""GPU parity of the tensor-core window forms (DFT-matrix products on tcgen05
tensor cores with FP16 or BF16 hi+lo split operands) against the FP64 oracle,
at every box size the library compiles (n = 4..64, multiples of 4).

Tolerances: the split-FP16 form is held to the same bar as the FP32 form
(max |dv| <= 1e-3 px/frame, bit-exact mask, integer peaks identical except at
documented ties).  The BF16 hi+lo form keeps ~16 significant bits per
operand; it is held to 1e-2 px and its measured error is reported.  The
every-box and every-sigma cases run the FP32 form too (its radix-4/2/3/5
and odd-prime register transforms differ by box size).
"""
import numpy as np
import pytest

import pyoracle as po
from _compare import TIE_REL, compare
from _golden import parse_cli_args, window_cases

pytestmark = pytest.mark.gpu
TOL = {"fp32": 1e-3, "tc_fp16": 1e-3, "tc_bf16": 1e-2}
BOXES = list(range(4, 68, 4))
# sigma -> box side through flct.c:567-580 (frames large enough not to shrink it)
SIGMA_BOX = {1: 4, 2: 8, 3: 12, 4: 16, 5: 20, 6: 24, 7: 28, 8: 32, 9: 36, 10: 40, 11: 44, 12: 48,
             13: 52, 14: 60, 15: 64}


@pytest.fixture(scope="module", autouse=True)
def gpu():
    from pyflct_gb300 import _lib, build
    build.build()
    return _lib.context(0)


def run(f1, f2, form, **kw):
    from pyflct_gb300.flct import flct
    return flct(f1, f2, kw.pop("deltat", 1.0), kw.pop("deltas", 1.0), kw.pop("sigma"), form=form, **kw)


def window_stack(rng, n, count):
    """`count` pairs of n x n windows cut from shifted k^-2 fields."""
    from pyflct_gb300 import synth
    g1 = np.empty((count, n, n))
    g2 = np.empty((count, n, n))
    for k in range(count):
        f = synth.kfield((n + 8, n + 8), rng)
        s = synth.fourier_shift(f, *rng.uniform(-1.5, 1.5, 2))
        g1[k], g2[k] = f[4:4 + n, 4:4 + n], s[4:4 + n, 4:4 + n]
    return g1, g2


def check_windows(g1, g2, kr, form, gx, gy, ox, oy):
    """Shifts within TOL of the oracle's; a window beyond it must be an
    argmax tie (another FP64 |c| within TIE_REL of the maximum next to the
    GPU's integer peak).  Returns the max |d| over the other windows."""
    n = g1.shape[1]
    d = np.maximum(np.abs(gx - ox), np.abs(gy - oy))
    for k in np.nonzero(d > TOL[form])[0]:
        _, _, ab = po.cross_cor(g1[k], g2[k], kr=kr, want_abs=True)
        I = int(np.floor(gx[k] + n // 2 + 0.5))  # shiftx: slow axis
        J = int(np.floor(gy[k] + n // 2 + 0.5))
        m = ab.max()
        near = any(0 <= I + a < n and 0 <= J + b < n and ab[I + a, J + b] >= (1 - TIE_REL) * m
                   for a in (-1, 0, 1) for b in (-1, 0, 1))
        assert near, (n, kr, form, int(k), float(d[k]))
    return float(d[d <= TOL[form]].max(initial=0.0))


@pytest.mark.parametrize("form", ["tc_fp16", "tc_bf16"])
def test_golden_windows(form):
    """The reference's own per-window shifts (cross_cor of the compiled
    reference) at box sizes 12, 20, 32 and 48."""
    from pyflct_gb300.flct import cross_cor
    seen = set()
    for n, kr, g1, g2, sx, sy in window_cases():
        gx, gy = cross_cor(g1, g2, kr=kr, form=form)
        assert np.abs(gx - sx).max() <= TOL[form], (n, kr, np.abs(gx - sx).max())
        assert np.abs(gy - sy).max() <= TOL[form], (n, kr, np.abs(gy - sy).max())
        seen.add(n)
    assert {12, 20, 32, 48} <= seen


@pytest.mark.parametrize("form", ["fp32", "tc_fp16", "tc_bf16"])
@pytest.mark.parametrize("n", BOXES)
def test_direct_windows_every_box(form, n):
    """Random windows at every box size, with and without the -k filter."""
    from pyflct_gb300.flct import cross_cor
    rng = np.random.default_rng(1000 + n)
    g1, g2 = window_stack(rng, n, 40)
    for kr in (None, 0.5):
        ox, oy = po.cross_cor_batch(g1, g2, kr=kr)
        gx, gy = cross_cor(g1, g2, kr=kr, form=form)
        worst = check_windows(g1, g2, kr, form, gx, gy, ox, oy)
        print(form, n, kr, f"max|d| {worst:.2e}")


@pytest.mark.parametrize("sigma,shape,extra", [
    (1.0, (40, 44), {}), (2.0, (50, 46), {"kr": 0.4}), (3.0, (60, 64), {"skip": "2i"}),
    (4.0, (70, 66), {"hires": True}), (5.0, (72, 80), {"thresh": 0.3}), (6.0, (84, 90), {}),
    (7.0, (96, 92), {"kr": 0.6, "skip": "3p1q2i"}), (9.0, (120, 112), {}),
    (10.0, (130, 128), {"hires": True}), (11.0, (140, 150), {"skip": "2"}),
    (12.0, (150, 160), {"kr": 0.5}), (13.0, (170, 162), {"skip": "3i"}),
    (14.0, (190, 184), {"skip": "2i"}), (15.0, (200, 204), {"skip": "2i", "kr": 0.5}),
])
def test_random_fields_every_sigma(sigma, shape, extra):
    """Whole velocity fields at every box size the sigmas reach, with the
    options (-k, -s, -t, -h) spread over them, split FP16 and BF16."""
    from pyflct_gb300 import synth
    rng = np.random.default_rng(int(sigma * 10))
    f1 = synth.kfield(shape, rng)
    f2 = synth.fourier_shift(f1, *rng.uniform(-1.5, 1.5, 2))
    args = [1, 1, sigma]
    for k, v in extra.items():
        args += {"kr": ["-k", v], "skip": ["-s", v], "thresh": ["-t", v], "hires": ["-h"]}[k]
    kw = parse_cli_args(args)
    assert 2 * po.derive(f1, f2, **kw).nsize == SIGMA_BOX[int(sigma)]
    ref = po.velocity(f1, f2, **kw)
    for form in ("fp32", "tc_fp16", "tc_bf16"):
        rep = compare(f1, f2, run(f1, f2, form, sigma=sigma, **extra), ref, kw, tol=TOL[form])
        print(form, sigma, extra, rep)


@pytest.mark.parametrize("form", ["tc_fp16", "tc_bf16"])
@pytest.mark.parametrize("seed,shape,extra", [
    (1, (96, 100), {}), (2, (128, 80), {"kr": 0.5}), (3, (140, 150), {"skip": "3p1q2i"}),
    (4, (100, 104), {"thresh": 0.3}), (5, (90, 96), {"hires": True}),
])
def test_random_fields_sigma8(form, seed, shape, extra):
    from pyflct_gb300 import synth
    rng = np.random.default_rng(seed)
    f1 = synth.kfield(shape, rng)
    f2 = synth.fourier_shift(f1, *rng.uniform(-1.5, 1.5, 2))
    got = run(f1, f2, form, sigma=8.0, **extra)
    args = [1, 1, 8]
    for k, v in extra.items():
        args += {"kr": ["-k", v], "skip": ["-s", v], "thresh": ["-t", v], "hires": ["-h"]}[k]
    kw = parse_cli_args(args)
    rep = compare(f1, f2, got, po.velocity(f1, f2, **kw), kw, tol=TOL[form])
    print(form, shape, extra, rep)


@pytest.mark.parametrize("offset", [1e4, -3e7, 2e-9])
def test_large_offsets_tensor_core(offset):
    """Frames on a large (or tiny) constant offset: the window values are
    formed in FP32 from the exact means before the 16-bit split."""
    from pyflct_gb300 import synth
    rng = np.random.default_rng(int(abs(offset)) % 1000 + 5)
    f1 = synth.kfield((96, 104), rng)
    f2 = synth.fourier_shift(f1, 0.6, -0.4)
    scale = abs(offset) if abs(offset) < 1 else 1.0
    a, b = f1 * scale + offset, f2 * scale + offset
    for kw in (dict(sigma=5), dict(sigma=4, skip=3, interpolate=True)):
        args = {"sigma": kw["sigma"]}
        if "skip" in kw:
            args["skip"] = "3i"
        rep = compare(a, b, run(a, b, "tc_fp16", **args), po.velocity(a, b, **kw), kw)
        print(offset, kw, rep)


def test_nonfinite_inputs_tensor_core():
    """NaN and infinities in the frames, through the split-FP16 form: the
    windows holding them give what the oracle gives."""
    from pyflct_gb300 import synth
    rng = np.random.default_rng(11)
    f1 = synth.kfield((90, 100), rng)
    f2 = synth.fourier_shift(f1, 0.3, 0.5)
    f1[10, 12] = np.nan
    f2[60, 70] = np.inf
    f1[70, 20] = -np.inf
    f2[30, 80] = np.inf
    f2[32, 84] = -np.inf
    kw = dict(sigma=3)
    rep = compare(f1, f2, run(f1, f2, "tc_fp16", sigma=3.0), po.velocity(f1, f2, **kw), kw)
    print(rep)


@pytest.mark.parametrize("form", ["tc_fp16", "tc_bf16"])
def test_config3_full_size(form):
    from pyflct_gb300 import synth
    rng = np.random.default_rng(20263)
    f1 = synth.kfield((1024, 1024), rng)
    f2 = synth.spectral_warp(f1, *synth.vortex_shift(f1.shape, rng))
    kw = dict(sigma=8, skip=4, interpolate=True)
    got = run(f1, f2, form, sigma=8.0, skip="4i")
    rep = compare(f1, f2, got, po.velocity(f1, f2, **kw), kw, tol=TOL[form])
    print(form, rep)


def test_precision_study_config2():
    """512^2, sigma 8, -t 0.1a -k 0.5: FP32, split-FP16 and BF16 hi+lo side by
    side against the FP64 oracle."""
    from pyflct_gb300 import synth
    rng = np.random.default_rng(20262)
    f1 = synth.config2_image1(rng)
    f2 = synth.spectral_warp(f1, *synth.rotation_shift(f1.shape, 0.01))
    kw = dict(sigma=8, thresh=0.1, thresh_abs=True, kr=0.5)
    ref = po.velocity(f1, f2, **kw)
    for form, tol in (("fp32", 1e-3), ("tc_fp16", 1e-3), ("tc_bf16", 1e-2)):
        got = run(f1, f2, form, sigma=8.0, thresh="0.1a", kr=0.5)
        rep = compare(f1, f2, got, ref, kw, tol=tol)
        print("precision", form, rep)


def test_auto_form_and_unsupported_box():
    from pyflct_gb300 import _lib
    from pyflct_gb300.flct import FlctError
    rng = np.random.default_rng(9)
    a = rng.standard_normal((60, 60))
    got = run(a, a, "auto", sigma=8.0)
    # the autotuner measured the candidates on this call's work list and
    # chose one of the FP32-accurate forms
    assert _lib.context(0).timing().form in (_lib.FORMS["fp32"], _lib.FORMS["tc_fp16"])
    assert np.all(got[2] == 1)
    # boxes above 64 have no tensor-core kernel (the FP32 big-box kernel serves them)
    big = rng.standard_normal((220, 220))
    with pytest.raises(FlctError) as e:
        run(big, big, "tc_fp16", sigma=16.0)
    assert e.value.code == _lib.ERR_UNSUPPORTED


def test_stage_wait_timeout_reports_and_context_survives(monkeypatch):
    """Failure detection without a GPU fault: the test hook makes the
    tensor-core kernel's first stage wait on a barrier that nothing completes,
    with a 1 ms limit; the wait runs out, the kernel lets its own MMAs finish
    (bounded exit wait), frees its TMEM and returns, the call reports
    FLCT_ERR_TIMEOUT, and the context computes correctly afterwards."""
    from pyflct_gb300 import _lib, synth
    from pyflct_gb300.flct import FlctError
    rng = np.random.default_rng(21)
    f1 = synth.kfield((96, 96), rng)
    f2 = synth.fourier_shift(f1, 0.5, -0.25)
    monkeypatch.setenv("FLCT_TEST_TC_STALL_NS", "1000000")
    with pytest.raises(FlctError) as e:
        run(f1, f2, "tc_fp16", sigma=8.0)
    assert e.value.code == _lib.ERR_TIMEOUT
    monkeypatch.delenv("FLCT_TEST_TC_STALL_NS")
    got = run(f1, f2, "tc_fp16", sigma=8.0)
    compare(f1, f2, got, po.velocity(f1, f2, sigma=8), dict(sigma=8), tol=TOL["tc_fp16"])
