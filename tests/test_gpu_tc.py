"""GPU parity of the tensor-core window forms (DFT-matrix products on tcgen05
tensor cores with FP16 or BF16 hi+lo split operands) against the FP64 oracle.

Tolerances: the split-FP16 form is held to the same bar as the FP32 form
(max |dv| <= 1e-3 px/frame, bit-exact mask, integer peaks identical except at
documented ties).  The BF16 hi+lo form keeps ~16 significant bits per
operand; it is held to 1e-2 px and its measured error is reported.
"""
import numpy as np
import pytest

import pyoracle as po
from _compare import compare
from _golden import window_cases

pytestmark = pytest.mark.gpu
TOL = {"tc_fp16": 1e-3, "tc_bf16": 1e-2}


@pytest.fixture(scope="module", autouse=True)
def gpu():
    from pyflct_gb300 import _lib, build
    build.build()
    return _lib.context(0)


def run(f1, f2, form, **kw):
    from pyflct_gb300.flct import flct
    return flct(f1, f2, kw.pop("deltat", 1.0), kw.pop("deltas", 1.0), kw.pop("sigma"), form=form, **kw)


@pytest.mark.parametrize("form", ["tc_fp16", "tc_bf16"])
def test_golden_windows_n32(form):
    from pyflct_gb300.flct import cross_cor
    for n, kr, g1, g2, sx, sy in window_cases():
        if n != 32:
            continue
        gx, gy = cross_cor(g1, g2, kr=kr, form=form)
        assert np.abs(gx - sx).max() <= TOL[form], (kr, np.abs(gx - sx).max())
        assert np.abs(gy - sy).max() <= TOL[form]


@pytest.mark.parametrize("form", ["tc_fp16", "tc_bf16"])
@pytest.mark.parametrize("seed,shape,extra", [
    (1, (96, 100), {}), (2, (128, 80), {"kr": 0.5}), (3, (140, 150), {"skip": "3p1q2i"}),
    (4, (100, 104), {"thresh": 0.3}), (5, (90, 96), {"hires": True}),
])
def test_random_fields_sigma8(form, seed, shape, extra):
    from pyflct_gb300 import synth
    from _golden import parse_cli_args
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


@pytest.mark.parametrize("form", ["tc_fp16", "tc_bf16"])
def test_config3_full_size(form):
    from pyflct_gb300 import synth
    rng = np.random.default_rng(20263)
    f1 = synth.kfield((1024, 1024), rng)
    f2 = synth.spline_warp(f1, *synth.vortex_shift(f1.shape, rng))
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
    f2 = synth.spline_warp(f1, *synth.rotation_shift(f1.shape, 0.01))
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
    with pytest.raises(FlctError) as e:
        run(a, a, "tc_fp16", sigma=4.0)
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
