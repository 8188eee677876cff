"""GPU parity of the warp program's transforms (shift_frac2d, warp_frac2d)
against the FP64 oracle and the reference's golden outputs.

The GPU evaluates the transforms in FP32 with FP64 phase bases and FP64
circulant/twiddle tables; warp_frac2d's spectral sum runs on the tensor
cores (split FP16) by default, or as FP32 on the CUDA cores with
FLCT_WARP_SUM=fp32; power-of-two axes take warp_frac2d's spectrum by FFTs.
Tolerances, relative to max |image|: warp_frac2d 1e-6 (measured up to
6.5e-7 over the test shapes with the tensor-core sum), shift_frac2d 4e-6
(measured up to 1.9e-6 at 512^2); against the reference's golden files,
which are float32-rounded, 2e-6.
"""
import numpy as np
import pytest

import pyoracle as po
from _golden import load

pytestmark = pytest.mark.gpu
REL = 2e-6        # against the float32-rounded golden files
REL_WARP = 1e-6
REL_SHIFT = 4e-6


@pytest.fixture(scope="module", autouse=True)
def gpu():
    from pyflct_gb300 import _lib, build
    build.build()
    return _lib.context(0)


def close(a, b, scale, rel=REL):
    err = np.abs(a - b).max() / scale
    print(f"max |d| / max |image| = {err:.3e} (bound {rel:.1e})")
    return err <= rel


def test_golden_warp_and_shift():
    from pyflct_gb300.flct import shift_frac2d, warp_frac2d
    z = load("ref_warp_cases.npz")
    img = z["warp_img"].astype(np.float64)
    s = np.abs(img).max()
    out = warp_frac2d(img, z["warp_dx"].astype(np.float64), z["warp_dy"].astype(np.float64))
    assert close(out, z["warp_out"].astype(np.float64), s)
    sx, sy = (float(v) for v in z["shift_xy"])
    out = shift_frac2d(img, sx, sy)
    assert close(out, z["shift_out"].astype(np.float64), s)


@pytest.mark.parametrize("shape", [(37, 53), (64, 48), (101, 201), (16, 16), (5, 7)])
@pytest.mark.parametrize("transp", [1, 0])
def test_shift_sizes(shape, transp):
    from pyflct_gb300.flct import shift_frac2d
    rng = np.random.default_rng(shape[0] * 1000 + shape[1] + transp)
    img = rng.standard_normal(shape) + 3.0
    dx, dy = rng.uniform(-6, 6, 2)
    got = shift_frac2d(img, dx, dy, transp)
    ref = po.shift_frac2d(img, dx, dy, transp)
    assert close(got, ref, np.abs(img).max(), REL_SHIFT)


@pytest.mark.parametrize("shape", [(64, 128), (256, 64), (1024, 512), (2048, 2048)])
@pytest.mark.parametrize("transp", [1, 0])
def test_shift_power_of_two_transform(shape, transp):
    """Power-of-two axes take the transform path (forward FFT, phase
    factors, inverse FFT per line); the oracle follows the reference's own
    2-D FFT."""
    from pyflct_gb300.flct import shift_frac2d
    rng = np.random.default_rng(shape[0] * 31 + shape[1] + transp)
    img = rng.standard_normal(shape) + 3.0
    dx, dy = rng.uniform(-40, 40, 2)
    got = shift_frac2d(img, dx, dy, transp)
    ref = po.shift_frac2d(img, dx, dy, transp)
    assert close(got, ref, np.abs(img).max(), REL_SHIFT)


@pytest.mark.parametrize("shape", [(37, 53), (64, 48), (20, 31), (9, 8)])
@pytest.mark.parametrize("transp", [1, 0])
def test_warp_sizes(shape, transp):
    from pyflct_gb300 import synth
    from pyflct_gb300.flct import warp_frac2d
    rng = np.random.default_rng(shape[0] * 77 + shape[1] + transp)
    img = synth.kfield(shape, rng)
    dfast, dslow = synth.smooth_shift(shape, rng, rms=1.5)
    got = warp_frac2d(img, dfast, dslow, transp)
    ref = po.warp_frac2d(img, dfast, dslow, transp)
    assert close(got, ref, np.abs(img).max(), REL_WARP)


@pytest.mark.parametrize("shape", [(300, 130), (129, 257), (130, 33), (128, 256), (64, 64), (2, 2), (1, 4), (4, 1), (3, 5)])
@pytest.mark.parametrize("form", ["tc", "fp32"])
def test_warp_sum_forms(shape, form, monkeypatch):
    """Both spectral-sum kernels against the oracle: the tensor-core form
    (half spectrum, split FP16) over several 128-row chunks and stage-ring
    wraps, odd and even axes (Nyquist row and column), degenerate axes; the
    FP32 CUDA-core form (FLCT_WARP_SUM=fp32) on the same inputs.  Power-of-
    two shapes take the spectrum by FFTs, the others by DFT matrices."""
    if form == "fp32":
        monkeypatch.setenv("FLCT_WARP_SUM", "fp32")
    else:
        monkeypatch.delenv("FLCT_WARP_SUM", raising=False)
    from pyflct_gb300 import synth
    from pyflct_gb300.flct import warp_frac2d
    rng = np.random.default_rng(shape[0] * 131 + shape[1])
    if min(shape) >= 8:
        img = synth.kfield(shape, rng)
        dfast, dslow = synth.smooth_shift(shape, rng, rms=1.5)
    else:
        img = rng.standard_normal(shape) + 2.0
        dfast, dslow = rng.uniform(-2, 2, shape), rng.uniform(-2, 2, shape)
    for transp in (1, 0):
        got = warp_frac2d(img, dfast, dslow, transp)
        ref = po.warp_frac2d(img, dfast, dslow, transp)
        assert close(got, ref, np.abs(img).max(), REL_WARP)


def test_warp_sum_wait_timeout_reports_and_context_survives(monkeypatch):
    """Failure detection without a GPU fault: the test hook makes the warp
    sum's MMA thread wait first on a barrier that nothing completes, with a
    1 ms limit; the CTA aborts every role's waits, drains its own copies,
    frees its TMEM and returns, the call reports FLCT_ERR_TIMEOUT, and the
    same context then computes the warp correctly."""
    from pyflct_gb300 import _lib, synth
    from pyflct_gb300.flct import FlctError, warp_frac2d
    monkeypatch.delenv("FLCT_WARP_SUM", raising=False)
    rng = np.random.default_rng(33)
    img = synth.kfield((64, 48), rng)
    dfast, dslow = synth.smooth_shift(img.shape, rng, rms=1.0)
    monkeypatch.setenv("FLCT_TEST_WARP_STALL_NS", "1000000")
    with pytest.raises(FlctError) as e:
        warp_frac2d(img, dfast, dslow)
    assert e.value.code == _lib.ERR_TIMEOUT
    monkeypatch.delenv("FLCT_TEST_WARP_STALL_NS")
    got = warp_frac2d(img, dfast, dslow)
    assert close(got, po.warp_frac2d(img, dfast, dslow), np.abs(img).max(), REL_WARP)


def test_warp_dispatch_and_constant_field():
    from pyflct_gb300.flct import FlctError, warp
    rng = np.random.default_rng(4)
    img = rng.standard_normal((24, 30))
    a = warp(img, np.full(img.shape, 0.7), np.full(img.shape, -1.2))
    b = warp(img, 0.7, -1.2)
    assert np.abs(a - b).max() <= REL_SHIFT * np.abs(img).max()
    with pytest.raises(FlctError) as e:
        warp(img, np.zeros((3, 3)), np.zeros((3, 3)))
    assert e.value.code == 11


def test_warp_crop_256_and_shift_512():
    """A 256^2 crop through the non-uniform warp and a 512^2 uniform shift."""
    from pyflct_gb300 import synth
    from pyflct_gb300.flct import shift_frac2d, warp_frac2d
    rng = np.random.default_rng(20265)
    img = synth.kfield((512, 512), rng)
    got = shift_frac2d(img, 0.37, -2.6)
    assert close(got, po.shift_frac2d(img, 0.37, -2.6), np.abs(img).max(), REL_SHIFT)
    crop = img[100:356, 40:296]
    dfast, dslow = synth.smooth_shift(crop.shape, rng, rms=0.3)
    got = warp_frac2d(crop, dfast, dslow)
    assert close(got, po.warp_frac2d(crop, dfast, dslow), np.abs(crop).max(), REL_WARP)
