"""The window-form autotuner: FLCT_FORM_AUTO times the candidate window
configurations (the FP32 radix form in both launch shapes -- windows per
CTA -- at full and half occupancy, and the split-FP16 tensor-core form) on
the first call's own work list, keeps the fastest per box size for the
context, and with FLCT_AUTOTUNE_CACHE set persists the choices to a JSON
file that later contexts on the same device load instead of measuring
again."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def gpu():
    from pyflct_gb300 import _lib, build
    build.build()
    return _lib.context(0)


def test_cache_file_round_trip(tmp_path, monkeypatch):
    from pyflct_gb300 import _lib, synth
    from pyflct_gb300.flct import make_params
    import ctypes as C
    path = tmp_path / "tune.json"
    monkeypatch.setenv("FLCT_AUTOTUNE_CACHE", str(path))
    rng = np.random.default_rng(5)
    f1 = synth.kfield((160, 150), rng)
    f2 = synth.fourier_shift(f1, 0.3, -0.4)
    out = [np.empty_like(f1) for _ in range(3)]
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    results = {}
    for sigma in (8.0, 5.0):
        ctx = _lib.Context(0)
        p = make_params(1.0, 1.0, sigma, form="auto")
        ctx.check(ctx.lib.flct_gpu_velocity(ctx.h, C.byref(p), dp(f1), dp(f2), *f1.shape, *[dp(o) for o in out]))
        results[sigma] = (ctx.timing().form, [o.copy() for o in out])
        ctx.close()
    data = json.loads(path.read_text())
    boxes = {e["box"]: e for e in data["entries"]}
    assert set(boxes) == {32, 20}
    assert boxes[20]["form"] == _lib.FORMS["fp32"]  # no tensor-core kernel for 20x20 boxes
    assert boxes[32]["form"] in (_lib.FORMS["fp32"], _lib.FORMS["tc_fp16"])
    assert all(e["ns_per_window"] > 0 and e["grid_div"] in (1, 2) and e["variant"] in (0, 1)
               for e in data["entries"])
    assert results[8.0][0] == boxes[32]["form"]
    # a new context loads the file: same choice, no new measurement needed
    mtime = os.path.getmtime(path)
    ctx = _lib.Context(0)
    p = make_params(1.0, 1.0, 8.0, form="auto")
    ctx.check(ctx.lib.flct_gpu_velocity(ctx.h, C.byref(p), dp(f1), dp(f2), *f1.shape, *[dp(o) for o in out]))
    assert ctx.timing().form == boxes[32]["form"]
    assert os.path.getmtime(path) == mtime
    for a, b in zip(out, results[8.0][1]):
        assert np.array_equal(a, b, equal_nan=True)
    ctx.close()


def test_auto_matches_the_chosen_form():
    """AUTO's output equals the output of the form it chose."""
    from pyflct_gb300 import _lib, synth
    from pyflct_gb300.flct import flct
    rng = np.random.default_rng(6)
    f1 = synth.kfield((200, 180), rng)
    f2 = synth.fourier_shift(f1, -0.6, 0.2)
    a = flct(f1, f2, 1, 1, 8, form="auto")
    chosen = _lib.context(0).timing().form
    name = {v: k for k, v in _lib.FORMS.items()}[chosen]
    b = flct(f1, f2, 1, 1, 8, form=name)
    for x, y in zip(a, b):
        assert np.array_equal(x, y, equal_nan=True)


@pytest.mark.parametrize("sigma", [1.0, 3.0, 5.0, 7.0, 8.0, 11.0, 12.0, 15.0])
def test_shape_variants_identical(tmp_path, monkeypatch, sigma):
    """Both launch shapes of the FP32 window kernel give identical fields:
    a cache file naming shape 1 for the box makes FLCT_FORM_AUTO use it,
    and its output must equal the explicit FP32 form's (shape 0)."""
    import ctypes as C
    import torch
    from pyflct_gb300 import _lib, synth
    from pyflct_gb300.flct import make_params
    n = 2 * (int(int(sigma) * np.sqrt(np.log(100.0))) // 2 * 2)  # flct.c:567-580
    path = tmp_path / "tune.json"
    entry = {"box": n, "form": _lib.FORMS["fp32"], "grid_div": 1, "ns_per_window": 1.0, "variant": 1}
    path.write_text('{"device": "%s", "entries": [\n  %s\n]}\n' % (torch.cuda.get_device_name(0), json.dumps(entry)))
    rng = np.random.default_rng(int(sigma * 7))
    f1 = synth.kfield((4 * n + 30, 4 * n + 22), rng)
    f2 = synth.fourier_shift(f1, 0.7, -0.45)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    outs = []
    for form, cache in (("auto", str(path)), ("fp32", "")):
        monkeypatch.setenv("FLCT_AUTOTUNE_CACHE", cache)
        ctx = _lib.Context(0)
        out = [np.empty_like(f1) for _ in range(3)]
        p = make_params(1.0, 1.0, sigma, skip="2i" if n >= 32 else None, form=form)
        ctx.check(ctx.lib.flct_gpu_velocity(ctx.h, C.byref(p), dp(f1), dp(f2), *f1.shape, *[dp(o) for o in out]))
        t = ctx.timing()
        assert t.form == _lib.FORMS["fp32"] and t.box == n
        outs.append(out)
        ctx.close()
    assert path.read_text().count('"variant": 1') == 1  # the choice was loaded, not re-measured
    for a, b in zip(*outs):
        assert np.array_equal(a, b, equal_nan=True)
