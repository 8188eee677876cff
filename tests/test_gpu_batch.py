"""GPU batched velocity (flct_gpu_velocity_batch): a heterogeneous list of
frame pairs (uneven sizes, sigmas, thresholds, -k and -s) runs as one
captured CUDA graph with one persistent window launch per box size.

The batch uses the same kernels and arithmetic per window as the single-pair
call, so its outputs must equal the single-pair outputs bit for bit; those
are parity-tested against the FP64 oracle elsewhere, and a subset of pairs is
compared with the oracle here too (max |dv| <= 1e-3 px/frame, bit-exact mask).
"""
import numpy as np
import pytest

import pyoracle as po
from _compare import compare

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def gpu():
    from pyflct_gb300 import build
    build.build()
    from pyflct_gb300 import _lib
    return _lib.context(0)


# (shape, flct keyword arguments, the oracle's keyword arguments)
SPECS = [
    ((96, 80), dict(sigma=3), dict(sigma=3)),
    ((64, 130), dict(sigma=5, kr=0.25), dict(sigma=5, kr=0.25)),
    ((128, 128), dict(sigma=8), dict(sigma=8)),
    ((100, 72), dict(sigma=8), dict(sigma=8)),
    ((150, 140), dict(sigma=12, thresh=0.3), dict(sigma=12, thresh=0.3)),
    ((80, 84), dict(sigma=4, skip="3p2q-1i"),
     dict(sigma=4, skip=3, poffset=2, qoffset=-1, interpolate=True)),
    ((90, 90), dict(sigma=6, skip="5i", thresh="0.4a"),
     dict(sigma=6, skip=5, interpolate=True, thresh=0.4, thresh_abs=True)),
    ((70, 96), dict(sigma=5), dict(sigma=5)),
    ((128, 100), dict(sigma=8, kr=0.5), dict(sigma=8, kr=0.5)),
    ((80, 76), dict(sigma=5, hires=True), dict(sigma=5, hires=True)),
]


def frames_for(specs, seed):
    from pyflct_gb300 import synth
    rng = np.random.default_rng(seed)
    out = []
    for shape, _, _ in specs:
        f1 = synth.kfield(shape, rng)
        out.append((f1, synth.fourier_shift(f1, *rng.uniform(-1, 1, 2))))
    return out


def run_batch(specs, frames, form):
    import torch
    from pyflct_gb300.flct import FlctBatch, make_params
    params = [make_params(1.0, 1.0, form=form, **kw) for _, kw, _ in specs]
    b = FlctBatch([s for s, _, _ in specs], params)
    b.load(frames)
    b.run()
    torch.cuda.synchronize()
    return b


def outputs(b, k):
    return tuple(t[k].cpu().numpy() for t in (b.vx, b.vy, b.vm))


def single(f1, f2, kw, form):
    """One pair through the one-shot device entry point (the batch runs the
    same whole-frame passes, so the outputs must agree bit for bit; the
    host-buffer entry point pipelines large frames in row bands, whose FP64
    box sums round differently in the last bits)."""
    import ctypes as C
    import torch
    from pyflct_gb300 import _lib
    from pyflct_gb300.flct import make_params
    ctx = _lib.context(0)
    p = make_params(1.0, 1.0, form=form, **kw)
    dev = torch.device("cuda", 0)
    d1, d2 = torch.from_numpy(np.ascontiguousarray(f1)).to(dev), torch.from_numpy(np.ascontiguousarray(f2)).to(dev)
    out = [torch.empty(f1.shape, dtype=torch.float64, device=dev) for _ in range(3)]
    ctx.check(ctx.lib.flct_gpu_velocity_device(ctx.h, C.byref(p), C.c_void_p(d1.data_ptr()),
                                               C.c_void_p(d2.data_ptr()), f1.shape[0], f1.shape[1],
                                               *[C.c_void_p(o.data_ptr()) for o in out], None))
    ctx.timing()
    return tuple(o.cpu().numpy() for o in out)


@pytest.mark.parametrize("form", ["fp32", "auto"])
def test_batch_equals_single_pairs(form):
    frames = frames_for(SPECS, 11)
    b = run_batch(SPECS, frames, form)
    total = 0
    for k, ((f1, f2), (_, kw, _)) in enumerate(zip(frames, SPECS)):
        want = single(f1, f2, kw, form)
        got = outputs(b, k)
        for name, x, y in zip(("vx", "vy", "vm"), got, want):
            assert np.array_equal(x, y, equal_nan=True), (k, name)
        total += int((want[2] == 1).sum())
    t = b.timing()
    # one window per computed pixel (mask 1); interpolated pixels are not windows
    assert t.windows == total
    # at most 11 merged kernels (counters, thresholds, classification, box
    # sums, means, prefix sums, fits, interpolation) plus one window launch
    # per group of pairs sharing box size, form and tables (9 groups here)
    assert t.launches <= 11 + 9, t.launches


def test_batch_tensor_core_form_equals_single():
    specs = list(SPECS)
    frames = frames_for(specs, 12)
    b = run_batch(specs, frames, "tc_fp16")
    for k, ((f1, f2), (_, kw, _)) in enumerate(zip(frames, specs)):
        want = single(f1, f2, kw, "tc_fp16")
        for x, y in zip(outputs(b, k), want):
            assert np.array_equal(x, y, equal_nan=True), k


def test_batch_against_oracle():
    frames = frames_for(SPECS, 13)
    b = run_batch(SPECS, frames, "auto")
    for k, ((f1, f2), (_, _, okw)) in enumerate(zip(frames, SPECS)):
        rep = compare(f1, f2, outputs(b, k), po.velocity(f1, f2, **okw), okw)
        print(k, okw, rep)


def test_graph_replay_sees_new_inputs():
    """Same pair list (same device pointers): the captured graph is replayed
    and must pick up the new frame contents."""
    import torch
    frames = frames_for(SPECS, 14)
    b = run_batch(SPECS, frames, "fp32")
    first = [outputs(b, k) for k in range(len(SPECS))]
    frames2 = frames_for(SPECS, 15)
    b.load(frames2)
    b.run()
    torch.cuda.synchronize()
    for k, ((f1, f2), (_, kw, _)) in enumerate(zip(frames2, SPECS)):
        want = single(f1, f2, kw, "fp32")
        got = outputs(b, k)
        for x, y in zip(got, want):
            assert np.array_equal(x, y, equal_nan=True), k
    assert any(not np.array_equal(first[k][0], outputs(b, k)[0]) for k in range(len(SPECS)))
    # and a third run on the first frames reproduces the first outputs
    b.load(frames)
    b.run()
    torch.cuda.synchronize()
    for k in range(len(SPECS)):
        for x, y in zip(outputs(b, k), first[k]):
            assert np.array_equal(x, y, equal_nan=True), k


def test_batch_errors_and_empty():
    from pyflct_gb300 import _lib
    from pyflct_gb300.flct import FlctBatch, FlctError, make_params
    good = make_params(1.0, 1.0, 4)
    bad = make_params(1.0, 1.0, 4, skip="0")
    b = FlctBatch([(40, 40), (40, 40)], [good, bad])
    with pytest.raises(FlctError) as e:
        b.run()
    assert e.value.code == _lib.ERR_SKIP_NONPOSITIVE
    assert "pair 1" in e.value.message
    # a box above 64 (sigma 16) has no tensor-core kernel
    big = FlctBatch([(220, 220)], [make_params(1.0, 1.0, 16, form="tc_fp16")])
    with pytest.raises(FlctError) as e:
        big.run()
    assert e.value.code == _lib.ERR_UNSUPPORTED
    empty = FlctBatch([], [])
    empty.run()
    ctx = _lib.context(0)
    assert ctx.lib.flct_gpu_velocity_batch(ctx.h, -1, None, None) == _lib.ERR_ARG


def test_config4_batch_64_pairs():
    """The 64-pair heterogeneous workload (sides 128..768, sigma 3/5/8/12):
    batch equals single-pair calls everywhere; a few pairs against the
    oracle, one per sigma."""
    import torch
    from pyflct_gb300 import synth
    from pyflct_gb300.flct import FlctBatch, make_params
    pairs = synth.config4_pairs()
    params = [make_params(1.0, 1.0, kw["sigma"], form="auto") for _, _, kw, _ in pairs]
    b = FlctBatch([f1.shape for f1, _, _, _ in pairs], params)
    b.load([(f1, f2) for f1, f2, _, _ in pairs])
    b.run()
    torch.cuda.synchronize()
    t = b.timing()
    assert t.windows == sum(f1.size for f1, _, _, _ in pairs)  # thresh 0, no skip
    # every pair's prepass, fit and interpolation run as merged launches:
    # a few kernels for the whole batch, one window launch per box size
    assert t.launches <= 16, t.launches
    seen = set()
    for k, (f1, f2, kw, _) in enumerate(pairs):
        got = outputs(b, k)
        want = single(f1, f2, dict(sigma=kw["sigma"]), "auto")
        for x, y in zip(got, want):
            assert np.array_equal(x, y, equal_nan=True), k
        if kw["sigma"] not in seen and f1.size <= 256 * 384:
            seen.add(kw["sigma"])
            okw = dict(sigma=kw["sigma"])
            rep = compare(f1, f2, got, po.velocity(f1, f2, **okw), okw)
            print("pair", k, f1.shape, okw, rep)
