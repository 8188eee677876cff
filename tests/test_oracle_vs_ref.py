"""Live cross-check of the oracle restatement against the reference compiled
in place (oracle/_ref), on fresh random inputs.  Skipped where the reference
build is absent (it needs the reference sources)."""
import os
import tempfile

import numpy as np
import pytest

import pyoracle as po
from pyflct_gb300 import synth

pytestmark = pytest.mark.skipif(not po.ref_available(), reason="oracle/_ref not built")


@pytest.mark.parametrize("seed,args", [
    (1, [1, 1, 4, "-k", 0.4]),
    (2, [1, 1, 5, "-t", 0.4, "-s", "3p-1q1i"]),
    (3, [3, 2, 3, "-s", "2", "-t", "0.1a"]),
])
def test_random_vs_ref(seed, args):
    from _golden import parse_cli_args
    rng = np.random.default_rng(seed)
    f1 = synth.kfield((45, 50), rng).astype(np.float32).astype(np.float64)
    f2 = synth.fourier_shift(f1, *rng.uniform(-1, 1, 2)).astype(np.float32).astype(np.float64)
    r, ref = po.ref_flct(f1, f2, tempfile.mkdtemp(), args)
    assert r.returncode == 0
    got = po.velocity(f1, f2, nthreads=2, **parse_cli_args(args))
    for g, rr in zip(got, ref):
        assert np.array_equal(g.astype(np.float32).astype(np.float64), rr)
