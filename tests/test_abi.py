"""CPU-side checks of the product's C ABI and host logic (no GPU calls)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from pyflct_gb300 import _lib
from pyflct_gb300.flct import make_params, parse_skip, parse_thresh

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(flct_gpu_\w+)\s*\(", txt))
    return names


@pytest.fixture(scope="module")
def lib():
    from pyflct_gb300 import build
    build.build()
    return _lib.load()


def test_library_exports_every_declared_symbol(lib):
    declared = _declared_symbols()
    assert len(declared) >= 14
    for name in declared:
        assert hasattr(lib, name), name
    # and the Python binding knows each one
    assert declared <= set(_lib.SIGNATURES), declared - set(_lib.SIGNATURES)


def test_status_strings(lib):
    for code in range(13):
        s = lib.flct_gpu_status_string(code)
        assert s and s.decode() != "unknown status"
    assert lib.flct_gpu_version().decode().endswith("sm_103a")


def test_output_len(lib):
    p = make_params(1, 1, 4)
    assert lib.flct_gpu_output_len(C.byref(p), 10, 20) == 200
    p = make_params(1, 1, 0)
    assert lib.flct_gpu_output_len(C.byref(p), 10, 20) == 1


def test_no_cpu_fallback_without_gpu(lib):
    try:
        import torch
        has = torch.cuda.is_available()
    except Exception:
        has = False
    if has:
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert lib.flct_gpu_create(0, C.byref(h)) == _lib.ERR_NO_DEVICE
    with pytest.raises(_lib.FlctError):
        _lib.Context(0)


def test_null_context_is_an_error(lib):
    p = make_params(1, 1, 4)
    a = np.zeros((8, 8))
    dp = a.ctypes.data_as(C.POINTER(C.c_double))
    assert lib.flct_gpu_velocity(None, C.byref(p), dp, dp, 8, 8, dp, dp, dp) == _lib.ERR_ARG


@pytest.mark.parametrize("s,exp", [
    ("4", (4, 0, 0, False)), ("4i", (4, 0, 0, True)), ("10p5q5", (10, 5, 5, False)),
    ("5p-2q3i", (5, -2, 3, True)), ("3q-1", (3, 0, -1, False)), ("0", (-1, 0, 0, False)),
    (None, (0, 0, 0, False)), (7, (7, 0, 0, False)),
])
def test_parse_skip(s, exp):
    assert parse_skip(s) == exp


@pytest.mark.parametrize("s,exp", [("0.1", (0.1, False)), ("0.1a", (0.1, True)), (5, (5.0, False)),
                                   ("2.5a", (2.5, True)), (None, (0.0, False))])
def test_parse_thresh(s, exp):
    assert parse_thresh(s) == exp
