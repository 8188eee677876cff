"""GPU test of flct_gpu_interpcc2d_noalloc, the entry point for callers that
cannot allocate device memory (programs whose own pool or fixed budget owns
all GPU memory).  It must give what the allocating flct_gpu_interpcc2d gives,
call after call, although every call reuses one fixed scratch array inside
the library.

This file sorts last so that, if it fails, a run stopping at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

XMISS = -999999.0


def _case(rng, gx, gy, nxi, nyi):
    f = rng.standard_normal((gx, gy))
    f[rng.random(f.shape) < 0.1] = XMISS
    xw = np.sort(rng.uniform(-0.7, gx - 0.3, nxi))
    yw = np.sort(rng.uniform(-0.7, gy - 0.3, nyi))
    return f, xw, yw


def test_noalloc_matches_allocating_entry_point():
    import torch
    from pyflct_gb300 import _lib, build
    from pyflct_gb300.flct import interpcc2d

    build.build()
    lib = _lib.load()
    _lib.context(0)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(20261203)

    def ptr(t):
        return C.c_void_p(t.data_ptr())

    # two calls in a row with different sizes and data: the second must not
    # see anything the first left in the shared scratch array
    for gx, gy, nxi, nyi in ((9, 7, 61, 40), (14, 11, 37, 90)):
        f, xw, yw = _case(rng, gx, gy, nxi, nyi)
        want = interpcc2d(f, XMISS, xw, yw)  # the allocating entry point
        d_f = torch.from_numpy(f).to(dev)
        d_x = torch.from_numpy(xw).to(dev)
        d_y = torch.from_numpy(yw).to(dev)
        d_o = torch.full((nxi, nyi), np.nan, dtype=torch.float64, device=dev)
        rc = lib.flct_gpu_interpcc2d_noalloc(ptr(d_f), XMISS, gx, gy, ptr(d_x), nxi, ptr(d_y), nyi,
                                             ptr(d_o), None)
        torch.cuda.synchronize()
        assert rc == _lib.OK
        got = d_o.cpu().numpy()
        # same kernels and operation order as the allocating entry point: the
        # tolerance of the interpolation tests is exact equality
        assert np.array_equal(got, want)

    # the largest accepted axes fill the fixed array to its end (each axis
    # at FLCT_NOALLOC_MAX_AXIS once), and a call on a non-default stream
    side = torch.cuda.Stream(device=dev)
    for gx, gy, nxi, nyi, st in ((12, 9, 16384, 3, None), (8, 13, 5, 16384, side)):
        f, xw, yw = _case(rng, gx, gy, nxi, nyi)
        want = interpcc2d(f, XMISS, xw, yw)
        d_f = torch.from_numpy(f).to(dev)
        d_x = torch.from_numpy(xw).to(dev)
        d_y = torch.from_numpy(yw).to(dev)
        d_o = torch.full((nxi, nyi), np.nan, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        handle = C.c_void_p(st.cuda_stream) if st is not None else None
        rc = lib.flct_gpu_interpcc2d_noalloc(ptr(d_f), XMISS, gx, gy, ptr(d_x), nxi, ptr(d_y), nyi,
                                             ptr(d_o), handle)
        if st is not None:
            st.synchronize()
        torch.cuda.synchronize()
        assert rc == _lib.OK
        assert np.array_equal(d_o.cpu().numpy(), want)

    # sizes beyond the fixed scratch are refused, small grids too
    d_big = torch.zeros(1, dtype=torch.float64, device=dev)
    too_many = _lib.load().flct_gpu_interpcc2d_noalloc(
        ptr(d_f), XMISS, gx, gy, ptr(d_big), 16385, ptr(d_big), 4, ptr(d_big), None)
    assert too_many == _lib.ERR_UNSUPPORTED
    small = lib.flct_gpu_interpcc2d_noalloc(ptr(d_f), XMISS, 2, gy, ptr(d_x), nxi, ptr(d_y), nyi,
                                            ptr(d_o), None)
    assert small == _lib.ERR_GRID_TOO_SMALL
