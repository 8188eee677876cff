"""The half-spectrum identity behind the tensor-core warp sum (CPU, numpy).

warp_frac2d's per-pixel sum (source/warp.c:940-1000)
    out[p] = (1/N) sum_{ii,jj} Re(F[ii][jj] exp(2 pi i (kx_ii tx + ky_jj ty)))
runs on the GPU over the columns jj = 0 .. ny/2 only, with weight 1 for
the self-paired columns (0 and, for even ny, ny/2) and 2 for the rest; the
Nyquist row ii = nx/2 of an even nx keeps weight 1 in every column and is
corrected by Re(ex A0) + 2 cos(kx tx) (Re G - Re A0).  This restates that
rearrangement in FP64 and checks it against the full sum for odd, even and
degenerate axes, with the reference's wavenumber order (make_freq,
warp.c:316-360).
"""
import numpy as np
import pytest


def freq(k, n):
    return k if k <= n // 2 else k - n


def full_sum(F, tx, ty):
    nx, ny = F.shape
    kx = np.array([freq(i, nx) for i in range(nx)])
    ky = np.array([freq(j, ny) for j in range(ny)])
    ex = np.exp(2j * np.pi * kx * tx)
    ey = np.exp(2j * np.pi * ky * ty)
    return np.real(np.sum(F * np.outer(ex, ey))) / F.size


def half_sum(F, tx, ty):
    nx, ny = F.shape
    ncol = ny // 2 + 1
    nyq_row = nx // 2 if nx % 2 == 0 else -1
    nyq_col = ny // 2 if ny % 2 == 0 else -1
    ky = np.arange(ncol)                      # 0 .. ny/2: no wrap in this range
    ey = np.exp(2j * np.pi * ky * ty)
    s = 0.0
    for ii in range(nx):
        w = np.where((ky == 0) | (ky == nyq_col) | (ii == nyq_row), 1.0, 2.0)
        G = np.sum(w * F[ii, :ncol] * ey)
        ex = np.exp(2j * np.pi * freq(ii, nx) * tx)
        if ii == nyq_row:
            a0 = F[ii, 0] + (F[ii, ny // 2] * ey[ny // 2] if ny % 2 == 0 else 0.0)
            s += np.real(ex * a0) + 2.0 * np.real(ex) * (np.real(G) - np.real(a0))
        else:
            s += np.real(ex * G)
    return s / F.size


@pytest.mark.parametrize("shape", [(6, 8), (7, 8), (6, 9), (7, 9), (2, 2), (1, 4), (4, 1), (2, 3), (16, 10)])
def test_half_spectrum_matches_full_sum(shape):
    rng = np.random.default_rng(shape[0] * 100 + shape[1])
    img = rng.standard_normal(shape) + 1.5
    F = np.fft.fft2(img)
    for _ in range(12):
        tx, ty = rng.uniform(-3, 3, 2)
        a, b = full_sum(F, tx, ty), half_sum(F, tx, ty)
        assert abs(a - b) <= 1e-12 * max(1.0, np.abs(img).max())


def test_half_spectrum_reproduces_integer_shift():
    """At tx = (i - s) / nx, ty = (j - t) / ny with integer s, t the sum is the
    circularly shifted image itself."""
    rng = np.random.default_rng(5)
    img = rng.standard_normal((8, 6))
    F = np.fft.fft2(img)
    for i, j, s, t in ((3, 2, 1, -2), (0, 5, -3, 4), (7, 0, 2, 1)):
        got = half_sum(F, (i - s) / 8.0, (j - t) / 6.0)
        assert abs(got - img[(i - s) % 8, (j - t) % 6]) <= 1e-12
