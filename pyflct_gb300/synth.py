"""Seeded synthetic FLCT inputs.

There is no public benchmark data for FLCT; the workloads are synthetic
image pairs with the shapes, sizes and value distributions of the five
benchmark configurations (128^2 Gaussian blobs, k^-2 random fields at 512^2,
1024^2 and 4096^2, and a batch of 64 heterogeneous pairs).  Every generator
takes a numpy Generator so results are reproducible; seeds are
``default_rng(20260 + k)`` for configuration k.

Arrays are C-order [nx][ny] (nx = slow axis = IDL y), as inside the
reference after reading a vel_ccor file.  A shift ``(delx, dely)`` is along
the (fast, slow) axis, matching the reference warp's transposed convention:
image2(r) = image1(r - d).
"""
from __future__ import annotations

import numpy as np

WARP_PI = 3.1415926535898  # the reference warp's truncated pi (warp.c:768)


def make_freq(n: int) -> np.ndarray:
    """Integer wavenumbers in FFT order with the Nyquist entry +n/2."""
    k = np.fft.fftfreq(n) * n
    if n % 2 == 0:
        k[n // 2] = n // 2
    return k


def kfield(shape, rng, slope: float = 2.0) -> np.ndarray:
    """Random field with isotropic power spectrum ~ k^-slope, unit RMS."""
    n0, n1 = shape
    kx = np.fft.fftfreq(n0)[:, None] * n0
    ky = np.fft.fftfreq(n1)[None, :] * n1
    k = np.hypot(kx, ky)
    amp = np.zeros_like(k)
    amp[k > 0] = k[k > 0] ** (-slope / 2.0)
    z = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    f = np.real(np.fft.ifft2(z * amp))
    return f / np.sqrt(np.mean(f * f))


def blobs(shape, rng, count=200, noise=0.01) -> np.ndarray:
    """Sum of Gaussian blobs (centres uniform, amplitude N(0,1), width U[2,6])."""
    n0, n1 = shape
    ii, jj = np.meshgrid(np.arange(n0), np.arange(n1), indexing="ij")
    f = np.zeros(shape)
    for _ in range(count):
        ci, cj = rng.uniform(0, n0), rng.uniform(0, n1)
        a, w = rng.standard_normal(), rng.uniform(2, 6)
        f += a * np.exp(-((ii - ci) ** 2 + (jj - cj) ** 2) / (2 * w * w))
    return f + rng.normal(0.0, noise, shape)


def fourier_shift(arr, delx: float, dely: float) -> np.ndarray:
    """Exact periodic sub-pixel shift by (delx fast, dely slow), the uniform
    warp's semantics (phase exp(i 2 pi (kx dxarg + ky dyarg)) with the +n/2
    Nyquist convention, real part of the inverse)."""
    n0, n1 = arr.shape
    kx = make_freq(n0)[:, None]
    ky = make_freq(n1)[None, :]
    dxarg = -dely / n0
    dyarg = -delx / n1
    ph = np.exp(1j * 2.0 * WARP_PI * (kx * dxarg + ky * dyarg))
    return np.real(np.fft.ifft2(np.fft.fft2(arr) * ph))


def rotation_shift(shape, degrees: float):
    """Displacement (delx fast, dely slow) of a rigid rotation about the
    image centre: d = R(theta)(r - c) - (r - c)."""
    n0, n1 = shape
    c0, c1 = (n0 - 1) / 2.0, (n1 - 1) / 2.0
    ii, jj = np.meshgrid(np.arange(n0) - c0, np.arange(n1) - c1, indexing="ij")
    t = np.deg2rad(degrees)
    dfast = np.cos(t) * jj - np.sin(t) * ii - jj
    dslow = np.sin(t) * jj + np.cos(t) * ii - ii
    return dfast, dslow


def vortex_shift(shape, rng, count=5, rmin=40, rmax=120, vmin=0.05, vmax=0.8):
    """Sum of Gaussian vortices v_theta = V (r/R) exp((1 - r^2/R^2)/2)."""
    n0, n1 = shape
    ii, jj = np.meshgrid(np.arange(n0), np.arange(n1), indexing="ij")
    dfast = np.zeros(shape)
    dslow = np.zeros(shape)
    for _ in range(count):
        ci, cj = rng.uniform(0, n0), rng.uniform(0, n1)
        R, V = rng.uniform(rmin, rmax), rng.uniform(vmin, vmax) * rng.choice([-1.0, 1.0])
        di, dj = ii - ci, jj - cj
        r = np.hypot(di, dj)
        vt = V * (r / R) * np.exp((1.0 - (r / R) ** 2) / 2.0)
        with np.errstate(invalid="ignore", divide="ignore"):
            ur = np.where(r > 0, -di / r, 0.0)
            uf = np.where(r > 0, dj / r, 0.0)
        # tangential direction (-sin, cos) in (slow, fast) coordinates
        dslow += vt * ur
        dfast += vt * uf
    return dfast, dslow


def smooth_shift(shape, rng, rms=0.3, slope=3.0):
    """Random displacement field with a k^-slope spectrum scaled to RMS |d|."""
    a = kfield(shape, rng, slope)
    b = kfield(shape, rng, slope)
    s = rms / np.sqrt(np.mean(a * a + b * b))
    return a * s, b * s


def spline_warp(arr, dfast, dslow) -> np.ndarray:
    """Periodic bicubic-spline resampling image2(r) = image1(r - d): a fast
    stand-in for the exact spectral warp when only the workload shape
    matters (timing), not the warp's own arithmetic."""
    from scipy.ndimage import map_coordinates

    n0, n1 = arr.shape
    ii, jj = np.meshgrid(np.arange(n0), np.arange(n1), indexing="ij")
    return map_coordinates(arr, [ii - dslow, jj - dfast], order=3, mode="grid-wrap")


def spectral_warp(arr, dfast, dslow, device=0) -> np.ndarray:
    """image2(r) = image1(r - d(r)) by the reference warp's own arithmetic
    (warp_frac2d, warp.c:883-1011: the image's Fourier series evaluated at
    every displaced point), run on the GPU by this library."""
    from .flct import warp_frac2d

    return warp_frac2d(arr, dfast, dslow, 1, device)


def config1(rng=None):
    """128x128 blobs; image2 = exact shift (vx, vy) = (+0.3, -0.2); sigma 4."""
    rng = rng or np.random.default_rng(20261)
    f1 = blobs((128, 128), rng)
    f2 = fourier_shift(f1, 0.3, -0.2)
    return f1, f2, dict(deltat=1.0, deltas=1.0, sigma=4.0)


def config2_image1(rng=None, n=512):
    """k^-2 field with 20% of pixels replaced by U(-0.05, 0.05)."""
    rng = rng or np.random.default_rng(20262)
    f1 = kfield((n, n), rng)
    mask = rng.random((n, n)) < 0.2
    f1[mask] = rng.uniform(-0.05, 0.05, mask.sum())
    return f1


def config3_image1(rng=None, n=1024):
    rng = rng or np.random.default_rng(20263)
    return kfield((n, n), rng)


def config4_pairs(rng=None, count=64):
    """64 pairs: sides from {128..768}, sigma from {3,5,8,12}, uniform shifts."""
    rng = rng or np.random.default_rng(20264)
    sides = [128, 256, 384, 512, 768]
    out = []
    for _ in range(count):
        n0, n1 = int(rng.choice(sides)), int(rng.choice(sides))
        sigma = float(rng.choice([3, 5, 8, 12]))
        f1 = kfield((n0, n1), rng)
        vx, vy = rng.uniform(-1, 1, 2)
        out.append((f1, fourier_shift(f1, vx, vy), dict(deltat=1.0, deltas=1.0, sigma=sigma),
                    (vx, vy)))
    return out

def config5(rng=None, n=4096, device=0):
    """4096^2 float32 k^-2 field; image2 = image1 displaced along a k^-3
    random field of RMS 0.3 px by the GPU spectral warp (warp_frac2d, the
    reference warp's arithmetic), rounded to float32; sigma 15 (box 64)."""
    rng = rng or np.random.default_rng(20265)
    f1 = kfield((n, n), rng).astype(np.float32).astype(np.float64)
    dfast, dslow = smooth_shift((n, n), rng, rms=0.3, slope=3.0)
    f2 = spectral_warp(f1, dfast, dslow, device).astype(np.float32).astype(np.float64)
    return f1, f2, dict(deltat=1.0, deltas=1.0, sigma=15.0), (dfast, dslow)
