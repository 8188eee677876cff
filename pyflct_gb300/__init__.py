"""pyflct_gb300: GB300-native FLCT (Fourier Local Correlation Tracking).

The compute path is hand-written CUDA for sm_103a behind a C ABI
(include/flct_gpu.h, built into libflctgpu.so); this package is the thin
Python host side over that ABI.  There is no CPU fallback: every entry point
raises if the CUDA library cannot be loaded or no GPU is present.
"""
__version__ = "0.1.0"
