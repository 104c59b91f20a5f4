"""ckfft_gb300 -- Cricket FFT's C API (power-of-two FP32 complex and real
transforms) implemented as hand-written CUDA kernels for GB300 (sm_103a).

The product is the shared library `libckfft_cuda.so` with the C ABI declared in
`include/ckfft_cuda.h`.  This package builds it (`python -m ckfft_gb300.build`)
and offers a thin ctypes binding (`ckfft_gb300.binding`) plus seeded workload
generators (`ckfft_gb300.workloads`).
"""
from .binding import Context, CkFftError, load, last_error, launch_count, header_functions  # noqa: F401

__all__ = ["Context", "CkFftError", "load", "last_error", "launch_count", "header_functions"]
