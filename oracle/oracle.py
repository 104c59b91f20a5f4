"""ctypes front end for the CPU oracle and for the reference build (test infrastructure).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this module.
It checks results and is never the product: the product library is
ckfft_gb300/libckfft_cuda.so and it has no CPU path.

Three back ends share one small interface (`complex`, `real_forward`,
`real_inverse`, `batch`):
  * Oracle    -- oracle/ckfft_oracle.c, a restatement of the reference's scalar
                 path (src/ckfft/fft_default.cpp, fft_real_default.cpp, ...).
  * Reference -- oracle/_ref/libckfft_ref.so, the reference's own sources built
                 by oracle/Makefile (present only where the reference tree is).
  * Kiss      -- oracle/_ref/libkissfft_ref.so, the reference tree's vendored
                 kiss_fft 1.3.0, the reference test harness's comparison library
                 (src/test/test.cpp:315-395).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF = os.path.join(HERE, "_ref")
# the reference source tree (read only; present only where the reference was checked out)
REF_TREE = os.environ.get("CKFFT_REFERENCE_TREE", "/root/reference")

FORWARD, INVERSE, BOTH = 1, 2, 3
KIND_CFWD, KIND_CINV, KIND_RFWD, KIND_RINV = 0, 1, 2, 3


def build(with_reference: bool | None = None) -> None:
    """Compile the oracle (and the reference build when its tree is present)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if with_reference is None:
        with_reference = os.path.isdir(os.path.join(REF_TREE, "src", "ckfft"))
    if with_reference:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_TREE}"], check=True)


def reference_available() -> bool:
    return os.path.exists(os.path.join(REF, "libckfft_ref.so"))


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.complex64)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class _Backend:
    """Common numpy wrappers; subclasses bind the four raw calls."""

    def complex(self, n, x, inverse=False):
        x = _c64(x)
        out = np.zeros(n, np.complex64)
        r = self._complex(n, x, out, inverse)
        return out if r else None

    def real_forward(self, n, x):
        x = _f32(x)
        # one spare bin: the reference writes n/2+2 bins for n == 4 (fft_real.cpp:46-47)
        out = np.zeros(n // 2 + 2, np.complex64)
        r = self._real_forward(n, x, out)
        return out[: n // 2 + 1].copy() if r else None

    def real_inverse(self, n, X):
        X = _c64(X)
        out = np.zeros(n, np.float32)
        tmp = np.zeros(n // 2 + 1, np.complex64)
        r = self._real_inverse(n, X, out, tmp)
        return out if r else None


class Oracle(_Backend):
    """The C restatement, one context per instance."""

    _lib = None

    @classmethod
    def lib(cls, fast=False):
        name = "libckfft_oracle_fast.so" if fast else "libckfft_oracle.so"
        path = os.path.join(BUILD, name)
        if not os.path.exists(path):
            build(with_reference=False)
        lib = C.CDLL(path)
        lib.ock_init.restype = C.c_void_p
        lib.ock_init.argtypes = [C.c_int, C.c_int]
        lib.ock_free.argtypes = [C.c_void_p]
        lib.ock_table.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        lib.ock_complex.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
        lib.ock_real_forward.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        lib.ock_real_inverse.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.ock_batch.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_longlong,
                                  C.c_void_p, C.c_void_p, C.c_int]
        return lib

    def __init__(self, nmax, direction=BOTH, fast=False):
        self.lib_ = Oracle.lib(fast)
        self.nmax = nmax
        self.ctx = self.lib_.ock_init(nmax, direction)
        if not self.ctx:
            raise ValueError(f"oracle init failed (nmax={nmax}, direction={direction})")

    def close(self):
        if self.ctx:
            self.lib_.ock_free(self.ctx)
            self.ctx = None

    __del__ = close

    def table(self, inverse=False):
        out = np.zeros(self.nmax, np.complex64)
        return out if self.lib_.ock_table(self.ctx, int(inverse), _ptr(out)) else None

    def _complex(self, n, x, out, inverse):
        return self.lib_.ock_complex(self.ctx, n, _ptr(x), _ptr(out), int(inverse))

    def _real_forward(self, n, x, out):
        return self.lib_.ock_real_forward(self.ctx, n, _ptr(x), _ptr(out))

    def _real_inverse(self, n, X, out, tmp):
        return self.lib_.ock_real_inverse(self.ctx, n, _ptr(X), _ptr(out), _ptr(tmp))

    def batch(self, kind, n, frames, inp, threads=1):
        """Runs `frames` transforms over a contiguous 2-D array; returns the output."""
        if kind in (KIND_CFWD, KIND_CINV):
            inp = _c64(inp).reshape(frames, n)
            out = np.empty((frames, n), np.complex64)
        elif kind == KIND_RFWD:
            inp = _f32(inp).reshape(frames, n)
            out = np.empty((frames, n // 2 + 1), np.complex64)
        else:
            inp = _c64(inp).reshape(frames, n // 2 + 1)
            out = np.empty((frames, n), np.float32)
        ok = self.lib_.ock_batch(self.ctx, kind, n, frames, _ptr(inp), _ptr(out), threads)
        if not ok:
            raise RuntimeError("oracle batch failed")
        return out

    def batch_into(self, kind, n, frames, inp, out, threads=1):
        """Like batch() but with caller-provided contiguous arrays (for timing)."""
        ok = self.lib_.ock_batch(self.ctx, kind, n, frames, _ptr(inp), _ptr(out), threads)
        if not ok:
            raise RuntimeError("oracle batch failed")


class Reference(_Backend):
    """The reference's own sources built into oracle/_ref (parity flags)."""

    def __init__(self, nmax, direction=BOTH, fast=False):
        name = "libckfft_ref_fast.so" if fast else "libckfft_ref.so"
        path = os.path.join(REF, name)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        lib = C.CDLL(path)
        lib.CkFftInit.restype = C.c_void_p
        lib.CkFftInit.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        lib.CkFftShutdown.argtypes = [C.c_void_p]
        for f in ("CkFftComplexForward", "CkFftComplexInverse", "CkFftRealForward"):
            getattr(lib, f).argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        lib.CkFftRealInverse.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        self.lib_ = lib
        self.nmax = nmax
        self.ctx = lib.CkFftInit(nmax, direction, None, None)
        if not self.ctx:
            raise ValueError("reference init failed")

    def close(self):
        if self.ctx:
            self.lib_.CkFftShutdown(self.ctx)
            self.ctx = None

    __del__ = close

    def _complex(self, n, x, out, inverse):
        f = self.lib_.CkFftComplexInverse if inverse else self.lib_.CkFftComplexForward
        return f(self.ctx, n, _ptr(x), _ptr(out))

    def _real_forward(self, n, x, out):
        return self.lib_.CkFftRealForward(self.ctx, n, _ptr(x), _ptr(out))

    def _real_inverse(self, n, X, out, tmp):
        return self.lib_.CkFftRealInverse(self.ctx, n, _ptr(X), _ptr(out), _ptr(tmp))


class Kiss:
    """kiss_fft 1.3.0 from the reference tree; outputs scaled like ckfft
    (real forward x2, as src/test/test.cpp:368-372 does)."""

    def __init__(self):
        lib = C.CDLL(os.path.join(REF, "libkissfft_ref.so"))
        lib.kiss_fft_alloc.restype = C.c_void_p
        lib.kiss_fft_alloc.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        lib.kiss_fft.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        lib.kiss_fftr_alloc.restype = C.c_void_p
        lib.kiss_fftr_alloc.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        lib.kiss_fftr.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        lib.kiss_fftri.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        self.lib_ = lib
        self.libc = C.CDLL(None)
        self.libc.free.argtypes = [C.c_void_p]

    def complex(self, n, x, inverse=False):
        x = _c64(x)
        out = np.zeros(n, np.complex64)
        cfg = self.lib_.kiss_fft_alloc(n, int(inverse), None, None)
        self.lib_.kiss_fft(cfg, _ptr(x), _ptr(out))
        self.libc.free(cfg)
        return out

    def real_forward(self, n, x):
        x = _f32(x)
        out = np.zeros(n // 2 + 1, np.complex64)
        cfg = self.lib_.kiss_fftr_alloc(n, 0, None, None)
        self.lib_.kiss_fftr(cfg, _ptr(x), _ptr(out))
        self.libc.free(cfg)
        return out * np.float32(2.0)


def rel_l2(a, b):
    """Relative L2 error ||a - b|| / ||b|| in float64."""
    a = np.asarray(a, np.complex128 if np.iscomplexobj(a) or np.iscomplexobj(b) else np.float64)
    b = np.asarray(b, a.dtype)
    den = np.linalg.norm(b.ravel())
    num = np.linalg.norm((a - b).ravel())
    return float(num / den) if den > 0 else float(num)


def fp64_complex(x, inverse=False):
    """Unscaled FP64 DFT with the reference's conventions (inverse is x n)."""
    x = np.asarray(x, np.complex128)
    return np.fft.ifft(x, axis=-1) * x.shape[-1] if inverse else np.fft.fft(x, axis=-1)


def fp64_real_forward(x):
    """2 * rfft(x): the reference's real forward output scale."""
    return 2.0 * np.fft.rfft(np.asarray(x, np.float64), axis=-1)


def fp64_real_inverse(X, n):
    """FP64 evaluation of the reference's real inverse as a linear map
    (src/ckfft/fft_real_default.cpp:65-114 for n >= 8, fft_real.cpp:62-93 below):
    Y[k] = (X[k] + conj X[m-k]) + i e^{+2 pi i k/n} (X[k] - conj X[m-k]), k < m = n/2,
    z = unscaled inverse DFT_m(Y), out = (Re z[0], Im z[0], Re z[1], ...).
    For Hermitian-consistent X this is n * irfft(X); unlike irfft it also
    defines the result for nonzero imaginary parts in bins 0 and n/2, exactly
    as the reference does.  A forward -> inverse round trip gains 2n."""
    X = np.asarray(X, np.complex128)
    if n == 1:
        return X[..., 0].real[..., None].copy()
    if n == 2:
        return np.stack([X[..., 0].real + X[..., 1].real, X[..., 0].real - X[..., 1].real], -1)
    if n == 4:
        s02 = X[..., 0].real + X[..., 2].real
        s13 = 2.0 * X[..., 1].real
        d02 = X[..., 0].real - X[..., 2].real
        d13 = 2.0 * X[..., 1].imag
        return np.stack([s02 + s13, d02 - d13, s02 - s13, d02 + d13], -1)
    m = n // 2
    k = np.arange(m)
    a = X[..., :m]
    b = np.conj(X[..., m - k])
    w = np.exp(2j * np.pi * k / n)
    y = (a + b) + 1j * w * (a - b)
    z = np.fft.ifft(y, axis=-1) * m
    out = np.empty(X.shape[:-1] + (n,), np.float64)
    out[..., 0::2] = z.real
    out[..., 1::2] = z.imag
    return out
