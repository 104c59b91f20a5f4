"""Generates tests/golden/kiss_golden.npz from kiss_fft 1.3.0 of the
reference tree (ext/kiss_fft130, built into oracle/_ref/libkissfft_ref.so by
`make -C oracle ref`), the comparison library of the reference's test
harness (src/test/test.cpp:315-395).

    python tests/golden/make_kiss_golden.py

Runs only where the reference tree and its build exist; the committed .npz
travels with the tests.  All outputs are kiss_fft's own, unscaled:
  cin_{l2} / cfwd_{l2} / cinv_{l2}  complex input, kiss_fft forward / inverse,
                                    n = 2^l2, l2 = 0..11
  rin_{l2} / rfwd_{l2}              real input and kiss_fftr, l2 = 1..11
  rinv_{l2}                         kiss_fftri of rfwd_{l2} (round trip, gain n)
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(ROOT, "oracle", "_ref", "libkissfft_ref.so")


def main():
    if not os.path.exists(LIB):
        sys.exit(f"{LIB} is missing: run `make -C oracle ref` where the reference tree exists")
    k = C.CDLL(LIB)
    vp = C.c_void_p
    k.kiss_fft_alloc.restype = vp
    k.kiss_fft_alloc.argtypes = [C.c_int, C.c_int, vp, vp]
    k.kiss_fft.argtypes = [vp, vp, vp]
    k.kiss_fftr_alloc.restype = vp
    k.kiss_fftr_alloc.argtypes = [C.c_int, C.c_int, vp, vp]
    k.kiss_fftr.argtypes = [vp, vp, vp]
    k.kiss_fftri.argtypes = [vp, vp, vp]
    libc = C.CDLL(None)
    libc.free.argtypes = [vp]
    rng = np.random.default_rng(20261204)
    out = {}
    for l2 in range(0, 12):
        n = 1 << l2
        x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
        out[f"cin_{l2}"] = x
        for inv, name in ((0, "cfwd"), (1, "cinv")):
            y = np.zeros(n, np.complex64)
            cfg = k.kiss_fft_alloc(n, inv, None, None)
            k.kiss_fft(cfg, x.ctypes.data, y.ctypes.data)
            libc.free(cfg)
            out[f"{name}_{l2}"] = y
        if l2 >= 1:
            r = rng.uniform(-1, 1, n).astype(np.float32)
            out[f"rin_{l2}"] = r
            X = np.zeros(n // 2 + 1, np.complex64)
            cfg = k.kiss_fftr_alloc(n, 0, None, None)
            k.kiss_fftr(cfg, r.ctypes.data, X.ctypes.data)
            libc.free(cfg)
            out[f"rfwd_{l2}"] = X
            y = np.zeros(n, np.float32)
            cfg = k.kiss_fftr_alloc(n, 1, None, None)
            k.kiss_fftri(cfg, X.ctypes.data, y.ctypes.data)
            libc.free(cfg)
            out[f"rinv_{l2}"] = y
    np.savez_compressed(os.path.join(HERE, "kiss_golden.npz"), **out)
    print(f"wrote {len(out)} arrays")


if __name__ == "__main__":
    main()
