"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on CPU.

Tolerances for the CUDA path against the reference's output (or the oracle,
which is bit-identical to it):
  relative L2 error            <= 1e-5
  max element error / rms(ref) <= 2e-6 * max(1, log2 n)
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

REL_L2_TOL = 1e-5
ELEM_TOL_PER_LOG2 = 2e-6


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libckfft_cuda.so")


@pytest.fixture(scope="session")
def golden():
    return np.load(os.path.join(ROOT, "tests", "golden", "ckfft_golden.npz"))


@pytest.fixture(scope="session")
def kiss_golden():
    return np.load(os.path.join(ROOT, "tests", "golden", "kiss_golden.npz"))


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as orc

    orc.build(with_reference=False)
    return orc


def rel_l2(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    dt = np.complex128 if (np.iscomplexobj(a) or np.iscomplexobj(b)) else np.float64
    a = a.astype(dt)
    b = b.astype(dt)
    den = np.linalg.norm(b.ravel())
    num = np.linalg.norm((a - b).ravel())
    return float(num / den) if den > 0 else float(num)


def assert_close(got, ref, n, what=""):
    """The parity bar: relative L2 and per-element-norm error."""
    got = np.asarray(got)
    ref = np.asarray(ref)
    assert got.shape == ref.shape, (what, got.shape, ref.shape)
    e = rel_l2(got, ref)
    assert e <= REL_L2_TOL, f"{what}: rel L2 {e:.3e} > {REL_L2_TOL}"
    r = ref.astype(np.complex128 if np.iscomplexobj(ref) else np.float64)
    rms = np.sqrt(np.mean(np.abs(r) ** 2))
    if rms > 0:
        worst = np.max(np.abs(got.astype(r.dtype) - r)) / rms
        lim = ELEM_TOL_PER_LOG2 * max(1, int(np.log2(max(n, 1))))
        assert worst <= lim, f"{what}: max element error {worst:.3e} rms > {lim:.3e}"
    return e


@pytest.fixture(scope="session")
def torch_cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for a gpu-marked test")
    return torch


@pytest.fixture(scope="session")
def lib(torch_cuda):
    from ckfft_gb300 import binding

    return binding.load()


@pytest.fixture(scope="session")
def ctx_cache(lib):
    from ckfft_gb300 import binding

    cache = {}

    def get(nmax, direction=binding.BOTH):
        key = (nmax, direction)
        if key not in cache:
            cache[key] = binding.Context(nmax, direction)
        return cache[key]

    yield get
    for c in cache.values():
        c.close()
