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


def assert_close_rows(got, ref, n, what="", chunk=2048):
    """assert_close applied to every row of two 2-D arrays (one transform per
    row), vectorised in chunks of rows; returns the worst relative L2 error."""
    got = np.asarray(got)
    ref = np.asarray(ref)
    assert got.shape == ref.shape, (what, got.shape, ref.shape)
    lim = ELEM_TOL_PER_LOG2 * max(1, int(np.log2(max(n, 1))))
    dt = np.complex128 if np.iscomplexobj(ref) else np.float64
    worst = 0.0
    for s in range(0, got.shape[0], chunk):
        r = ref[s:s + chunk].astype(dt)
        d = np.abs(got[s:s + chunk].astype(dt) - r)
        den = np.sqrt(np.sum(np.abs(r) ** 2, axis=1))
        num = np.sqrt(np.sum(d ** 2, axis=1))
        rel = np.where(den > 0, num / np.where(den > 0, den, 1.0), num)
        i = int(np.argmax(rel))
        assert rel[i] <= REL_L2_TOL, f"{what}: row {s + i} rel L2 {rel[i]:.3e} > {REL_L2_TOL}"
        rms = den / np.sqrt(r.shape[1])
        el = np.where(rms > 0, d.max(axis=1) / np.where(rms > 0, rms, 1.0), 0.0)
        j = int(np.argmax(el))
        assert el[j] <= lim, f"{what}: row {s + j} max element error {el[j]:.3e} rms > {lim:.3e}"
        worst = max(worst, float(rel[i]))
    return worst


def host_threads():
    return max(1, os.cpu_count() or 1)


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
