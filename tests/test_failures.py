"""Failure detection without a GPU fault: the bounded device-side waits run
out on purpose (CkFftCudaSelfTestWait) and report through the error word
while the context keeps working; injected allocation failures
(CKFFT_CUDA_FAIL_ALLOC) come back as 0 / NULL with a message, and the next
call succeeds.  Host-side rejections (malformed jobs, layouts, requests)
are covered next to their entry points."""
import os
import subprocess
import sys

import pytest

from conftest import ROOT
from ckfft_gb300 import binding


def test_self_test_needs_a_context():
    from ckfft_gb300 import build
    build.build()
    lib = binding.load()
    assert lib.CkFftCudaSelfTestWait(None, 0) == 0
    assert "context" in binding.last_error()


@pytest.mark.gpu
@pytest.mark.parametrize("which", [0, 1])
def test_bounded_wait_runs_out_and_reports(torch_cuda, ctx_cache, lib, which):
    ctx = ctx_cache(1024)
    assert lib.CkFftCudaSelfTestWait(ctx.handle, which) == 1, binding.last_error()
    assert lib.CkFftCudaSelfTestWait(ctx.handle, 7) == 0


CHILD = r"""
import sys, numpy as np, torch
sys.path.insert(0, ROOT)
from ckfft_gb300 import binding
lib = binding.load()
which = sys.argv[1]
if which == "init":
    h = lib.CkFftInit(1024, 3, None, None)
    assert not h, "the injected failure hits the twiddle table"
    assert "twiddles" in binding.last_error(), binding.last_error()
    ctx = binding.Context(1024)                   # the next allocation succeeds
    print("ok")
else:
    ctx = binding.Context(1 << 16)
    x = torch.randn((4, 1 << 16), dtype=torch.complex64, device="cuda")
    y = torch.zeros_like(x)
    assert ctx.batch("cfwd", 1 << 16, 4, x, y) == 0
    assert "scratch" in binding.last_error(), binding.last_error()
    assert ctx.batch("cfwd", 1 << 16, 4, x, y) == 1, binding.last_error()
    ref = torch.fft.fft(x.to(torch.complex128))
    err = (torch.linalg.norm(y.to(torch.complex128) - ref) / torch.linalg.norm(ref)).item()
    assert err < 1e-5, err
    print("ok")
"""


@pytest.mark.gpu
@pytest.mark.parametrize("which,k", [("init", "1"), ("batch", "2")])
def test_injected_allocation_failure(torch_cuda, which, k):
    env = dict(os.environ, CKFFT_CUDA_FAIL_ALLOC=k)
    r = subprocess.run([sys.executable, "-c", f"ROOT = {ROOT!r}\n" + CHILD, which], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0 and "ok" in r.stdout, r.stdout + r.stderr
