"""Complex 2^15 / 2^16 on the opt-in persistent kernel with asynchronously
copied tiles (fft_mid.cu, CKFFT_CUDA_MID=1; 2^16 as two-CTA clusters) and on
the default cluster two-pass kernel (fft_l2pass.cu, CKFFT_CUDA_MID=0): batches that fill the grid once, more than once and
partially, against the oracle.  Each setting runs in its own process (the
choice is read once per process)."""
import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

CHILD = r"""
import sys
import numpy as np
import torch
sys.path.insert(0, ROOT)
from ckfft_gb300 import binding
from oracle import oracle as orc
orc.build(with_reference=False)
ctx = binding.Context(1 << 16)
o = orc.Oracle(1 << 16)
worst = 0.0
for l2 in (15, 16):
    n = 1 << l2
    for count in (1, 3, 151, 153, 311):
        for kind in ("cfwd", "cinv"):
            g = torch.Generator(device="cuda")
            g.manual_seed(count * 31 + l2)
            x = torch.randn((count, n), dtype=torch.complex64, device="cuda", generator=g)
            y = torch.full_like(x, float("nan"))
            assert ctx.batch(kind, n, count, x, y) == 1, binding.last_error()
            xs, ys = x.cpu().numpy(), y.cpu().numpy()
            for f in sorted({0, count // 2, count - 1}):
                e = orc.rel_l2(ys[f], o.complex(n, xs[f], kind == "cinv"))
                assert e <= 1e-5, (l2, count, kind, f, e)
                worst = max(worst, e)
print("ok", worst)
"""


@pytest.mark.parametrize("mode", ["1", "0"])
def test_mid_sizes_each_kernel(torch_cuda, mode):
    env = dict(os.environ, CKFFT_CUDA_MID=mode)
    r = subprocess.run([sys.executable, "-c", f"ROOT = {ROOT!r}\n" + CHILD], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and "ok" in r.stdout, r.stdout + r.stderr


def test_blocking_call_sees_earlier_default_stream_work(torch_cuda, ctx_cache, oracle_mod):
    """A reference-style blocking call made right after work queued on the
    legacy default stream (here a 256 MiB copy into the input) reads the
    finished input: the library's streams are ordered after that stream."""
    torch = torch_cuda
    n, count = 1 << 15, 1024
    src = torch.randn((count, n), dtype=torch.complex64, device="cuda")
    x = torch.zeros_like(src)
    y = torch.zeros_like(src)
    ctx = ctx_cache(n)
    torch.cuda.synchronize()
    x.copy_(src)                                   # queued on the default stream, not waited for
    assert ctx.batch("cfwd", n, count, x, y) == 1
    o = oracle_mod.Oracle(n)
    xs, ys = src[-1].cpu().numpy(), y[-1].cpu().numpy()
    assert oracle_mod.rel_l2(ys, o.complex(n, xs)) <= 1e-5
