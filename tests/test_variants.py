"""Every kernel variant the autotuner can choose for the single-CTA sizes
(plain, pipelined with 2 / 3 buffers, half / twice the values per thread,
512- / 128-thread CTAs, pipelined with a split exchange area), forced with CKFFT_CUDA_VARIANT in its own process,
against the oracle: complex 2^6 .. 2^14 and real 2^7 .. 2^15, forward and
inverse, batches that end in a partial CTA."""
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
ctx = binding.Context(1 << 15)
o = orc.Oracle(1 << 15)
rng = np.random.default_rng(11)
worst = 0.0
for L in range(6, 15):
    for kind in ("cfwd", "cinv", "rfwd", "rinv"):
        real = kind[0] == "r"
        n = 1 << (L + 1) if real else 1 << L
        count = 37
        if kind == "rfwd":
            x = rng.standard_normal((count, n)).astype(np.float32)
            y = torch.full((count, n // 2 + 1), float("nan"), dtype=torch.complex64, device="cuda")
        elif kind == "rinv":
            x = (rng.standard_normal((count, n // 2 + 1)) + 1j * rng.standard_normal((count, n // 2 + 1))).astype(np.complex64)
            y = torch.full((count, n), float("nan"), device="cuda")
        else:
            x = (rng.standard_normal((count, n)) + 1j * rng.standard_normal((count, n))).astype(np.complex64)
            y = torch.full((count, n), float("nan"), dtype=torch.complex64, device="cuda")
        xd = torch.from_numpy(x).cuda()
        torch.cuda.synchronize()
        assert ctx.batch(kind, n, count, xd, y) == 1, binding.last_error()
        got = y.cpu().numpy()
        code = {"cfwd": 0, "cinv": 1, "rfwd": 2, "rinv": 3}[kind]
        ref = o.batch(code, n, count, x, 4)
        for f in range(count):
            e = orc.rel_l2(got[f], ref[f])
            assert e <= 1e-5, (kind, n, f, e)
            worst = max(worst, e)
print("ok", worst)
"""


@pytest.mark.parametrize("variant", [0, 2, 3, 4, 5, 6, 7, 8])
def test_variant_matches_oracle(torch_cuda, variant):
    env = dict(os.environ, CKFFT_CUDA_VARIANT=str(variant))
    r = subprocess.run([sys.executable, "-c", f"ROOT = {ROOT!r}\n" + CHILD], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0 and "ok" in r.stdout, r.stdout + r.stderr
