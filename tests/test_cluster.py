"""The opt-in cluster (distributed shared memory) path for complex 2^14..2^16,
run in a child process because the switch is read once per process."""
import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

CHILD = r"""
import sys, numpy as np, torch
sys.path.insert(0, ROOT)
sys.path.insert(0, ROOT + '/tests')
from conftest import assert_close
from ckfft_gb300 import binding
from oracle import oracle as orc
orc.build(with_reference=False)
ctx = binding.Context(1 << 16)
o = orc.Oracle(1 << 16)
rng = np.random.default_rng(5)
for l2 in (14, 15, 16):
    n = 1 << l2
    x = (rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))).astype(np.complex64)
    for kind, inv in (('cfwd', False), ('cinv', True)):
        xd = torch.from_numpy(x).cuda()
        y = torch.empty_like(xd)
        before = binding.launch_count()
        ctx.check(ctx.batch(kind, n, 3, xd, y))
        assert binding.launch_count() - before == 1       # one cluster launch, no second pass
        got = y.cpu().numpy()
        for f in range(3):
            assert_close(got[f], o.complex(n, x[f], inv), n, f'cluster {kind} 2^{l2}')
print('cluster ok')
""".replace("ROOT", repr(ROOT))


def test_cluster_path_matches_oracle():
    env = dict(os.environ, CKFFT_CUDA_CLUSTER="1")
    r = subprocess.run([sys.executable, "-c", CHILD], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "cluster ok" in r.stdout
