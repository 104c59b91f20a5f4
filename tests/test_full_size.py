"""GPU checks at the workloads' full sizes, through size-independent properties
(round trips) plus oracle spot checks of sampled frames."""
import numpy as np
import pytest

from conftest import assert_close, rel_l2
from ckfft_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def test_workload1_complex_round_trip(torch_cuda, ctx_cache, oracle_mod):
    """4096 x N=1024 complex, U[-1,1) seed 0: inverse(forward(x)) = 1024 x."""
    torch = torch_cuda
    n, frames = wl.W1_N, wl.W1_FRAMES
    x = wl.complex_uniform(frames, n, wl.W1_SEED)
    ctx = ctx_cache(n)
    xd = torch.from_numpy(x).cuda()
    X = torch.empty_like(xd)
    y = torch.empty_like(xd)
    ctx.check(ctx.batch("cfwd", n, frames, xd, X))
    ctx.check(ctx.batch("cinv", n, frames, X, y))
    assert rel_l2(y.cpu().numpy() / n, x) < 1e-6
    o = oracle_mod.Oracle(n)
    Xh = X.cpu().numpy()
    for f in (0, 1, 2047, 4095):
        assert_close(Xh[f], o.complex(n, x[f]), n, f"frame {f}")


def test_workload2_real_round_trip(torch_cuda, ctx_cache, oracle_mod):
    """65536 x N=4096 real sinusoid frames: inverse(forward(x)) = 2n x."""
    torch = torch_cuda
    n, frames = wl.W2_N, wl.W2_FRAMES
    x = wl.sine_frames_torch(frames, n, wl.W2_SEED)
    ctx = ctx_cache(n)
    X = torch.empty((frames, n // 2 + 1), dtype=torch.complex64, device="cuda")
    y = torch.empty_like(x)
    ctx.check(ctx.batch("rfwd", n, frames, x, X))
    ctx.check(ctx.batch("rinv", n, frames, X, y))
    err = (torch.linalg.vector_norm((y / (2 * n) - x).double()) / torch.linalg.vector_norm(x.double())).item()
    assert err < 1e-6
    o = oracle_mod.Oracle(n)
    xs = x[[0, 1, 32767, 65535]].cpu().numpy()
    Xs = X[[0, 1, 32767, 65535]].cpu().numpy()
    for i in range(4):
        assert_close(Xs[i], o.real_forward(n, xs[i]), n, f"frame {i}")


@pytest.mark.parametrize("l2", list(wl.W3_LOG2))
def test_workload3_round_trip(torch_cuda, ctx_cache, l2):
    torch = torch_cuda
    n = 1 << l2
    x = wl.complex_normal(n, seed=l2)
    ctx = ctx_cache(n)
    xd = torch.from_numpy(x).cuda()
    X = torch.empty_like(xd)
    y = torch.empty_like(xd)
    ctx.check(ctx.batch("cfwd", n, 1, xd, X))
    ctx.check(ctx.batch("cinv", n, 1, X, y))
    assert rel_l2(y.cpu().numpy() / n, x) < 5e-6
