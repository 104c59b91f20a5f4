"""GPU checks at the workloads' full sizes: every frame of workloads 1 and 2
against the oracle, forward and inverse checked separately (the inverse on the
GPU's own spectra, so errors cannot cancel between the two kernels), the large
single transforms of workload 3 against the oracle, plus the round trips."""
import numpy as np
import pytest

from conftest import assert_close, assert_close_rows, host_threads, rel_l2
from ckfft_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def test_workload1_every_frame(torch_cuda, ctx_cache, oracle_mod):
    """4096 x N=1024 complex, U[-1,1) seed 0: every forward and every inverse
    output against the oracle; inverse(forward(x)) = 1024 x."""
    torch = torch_cuda
    orc = oracle_mod
    n, frames = wl.W1_N, wl.W1_FRAMES
    x = wl.complex_uniform(frames, n, wl.W1_SEED)
    ctx = ctx_cache(n)
    xd = torch.from_numpy(x).cuda()
    X = torch.empty_like(xd)
    y = torch.empty_like(xd)
    ctx.check(ctx.batch("cfwd", n, frames, xd, X))
    ctx.check(ctx.batch("cinv", n, frames, X, y))
    Xh, yh = X.cpu().numpy(), y.cpu().numpy()
    assert rel_l2(yh / n, x) < 1e-6
    o = orc.Oracle(n)
    assert_close_rows(Xh, o.batch(orc.KIND_CFWD, n, frames, x, host_threads()), n, "w1 forward")
    assert_close_rows(yh, o.batch(orc.KIND_CINV, n, frames, Xh, host_threads()), n, "w1 inverse")


def test_workload2_every_frame(torch_cuda, ctx_cache, oracle_mod):
    """65536 x N=4096 real sinusoid frames: every forward spectrum against the
    oracle, every inverse (of the GPU's spectra) against the oracle's inverse
    of the same spectra; inverse(forward(x)) = 2n x."""
    torch = torch_cuda
    orc = oracle_mod
    n, frames = wl.W2_N, wl.W2_FRAMES
    x = wl.sine_frames_torch(frames, n, wl.W2_SEED)
    ctx = ctx_cache(n)
    X = torch.empty((frames, n // 2 + 1), dtype=torch.complex64, device="cuda")
    y = torch.empty_like(x)
    ctx.check(ctx.batch("rfwd", n, frames, x, X))
    ctx.check(ctx.batch("rinv", n, frames, X, y))
    err = (torch.linalg.vector_norm((y / (2 * n) - x).double()) / torch.linalg.vector_norm(x.double())).item()
    assert err < 1e-6
    o = orc.Oracle(n)
    step = 16384
    for s in range(0, frames, step):
        xs = x[s:s + step].cpu().numpy()
        Xs = X[s:s + step].cpu().numpy()
        ys = y[s:s + step].cpu().numpy()
        c = xs.shape[0]
        assert_close_rows(Xs, o.batch(orc.KIND_RFWD, n, c, xs, host_threads()), n, f"w2 forward from {s}")
        assert_close_rows(ys, o.batch(orc.KIND_RINV, n, c, Xs, host_threads()), n, f"w2 inverse from {s}")


@pytest.mark.parametrize("l2", list(wl.W3_LOG2))
def test_workload3_vs_oracle_and_round_trip(torch_cuda, ctx_cache, oracle_mod, l2):
    """Single complex transforms of 2^20 / 2^22 / 2^24 points, N(0,1): forward
    and inverse (of the GPU's spectrum) against the oracle, and the round trip."""
    torch = torch_cuda
    n = 1 << l2
    x = wl.complex_normal(n, seed=l2)
    ctx = ctx_cache(n)
    xd = torch.from_numpy(x).cuda()
    X = torch.empty_like(xd)
    y = torch.empty_like(xd)
    ctx.check(ctx.batch("cfwd", n, 1, xd, X))
    ctx.check(ctx.batch("cinv", n, 1, X, y))
    Xh, yh = X.cpu().numpy(), y.cpu().numpy()
    assert rel_l2(yh / n, x) < 5e-6
    o = oracle_mod.Oracle(n)
    assert_close(Xh, o.complex(n, x), n, f"2^{l2} forward")
    assert_close(yh, o.complex(n, Xh, True), n, f"2^{l2} inverse")
