"""CkFftCudaComplexBatchNoAlloc: the complex batch entry point for callers that
cannot allocate while they run (real-time callbacks that must not wait on
cudaMalloc/cudaFree, hosts with a fixed memory budget or their own device
allocator).  It must give the same results as the regular batch entry point
while keeping its multi-pass intermediate in the library's fixed 8 MiB device
array, and it must not allocate: free device memory stays the same across
calls, and an injected failure of the library's next allocation does not
touch it.  Collected last so that a failure here never hides the other tests."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, assert_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(lib):
    from ckfft_gb300 import binding

    c = binding.Context(1 << 21)
    yield c
    c.close()


def no_alloc(lib, ctx, n, count, inverse, x, y, stream=None):
    s = getattr(stream, "cuda_stream", stream)
    return lib.CkFftCudaComplexBatchNoAlloc(ctx.handle, n, count, int(inverse), x.data_ptr(), y.data_ptr(), s)


@pytest.mark.parametrize("l2,count", [(10, 3), (16, 3), (20, 2)])
@pytest.mark.parametrize("inverse", [False, True])
def test_matches_regular_batch_twice(torch_cuda, lib, ctx, l2, count, inverse):
    torch = torch_cuda
    n = 1 << l2
    rng = np.random.default_rng(l2 * 2 + int(inverse))
    x = (rng.standard_normal((count, n)) + 1j * rng.standard_normal((count, n))).astype(np.complex64)
    xd = torch.from_numpy(x).cuda()
    ref = torch.empty_like(xd)
    ctx.check(ctx.batch("cinv" if inverse else "cfwd", n, count, xd, ref), "regular batch")
    ref = ref.cpu().numpy()
    stream = torch.cuda.Stream()
    for call in range(2):                      # two calls in a row share the scratch array
        y = torch.full_like(xd, float("nan"))
        if call:
            # the NaN fill runs on torch's current stream: order the call after it
            stream.wait_stream(torch.cuda.current_stream())
        rc = no_alloc(lib, ctx, n, count, inverse, xd, y, stream if call else None)
        if call:
            stream.synchronize()
        assert rc == 1, ctx.lib.CkFftCudaGetLastError()
        got = y.cpu().numpy()
        for f in range(count):
            assert_close(got[f], ref[f], n, f"no-alloc call {call} n=2^{l2} frame {f}")


def test_free_memory_unchanged(torch_cuda, lib, ctx):
    """After one call per size, further calls leave the device's free memory as it was."""
    torch = torch_cuda
    bufs = {}
    for l2, count in ((10, 8), (16, 4), (20, 2)):
        n = 1 << l2
        x = torch.randn((count, n), dtype=torch.complex64, device="cuda")
        bufs[l2] = (n, count, x, torch.empty_like(x))
    for n, count, x, y in bufs.values():                    # first call of each size
        assert no_alloc(lib, ctx, n, count, False, x, y) == 1, lib.CkFftCudaGetLastError()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        for n, count, x, y in bufs.values():
            assert no_alloc(lib, ctx, n, count, False, x, y) == 1
            assert no_alloc(lib, ctx, n, count, True, y, x) == 1
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"free device memory moved by {free0 - free1} bytes"


CHILD = r"""
import sys
import numpy as np
import torch
sys.path.insert(0, ROOT)
from ckfft_gb300 import binding
lib = binding.load()
x = {l2: torch.randn((2, 1 << l2), dtype=torch.complex64, device="cuda") for l2 in (16, 20)}
y = {l2: torch.zeros_like(v) for l2, v in x.items()}
ctx = binding.Context(1 << 20)             # allocation 1: the twiddle table
for rep in range(2):                        # the library's allocation 2 is set to fail
    for l2 in (16, 20):
        rc = lib.CkFftCudaComplexBatchNoAlloc(ctx.handle, 1 << l2, 2, 0, x[l2].data_ptr(), y[l2].data_ptr(), None)
        assert rc == 1, binding.last_error()
torch.cuda.synchronize()
for l2 in (16, 20):
    ref = torch.fft.fft(x[l2].to(torch.complex128))
    err = (torch.linalg.norm(y[l2].to(torch.complex128) - ref) / torch.linalg.norm(ref)).item()
    assert err < 1e-5, (l2, err)
# the regular batch at 2^16 needs scratch: its allocation is the one that fails
z = torch.zeros_like(x[16])
assert ctx.batch("cfwd", 1 << 16, 2, x[16], z) == 0, "the injected failure was not reached"
assert "scratch" in binding.last_error(), binding.last_error()
print("ok")
"""


def test_injected_allocation_failure_is_never_reached(torch_cuda):
    """With the library's second allocation set to fail (the first one after
    the context exists), no-allocation calls at 2^16 and 2^20 still succeed;
    the regular batch then takes the injected failure."""
    env = dict(os.environ, CKFFT_CUDA_FAIL_ALLOC="2")
    r = subprocess.run([sys.executable, "-c", f"ROOT = {ROOT!r}\n" + CHILD], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0 and "ok" in r.stdout, r.stdout + r.stderr


def test_rejects_what_it_cannot_do_without_allocating(torch_cuda, lib, ctx):
    torch = torch_cuda
    n = 1 << 21
    xd = torch.zeros(n, dtype=torch.complex64, device="cuda")
    yd = torch.zeros(n, dtype=torch.complex64, device="cuda")
    assert no_alloc(lib, ctx, n, 1, False, xd, yd) == 0
    assert "2^20" in lib.CkFftCudaGetLastError().decode()
    xh = torch.zeros(1024, dtype=torch.complex64)
    yh = torch.zeros(1024, dtype=torch.complex64)
    assert no_alloc(lib, ctx, 1024, 1, False, xh, yh) == 0
    assert "device" in lib.CkFftCudaGetLastError().decode()
    assert no_alloc(lib, ctx, 1024, 1, False, xd, xd) == 0
    assert no_alloc(lib, ctx, 1000, 1, False, xd, yd) == 0
    assert no_alloc(lib, ctx, 1024, 0, False, xd, yd) == 1
