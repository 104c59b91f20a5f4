"""CkFftCudaComplexBatchNoAlloc: the complex batch entry point for callers that
cannot allocate while they run (real-time callbacks that must not wait on
cudaMalloc/cudaFree, hosts with a fixed memory budget or their own device
allocator).  It must give the same results as the regular batch entry point
while keeping its multi-pass intermediate in the library's fixed 8 MiB device
array.  Collected last so that a failure here never hides the other tests."""
import numpy as np
import pytest

from conftest import assert_close

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
        rc = no_alloc(lib, ctx, n, count, inverse, xd, y, stream if call else None)
        if call:
            stream.synchronize()
        assert rc == 1, ctx.lib.CkFftCudaGetLastError()
        got = y.cpu().numpy()
        for f in range(count):
            assert_close(got[f], ref[f], n, f"no-alloc call {call} n=2^{l2} frame {f}")


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
