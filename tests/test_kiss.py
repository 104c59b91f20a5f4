"""The kiss_fft-compatible boundary (include/kiss_fft_cuda.h) on the GPU.

Against kiss_fft 1.3.0's own outputs (tests/golden/kiss_golden.npz, made by
tests/golden/make_kiss_golden.py from the reference tree's ext/kiss_fft130)
within the parity tolerance, and bit for bit against this library's ckfft
calls in kiss scaling (complex unchanged, real forward halved, real inverse
unchanged).  Host (pageable, page-locked) and device buffers, fin == fout,
strided input, misaligned bins and the alloc protocol."""
import ctypes as C

import numpy as np
import pytest

from conftest import assert_close

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module")
def klib(lib):
    return lib


def addr(a):
    return a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data


def kiss_c(klib, n, x, inverse=False, where="host"):
    cfg = klib.kiss_fft_alloc(n, int(inverse), None, None)
    assert cfg
    try:
        return run_buf(klib.kiss_fft, cfg, x, np.zeros(n, np.complex64), where)
    finally:
        klib.kiss_fft_free(cfg)


def run_buf(fn, cfg, x, out, where, torch=None):
    if where == "host":
        fn(cfg, addr(x), addr(out))
        return out
    import torch as T
    if where == "pinned":
        xi, yo = T.from_numpy(x).pin_memory(), T.from_numpy(out).pin_memory()
    else:
        xi, yo = T.from_numpy(x).cuda(), T.from_numpy(out).cuda()
    fn(cfg, xi.data_ptr(), yo.data_ptr())
    return yo.cpu().numpy()


@pytest.mark.parametrize("where", ["host", "pinned", "device"])
def test_complex_vs_kiss_golden(torch_cuda, klib, kiss_golden, ctx_cache, where):
    for l2 in range(0, 12):
        n = 1 << l2
        x = kiss_golden[f"cin_{l2}"]
        for inv, name in ((False, "cfwd"), (True, "cinv")):
            got = kiss_c(klib, n, x, inv, where)
            want = kiss_golden[f"{name}_{l2}"]
            if n <= 2:
                assert np.array_equal(bits(got), bits(want)), (name, n)
            else:
                assert_close(got, want, n, f"kiss {name} n={n}")
            # the same bits as the ckfft entry points of this library
            ctx = ctx_cache(max(n, 8))
            ref = np.zeros(n, np.complex64)
            ctx.check(ctx.batch("cinv" if inv else "cfwd", n, 1, x, ref))
            assert np.array_equal(bits(got), bits(ref))


@pytest.mark.parametrize("where", ["host", "pinned", "device"])
def test_real_vs_kiss_golden(torch_cuda, klib, kiss_golden, ctx_cache, where):
    for l2 in range(1, 12):
        n = 1 << l2
        r = kiss_golden[f"rin_{l2}"]
        cfg = klib.kiss_fftr_alloc(n, 0, None, None)
        X = run_buf(klib.kiss_fftr, cfg, r, np.zeros(n // 2 + 1, np.complex64), where)
        klib.kiss_fftr_free(cfg)
        assert_close(X, kiss_golden[f"rfwd_{l2}"], n, f"kiss_fftr n={n}")
        ctx = ctx_cache(max(n, 8))
        ref = np.zeros(n // 2 + 1, np.complex64)
        ctx.check(ctx.batch("rfwd", n, 1, r, ref))
        half = np.empty_like(ref)
        half.real, half.imag = ref.real * np.float32(0.5), ref.imag * np.float32(0.5)
        assert np.array_equal(bits(X), bits(half)), n
        cfg = klib.kiss_fftr_alloc(n, 1, None, None)
        Xg = kiss_golden[f"rfwd_{l2}"]
        y = run_buf(klib.kiss_fftri, cfg, Xg, np.zeros(n, np.float32), where)
        klib.kiss_fftr_free(cfg)
        assert_close(y, kiss_golden[f"rinv_{l2}"], n, f"kiss_fftri n={n}")
        ref = np.zeros(n, np.float32)
        ctx.check(ctx.batch("rinv", n, 1, Xg, ref))
        assert np.array_equal(bits(y), bits(ref)), n


def test_in_place_stride_and_alignment(torch_cuda, klib, kiss_golden):
    torch = torch_cuda
    n, l2 = 2048, 11
    x = kiss_golden[f"cin_{l2}"]
    want = kiss_c(klib, n, x)
    cfg = klib.kiss_fft_alloc(n, 0, None, None)
    buf = x.copy()                                   # fin == fout, host
    klib.kiss_fft(cfg, addr(buf), addr(buf))
    assert np.array_equal(bits(buf), bits(want))
    d = torch.from_numpy(x).cuda()                   # fin == fout, device
    klib.kiss_fft(cfg, d.data_ptr(), d.data_ptr())
    assert np.array_equal(bits(d.cpu().numpy()), bits(want))
    wide = np.zeros(3 * n, np.complex64)             # every third element
    wide[::3] = x
    out = np.zeros(n, np.complex64)
    klib.kiss_fft_stride(cfg, addr(wide), addr(out), 3)
    assert np.array_equal(bits(out), bits(want))
    klib.kiss_fft_free(cfg)
    # bins at a 4-byte (not 8-byte) aligned address
    r = kiss_golden["rin_11"]
    cfg = klib.kiss_fftr_alloc(n, 0, None, None)
    ref = np.zeros(n // 2 + 1, np.complex64)
    klib.kiss_fftr(cfg, addr(r), addr(ref))
    raw = np.zeros(2 * (n // 2 + 1) + 1, np.float32)
    klib.kiss_fftr(cfg, addr(r), raw.ctypes.data + 4)
    assert np.array_equal(raw[1:].view(np.uint32), bits(ref))
    klib.kiss_fftr_free(cfg)


def test_alloc_protocol_and_errors(torch_cuda, klib):
    from ckfft_gb300 import binding
    need = C.c_size_t(0)
    assert klib.kiss_fft_alloc(256, 0, None, C.byref(need)) is None and need.value > 0
    mem = (C.c_char * need.value)()
    have = C.c_size_t(need.value)
    cfg = klib.kiss_fft_alloc(256, 0, C.addressof(mem), C.byref(have))
    assert cfg == C.addressof(mem) and have.value == need.value
    x = np.ones(256, np.complex64)
    y = np.zeros(256, np.complex64)
    klib.kiss_fft(cfg, addr(x), addr(y))
    assert y[0] == 256 and np.all(y[1:] == 0)
    klib.kiss_fft_free(cfg)                          # releases the GPU side, not `mem`
    rcfg = klib.kiss_fftr_alloc(256, 1, None, None)
    klib.kiss_fftr(rcfg, addr(np.zeros(256, np.float32)), addr(y))
    assert "inverse" in binding.last_error()
    klib.kiss_fftr_free(rcfg)
    assert klib.kiss_fft_alloc(768, 0, None, None) is None
