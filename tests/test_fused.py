"""Fused steps around the real transforms: CkFftCudaStft (windowed,
overlapping or zero-padded frames -> real forward x scale) and
CkFftCudaFilterInverse (bins x filter x scale -> real inverse).

Products are rounded one FP32 operation at a time, so each call must equal,
bit for bit, the unfused sequence: the same products formed in numpy FP32,
then the plain batch transform, then the scale.  The oracle checks the
transforms themselves."""
import numpy as np
import pytest

from conftest import assert_close

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def frames_of(signal, frames, hop, frame_len, n, window):
    out = np.zeros((frames, n), np.float32)
    for f in range(frames):
        out[f, :frame_len] = signal[f * hop: f * hop + frame_len]
    if window is not None:
        out = (out * window[None, :]).astype(np.float32)
    return out


STFT_CASES = [
    # n, frames, hop, frame_len, windowed, scale
    (1024, 300, 256, 1024, True, 1.0),
    (1024, 101, 255, 1024, True, 0.5),
    (4096, 40, 4096, 4096, False, 1.0),
    (2048, 64, 700, 1500, True, 1.0 / 3.0),
    (8, 33, 3, 8, True, 2.0),
    (1 << 15, 5, 10000, 1 << 15, True, 1.0),
    (4, 17, 2, 3, True, 0.5),
    (2, 9, 1, 2, False, 1.0),
    (1 << 16, 3, 30000, 50000, True, 0.25),
    (1 << 17, 2, 1 << 17, 1 << 17, False, 1.0),
]


@pytest.mark.parametrize("n,frames,hop,frame_len,windowed,scale", STFT_CASES)
def test_stft_equals_unfused(torch_cuda, ctx_cache, oracle_mod, n, frames, hop, frame_len, windowed, scale):
    torch = torch_cuda
    ctx = ctx_cache(max(n, 8))
    rng = np.random.default_rng(n + frames)
    sig = rng.uniform(-1, 1, (frames - 1) * hop + frame_len).astype(np.float32)
    win = (0.5 - 0.5 * np.cos(2 * np.pi * np.arange(n) / n)).astype(np.float32) if windowed else None
    out = torch.zeros((frames, n // 2 + 1), dtype=torch.complex64, device="cuda")
    ctx.check(ctx.stft(n, frames, torch.from_numpy(sig).cuda(), hop, frame_len,
                       torch.from_numpy(win).cuda() if windowed else None, scale, out))
    rows = frames_of(sig, frames, hop, frame_len, n, win)
    ref = torch.zeros_like(out)
    ctx.check(ctx.batch("rfwd", n, frames, torch.from_numpy(rows).cuda(), ref))
    ref = ref.cpu().numpy()
    want = np.empty_like(ref)                       # each part times the scale, one FP32 rounding
    want.real, want.imag = ref.real * np.float32(scale), ref.imag * np.float32(scale)
    got = out.cpu().numpy()
    assert np.array_equal(bits(got), bits(want))
    o = oracle_mod.Oracle(max(n, 8))
    for f in (0, frames - 1):
        exp = o.real_forward(n, rows[f]) * np.float32(scale)
        if n <= 4:
            assert np.array_equal(bits(got[f]), bits(exp.astype(np.complex64)))
        else:
            assert_close(got[f], exp, n, f"stft n={n} frame {f}")


FILTER_CASES = [(1024, 200, True, 1.0), (4096, 50, True, 1.0 / 8192), (64, 1000, False, 0.5),
                (1 << 15, 4, True, 1.0), (4, 30, True, 1.0), (1 << 17, 2, True, 1.0 / 3.0)]


@pytest.mark.parametrize("n,frames,filtered,scale", FILTER_CASES)
def test_filter_inverse_equals_unfused(torch_cuda, ctx_cache, oracle_mod, n, frames, filtered, scale):
    torch = torch_cuda
    ctx = ctx_cache(max(n, 8))
    bins = n // 2 + 1
    rng = np.random.default_rng(n * 7 + frames)
    X = (rng.uniform(-1, 1, (frames, bins)) + 1j * rng.uniform(-1, 1, (frames, bins))).astype(np.complex64)
    H = (rng.uniform(-1, 1, bins) + 1j * rng.uniform(-1, 1, bins)).astype(np.complex64) if filtered else None
    out = torch.zeros((frames, n), dtype=torch.float32, device="cuda")
    ctx.check(ctx.filter_inverse(n, frames, torch.from_numpy(X).cuda(),
                                 torch.from_numpy(H).cuda() if filtered else None, scale, out))
    # the products in FP32, one rounding per operation
    xr, xi = X.real.astype(np.float32), X.imag.astype(np.float32)
    if filtered:
        hr, hi = H.real.astype(np.float32)[None, :], H.imag.astype(np.float32)[None, :]
        pr = (xr * hr).astype(np.float32) - (xi * hi).astype(np.float32)
        pi = (xr * hi).astype(np.float32) + (xi * hr).astype(np.float32)
    else:
        pr, pi = xr, xi
    s = np.float32(scale)
    prod = np.empty((frames, bins), np.complex64)
    prod.real, prod.imag = (pr * s).astype(np.float32), (pi * s).astype(np.float32)
    ref = torch.zeros_like(out)
    ctx.check(ctx.batch("rinv", n, frames, torch.from_numpy(prod).cuda(), ref))
    got = out.cpu().numpy()
    assert np.array_equal(bits(got), bits(ref.cpu().numpy()))
    o = oracle_mod.Oracle(max(n, 8))
    exp = o.real_inverse(n, prod[frames - 1])
    if n <= 4:
        assert np.array_equal(bits(got[frames - 1]), bits(exp))
    else:
        assert_close(got[frames - 1], exp, n, f"filter n={n}")


def test_fft_convolution_matches_direct(torch_cuda, ctx_cache):
    """Overlap-add convolution built from the two calls equals a direct FP64
    convolution to FP32 accuracy."""
    torch = torch_cuda
    n, L, taps = 1024, 769, 256                    # L + taps - 1 <= n
    ctx = ctx_cache(n)
    rng = np.random.default_rng(11)
    x = rng.standard_normal(L * 40).astype(np.float32)
    h = rng.standard_normal(taps).astype(np.float32)
    hp = np.zeros(n, np.float32)
    hp[:taps] = h
    H = torch.zeros((1, n // 2 + 1), dtype=torch.complex64, device="cuda")
    ctx.check(ctx.stft(n, 1, torch.from_numpy(hp).cuda(), n, n, None, 0.5, H))     # unscaled DFT of h
    frames = len(x) // L
    X = torch.zeros((frames, n // 2 + 1), dtype=torch.complex64, device="cuda")
    ctx.check(ctx.stft(n, frames, torch.from_numpy(x).cuda(), L, L, None, 1.0, X))
    y = torch.zeros((frames, n), dtype=torch.float32, device="cuda")
    ctx.check(ctx.filter_inverse(n, frames, X, H, 1.0 / (2 * n), y))
    y = y.cpu().numpy()
    full = np.zeros(frames * L + n, np.float64)
    for f in range(frames):
        full[f * L: f * L + n] += y[f]
    direct = np.convolve(x.astype(np.float64), h.astype(np.float64))
    m = len(direct)
    err = np.linalg.norm(full[:m] - direct) / np.linalg.norm(direct)
    assert err < 3e-6, err


def test_host_buffers_and_stream(torch_cuda, ctx_cache):
    """Pageable and page-locked host buffers, and an asynchronous stream."""
    torch = torch_cuda
    n, frames, hop = 2048, 50, 512
    ctx = ctx_cache(n)
    rng = np.random.default_rng(3)
    sig = rng.uniform(-1, 1, (frames - 1) * hop + n).astype(np.float32)
    win = np.hanning(n).astype(np.float32)
    dev = torch.zeros((frames, n // 2 + 1), dtype=torch.complex64, device="cuda")
    ctx.check(ctx.stft(n, frames, torch.from_numpy(sig).cuda(), hop, n, torch.from_numpy(win).cuda(), 1.0, dev))
    ref = dev.cpu().numpy()
    host = np.zeros((frames, n // 2 + 1), np.complex64)
    ctx.check(ctx.stft(n, frames, sig, hop, n, win, 1.0, host))
    assert np.array_equal(bits(host), bits(ref))
    pin = torch.zeros((frames, n // 2 + 1), dtype=torch.complex64).pin_memory()
    ctx.check(ctx.stft(n, frames, torch.from_numpy(sig).pin_memory(), hop, n, torch.from_numpy(win).pin_memory(),
                       1.0, pin))
    assert np.array_equal(bits(pin.numpy()), bits(ref))
    s = torch.cuda.Stream()
    out = torch.zeros_like(dev)
    y = torch.zeros((frames, n), dtype=torch.float32, device="cuda")
    sd, wd = torch.from_numpy(sig).cuda(), torch.from_numpy(win).cuda()
    s.wait_stream(torch.cuda.current_stream())
    ctx.check(ctx.stft(n, frames, sd, hop, n, wd, 1.0, out, s))
    ctx.check(ctx.filter_inverse(n, frames, out, None, 1.0, y, s))
    s.synchronize()
    assert np.array_equal(bits(out.cpu().numpy()), bits(ref))


def test_fused_validation(torch_cuda, ctx_cache):
    from ckfft_gb300 import binding
    torch = torch_cuda
    ctx = ctx_cache(1024)
    sig = torch.zeros(1 << 14, device="cuda")
    out = torch.zeros((8, 513), dtype=torch.complex64, device="cuda")
    assert ctx.stft(1024, 8, sig, 256, 1025, None, 1.0, out) == 0          # frame_len > n
    assert ctx.stft(1024, 8, sig, -1, 1024, None, 1.0, out) == 0           # negative hop
    assert ctx.stft(1000, 8, sig, 256, 1000, None, 1.0, out) == 0          # not a power of two
    assert ctx.stft(1024, 0, sig, 256, 1024, None, 1.0, out) == 1          # nothing to do
    odd = out.view(torch.float32).view(-1)[1:]
    assert ctx.stft(1024, 1, sig, 256, 1024, None, 1.0, odd) == 0          # misaligned output
    assert "aligned" in binding.last_error()
    v = sig.view(torch.complex64)
    assert ctx.stft(1024, 2, sig, 256, 1024, None, 1.0, v[100:]) == 0      # output overlaps signal
    assert "overlap" in binding.last_error()
    y = torch.zeros((8, 1024), device="cuda")
    assert ctx.filter_inverse(1024, 8, out, None, 1.0, y) == 1
    assert ctx.filter_inverse(1024, 8, y.view(torch.complex64), None, 1.0, y) == 0
    fwd_only = binding.Context(1024, binding.FORWARD) if hasattr(binding, "FORWARD") else binding.Context(1024, 1)
    assert fwd_only.filter_inverse(1024, 1, out, None, 1.0, y) == 0
    fwd_only.close()
