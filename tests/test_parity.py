"""GPU parity: the CUDA path through the C ABI against the reference's own
outputs (golden fixtures) and the oracle (bit-identical to the reference).

Bar (conftest.assert_close): relative L2 <= 1e-5 and max element error
<= 2e-6 * log2 n of the reference's rms; closed-form sizes are bit-exact.
"""
import ctypes as C
import os
import pathlib
import subprocess
import sys
import threading

import numpy as np
import pytest

from conftest import assert_close, rel_l2

pytestmark = pytest.mark.gpu

OUT_SHAPE = {
    "cfwd": lambda n: (n, np.complex64),
    "cinv": lambda n: (n, np.complex64),
    "rfwd": lambda n: (n // 2 + 1, np.complex64),
    "rinv": lambda n: (n, np.float32),
}


def run_batch(torch, ctx, kind, n, x, count=None, where="device", stream=None):
    """Runs one batch through CkFftCuda*Batch with inputs in `where` memory."""
    x = np.ascontiguousarray(x)
    if count is None:
        count = x.shape[0] if x.ndim > 1 else 1
    m, dt = OUT_SHAPE[kind](n)
    if where == "device":
        xt = torch.from_numpy(x).cuda()
        out = torch.zeros((count, m), dtype=torch.complex64 if dt == np.complex64 else torch.float32,
                          device="cuda")
        rc = ctx.batch(kind, n, count, xt, out, stream)
        if stream is not None:
            stream.synchronize()
        ctx.check(rc, f"{kind} n={n}")
        return out.cpu().numpy()
    if where == "pinned":
        xt = torch.from_numpy(x).pin_memory()
        out = torch.zeros((count, m), dtype=torch.complex64 if dt == np.complex64 else torch.float32).pin_memory()
        ctx.check(ctx.batch(kind, n, count, xt, out), f"{kind} n={n}")
        return out.numpy()
    out = np.zeros((count, m), dt)
    ctx.check(ctx.batch(kind, n, count, x, out), f"{kind} n={n}")
    return out


def run_single(torch, ctx, kind, n, x, where="device"):
    """One transform through the reference-named entry points."""
    m, dt = OUT_SHAPE[kind](n)
    x = np.ascontiguousarray(x)
    if where == "device":
        xt = torch.from_numpy(x).cuda()
        out = torch.zeros(m, dtype=torch.complex64 if dt == np.complex64 else torch.float32, device="cuda")
        tmp = torch.zeros(n // 2 + 1, dtype=torch.complex64, device="cuda")
    else:
        xt, out, tmp = x, np.zeros(m, dt), np.zeros(n // 2 + 1, np.complex64)
    if kind == "cfwd":
        rc = ctx.complex_forward(n, xt, out)
    elif kind == "cinv":
        rc = ctx.complex_inverse(n, xt, out)
    elif kind == "rfwd":
        rc = ctx.real_forward(n, xt, out)
    else:
        rc = ctx.real_inverse(n, xt, out, tmp)
    ctx.check(rc, f"{kind} n={n}")
    return out.cpu().numpy() if where == "device" else out


def bits_equal(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


# ------------------------------------------------------------ golden vectors

def test_golden_matrix(torch_cuda, ctx_cache, golden):
    """The reference regression matrix on src/test/input.txt (test.cpp:866-921)."""
    x = golden["input_txt"]
    n = 4096
    while n >= 1:
        for nmax in (n, 8192):
            ctx = ctx_cache(nmax)
            sfx = f"{n}_{nmax}" if f"c_fwd_{n}_{nmax}" in golden.files else f"{n}_{n}"
            xr = x[:n].real.copy()
            cases = {
                "cfwd": (x[:n], golden[f"c_fwd_{sfx}"]),
                "cinv": (x[:n], golden[f"c_inv_{sfx}"]),
                "rfwd": (xr, golden[f"r_fwd_{sfx}"]),
                "rinv": (golden[f"r_fwd_{sfx}"], golden[f"r_rt_{sfx}"]),
            }
            for kind, (inp, ref) in cases.items():
                got = run_single(torch_cuda, ctx, kind, n, inp)
                exact = n <= (4 if kind in ("rfwd", "rinv") else 2)
                if exact:
                    assert bits_equal(got, ref), (kind, n, nmax)
                else:
                    assert_close(got, ref, n, f"{kind} n={n} nmax={nmax}")
            # the reference test's real inverse input: first n/2+1 complex bins
            cf = run_single(torch_cuda, ctx, "cfwd", n, xr.astype(np.complex64))
            got = run_single(torch_cuda, ctx, "rinv", n, cf[: n // 2 + 1])
            assert_close(got, golden[f"r_inv_{sfx}"], n, f"rinv(cfwd) n={n}")
        n //= 2


def test_golden_workloads(torch_cuda, ctx_cache, golden):
    ctx = ctx_cache(1 << 13)
    got = run_batch(torch_cuda, ctx, "cfwd", 1024, golden["w1_in"])
    assert_close(got, golden["w1_fwd"], 1024, "w1 fwd")
    got = run_batch(torch_cuda, ctx, "cinv", 1024, golden["w1_fwd"])
    assert_close(got, golden["w1_rt"], 1024, "w1 inv")
    got = run_batch(torch_cuda, ctx, "rfwd", 4096, golden["w2_in"])
    assert_close(got, golden["w2_fwd"], 4096, "w2 fwd")
    got = run_batch(torch_cuda, ctx, "rinv", 4096, golden["w2_fwd"])
    assert_close(got, golden["w2_rt"], 4096, "w2 inv")
    for l2 in range(6, 14):
        n = 1 << l2
        assert_close(run_single(torch_cuda, ctx, "cfwd", n, golden[f"w4_cin_{l2}"]), golden[f"w4_cfwd_{l2}"], n)
        assert_close(run_single(torch_cuda, ctx, "cinv", n, golden[f"w4_cin_{l2}"]), golden[f"w4_cinv_{l2}"], n)
        assert_close(run_single(torch_cuda, ctx, "rfwd", n, golden[f"w4_rin_{l2}"]), golden[f"w4_rfwd_{l2}"], n)
        assert_close(run_single(torch_cuda, ctx, "rinv", n, golden[f"w4_hin_{l2}"]), golden[f"w4_rinv_{l2}"], n)


def test_example_round_trip(torch_cuda, ctx_cache, golden):
    """src/example/main.cpp:55-76 with host buffers, as the example does."""
    ctx = ctx_cache(1024)
    x = golden["example_input"]
    fwd = run_single(torch_cuda, ctx, "rfwd", 1024, x, where="host")
    assert_close(fwd, golden["example_fwd"], 1024, "example fwd")
    y = run_single(torch_cuda, ctx, "rinv", 1024, fwd, where="host")
    assert_close(y, golden["example_rt"], 1024, "example rt")
    assert float(np.sum((y / 2048.0 - x) ** 2)) < 1e-8


# ------------------------------------------------------------ every size

@pytest.mark.parametrize("l2", list(range(0, 21)))
def test_complex_sizes_vs_oracle(torch_cuda, ctx_cache, oracle_mod, l2):
    n = 1 << l2
    frames = 3 if l2 <= 16 else 1
    rng = np.random.default_rng(100 + l2)
    x = (rng.uniform(-1, 1, (frames, n)) + 1j * rng.uniform(-1, 1, (frames, n))).astype(np.complex64)
    o = oracle_mod.Oracle(n)
    ctx = ctx_cache(n)
    for kind, inv in (("cfwd", False), ("cinv", True)):
        got = run_batch(torch_cuda, ctx, kind, n, x)
        for f in range(frames):
            ref = o.complex(n, x[f], inv)
            if n <= 2:
                assert bits_equal(got[f], ref), (kind, n)
            else:
                assert_close(got[f], ref, n, f"{kind} n=2^{l2} frame {f}")


@pytest.mark.parametrize("l2", list(range(0, 22)))
def test_real_sizes_vs_oracle(torch_cuda, ctx_cache, oracle_mod, l2):
    n = 1 << l2
    frames = 3 if l2 <= 17 else 1
    rng = np.random.default_rng(200 + l2)
    x = rng.uniform(-1, 1, (frames, n)).astype(np.float32)
    h = (rng.uniform(-1, 1, (frames, n // 2 + 1)) + 1j * rng.uniform(-1, 1, (frames, n // 2 + 1))).astype(np.complex64)
    o = oracle_mod.Oracle(n)
    ctx = ctx_cache(n)
    got_f = run_batch(torch_cuda, ctx, "rfwd", n, x)
    got_i = run_batch(torch_cuda, ctx, "rinv", n, h)
    for f in range(frames):
        rf, ri = o.real_forward(n, x[f]), o.real_inverse(n, h[f])
        if n <= 4:
            assert bits_equal(got_f[f], rf) and bits_equal(got_i[f], ri), n
        else:
            assert_close(got_f[f], rf, n, f"rfwd n=2^{l2}")
            assert_close(got_i[f], ri, n, f"rinv n=2^{l2}")


@pytest.mark.parametrize("l2", [21, 22, 23, 24])
def test_large_complex_vs_oracle_and_fp64(torch_cuda, ctx_cache, oracle_mod, l2):
    """Workload 3 sizes (and the three-pass sizes between): N(0,1) inputs,
    forward and inverse."""
    n = 1 << l2
    rng = np.random.default_rng(300 + l2)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    o = oracle_mod.Oracle(n)
    ctx = ctx_cache(n)
    for kind, inv in (("cfwd", False), ("cinv", True)):
        got = run_batch(torch_cuda, ctx, kind, n, x[None])[0]
        assert_close(got, o.complex(n, x, inv), n, f"{kind} 2^{l2}")
        assert rel_l2(got, oracle_mod.fp64_complex(x, inv)) < 2e-6


@pytest.mark.parametrize("kind,l2,count", [("cfwd", 21, 3), ("cinv", 22, 2), ("rfwd", 22, 2), ("rinv", 23, 2),
                                            ("rfwd", 18, 3), ("rfwd", 20, 3), ("rfwd", 21, 2),
                                            ("rinv", 18, 3), ("rinv", 20, 3), ("rinv", 21, 2),
                                            ("rfwd", 23, 2), ("rinv", 22, 2), ("cfwd", 20, 3), ("cinv", 19, 4)])
def test_three_pass_batches(torch_cuda, ctx_cache, oracle_mod, kind, l2, count):
    """Batches on the multi-pass paths (three passes; two passes with the
    real split fused into the row pass or the merge into the column pass):
    every transform against the oracle."""
    n = 1 << l2
    rng = np.random.default_rng(400 + l2)
    m = n // 2 + 1 if kind == "rinv" else n
    if kind == "rfwd":
        x = rng.standard_normal((count, n)).astype(np.float32)
    else:
        x = (rng.standard_normal((count, m)) + 1j * rng.standard_normal((count, m))).astype(np.complex64)
    o = oracle_mod.Oracle(n)
    ctx = ctx_cache(n)
    got = run_batch(torch_cuda, ctx, kind, n, x)
    for f in range(count):
        if kind == "rfwd":
            ref = o.real_forward(n, x[f])
        elif kind == "rinv":
            ref = o.real_inverse(n, x[f])
        else:
            ref = o.complex(n, x[f], kind == "cinv")
        assert_close(got[f], ref, n, f"{kind} 2^{l2} frame {f}")


# ------------------------------------------------- pipelined kernels + tails

def small_tpb(l2):
    """Frames per CTA group of the single-CTA kernels (SmallCfg in fft_small.cuh)."""
    r = l2 if l2 < 4 else (4 if l2 < 14 else 5)
    t = (1 << l2) >> r
    return 1 if t >= 256 else 256 // t


@pytest.mark.parametrize("l2", list(range(6, 15)))
def test_group_pipeline_with_tail(torch_cuda, ctx_cache, oracle_mod, l2):
    """3 whole frame groups (bulk-copy pipelined kernel) plus one extra frame (plain kernel)."""
    n = 1 << l2
    ctx = ctx_cache(2 * n)
    o = oracle_mod.Oracle(2 * n)
    rng = np.random.default_rng(500 + l2)
    frames = 3 * small_tpb(l2) + 1
    x = (rng.uniform(-1, 1, (frames, n)) + 1j * rng.uniform(-1, 1, (frames, n))).astype(np.complex64)
    xr = rng.uniform(-1, 1, (frames, 2 * n)).astype(np.float32)
    h = (rng.uniform(-1, 1, (frames, n + 1)) + 1j * rng.uniform(-1, 1, (frames, n + 1))).astype(np.complex64)
    got = {k: run_batch(torch_cuda, ctx, k, n, x) for k in ("cfwd", "cinv")}
    got["rfwd"] = run_batch(torch_cuda, ctx, "rfwd", 2 * n, xr)
    got["rinv"] = run_batch(torch_cuda, ctx, "rinv", 2 * n, h)
    for f in sorted({0, 1, frames // 2, frames - 2, frames - 1}):
        assert_close(got["cfwd"][f], o.complex(n, x[f], False), n, f"cfwd 2^{l2} frame {f}")
        assert_close(got["cinv"][f], o.complex(n, x[f], True), n, f"cinv 2^{l2} frame {f}")
        assert_close(got["rfwd"][f], o.real_forward(2 * n, xr[f]), 2 * n, f"rfwd 2^{l2 + 1} frame {f}")
        assert_close(got["rinv"][f], o.real_inverse(2 * n, h[f]), 2 * n, f"rinv 2^{l2 + 1} frame {f}")


def test_misaligned_input_takes_plain_path(torch_cuda, ctx_cache, oracle_mod):
    """An input 8 bytes off a 16-byte boundary cannot be bulk-copied; results stay right."""
    n, frames = 1024, 9
    ctx = ctx_cache(n)
    rng = np.random.default_rng(77)
    x = (rng.uniform(-1, 1, (frames, n)) + 1j * rng.uniform(-1, 1, (frames, n))).astype(np.complex64)
    buf = torch_cuda.zeros(frames * n + 1, dtype=torch_cuda.complex64, device="cuda")
    buf[1:] = torch_cuda.from_numpy(x.reshape(-1)).cuda()
    xin = buf[1:]
    assert xin.data_ptr() % 16 == 8
    out = torch_cuda.zeros((frames, n), dtype=torch_cuda.complex64, device="cuda")
    ctx.check(ctx.batch("cfwd", n, frames, xin, out))
    got = out.cpu().numpy()
    o = oracle_mod.Oracle(n)
    for f in (0, 4, 8):
        assert_close(got[f], o.complex(n, x[f]), n, f"frame {f}")


# ------------------------------------------------------------ memory kinds

@pytest.mark.parametrize("kind,n", [("cfwd", 64), ("cinv", 4096), ("rfwd", 4096), ("rinv", 2048),
                                    ("cfwd", 1 << 16), ("rinv", 1 << 17), ("rfwd", 4)])
def test_memory_kinds_agree(torch_cuda, ctx_cache, kind, n):
    """Device (blocking and stream-async), pageable host and pinned host give identical bits."""
    ctx = ctx_cache(max(n, 8))
    rng = np.random.default_rng(n)
    frames = 5
    if kind == "rfwd":
        x = rng.uniform(-1, 1, (frames, n)).astype(np.float32)
    else:
        m = n // 2 + 1 if kind == "rinv" else n
        x = (rng.uniform(-1, 1, (frames, m)) + 1j * rng.uniform(-1, 1, (frames, m))).astype(np.complex64)
    ref = run_batch(torch_cuda, ctx, kind, n, x, where="device")
    s = torch_cuda.cuda.Stream()
    assert bits_equal(run_batch(torch_cuda, ctx, kind, n, x, where="device", stream=s), ref)
    assert bits_equal(run_batch(torch_cuda, ctx, kind, n, x, where="host"), ref)
    assert bits_equal(run_batch(torch_cuda, ctx, kind, n, x, where="pinned"), ref)
    single = run_single(torch_cuda, ctx, kind, n, x[2], where="host")
    assert bits_equal(single, ref[2])


def test_staged_batch_spans_chunks(torch_cuda, ctx_cache):
    """A host batch larger than one 64 MiB staging chunk equals the device result."""
    n, frames = 4096, 2600                 # 83 MB of complex input
    ctx = ctx_cache(n)
    rng = np.random.default_rng(9)
    x = (rng.uniform(-1, 1, (frames, n)) + 1j * rng.uniform(-1, 1, (frames, n))).astype(np.complex64)
    ref = run_batch(torch_cuda, ctx, "cfwd", n, x, where="device")
    assert bits_equal(run_batch(torch_cuda, ctx, "cfwd", n, x, where="pinned"), ref)
    assert bits_equal(run_batch(torch_cuda, ctx, "cfwd", n, x, where="host"), ref)


@pytest.mark.parametrize("kind", ["cfwd", "rfwd", "rinv"])
def test_pinned_batch_runs_in_place(torch_cuda, ctx_cache, lib, kind):
    """Page-locked host buffers of a single-CTA size are read and written by
    one launch in place (no staging chunks), alone or mixed with device
    buffers, with the bits of the all-device run."""
    torch = torch_cuda
    n, frames = 4096, 2600                 # more than one 64 MiB staging chunk
    ctx = ctx_cache(n)
    rng = np.random.default_rng(19)
    if kind == "rfwd":
        x = rng.uniform(-1, 1, (frames, n)).astype(np.float32)
    else:
        m = n // 2 + 1 if kind == "rinv" else n
        x = (rng.uniform(-1, 1, (frames, m)) + 1j * rng.uniform(-1, 1, (frames, m))).astype(np.complex64)
    ref = run_batch(torch, ctx, kind, n, x, where="device")
    m, dt = OUT_SHAPE[kind](n)
    tdt = torch.complex64 if dt == np.complex64 else torch.float32
    xh = torch.from_numpy(x).pin_memory()
    xd = xh.cuda()
    for src in (xh, xd):
        for dst_dev in (False, True):
            if src is xd and dst_dev:
                continue
            out = torch.zeros((frames, m), dtype=tdt, device="cuda" if dst_dev else "cpu")
            if not dst_dev:
                out = out.pin_memory()
            before = lib.CkFftCudaLaunchCount()
            ctx.check(ctx.batch(kind, n, frames, src, out))
            assert lib.CkFftCudaLaunchCount() - before == 1
            assert bits_equal(out.cpu().numpy(), ref)


def test_zero_copy_switch_stages_pinned(torch_cuda):
    """CKFFT_CUDA_ZERO_COPY=0 moves pinned buffers through the staging chunks
    (several launches) and gives the same bits."""
    code = r"""
import numpy as np, torch
from ckfft_gb300 import binding
lib = binding.load()
ctx = binding.Context(4096)
rng = np.random.default_rng(19)
x = (rng.uniform(-1, 1, (2600, 4096)) + 1j * rng.uniform(-1, 1, (2600, 4096))).astype(np.complex64)
xh = torch.from_numpy(x).pin_memory()
yh = torch.zeros_like(xh).pin_memory()
yd = torch.zeros((2600, 4096), dtype=torch.complex64, device="cuda")
ctx.check(ctx.batch("cfwd", 4096, 2600, xh.cuda(), yd))
before = lib.CkFftCudaLaunchCount()
ctx.check(ctx.batch("cfwd", 4096, 2600, xh, yh))
assert lib.CkFftCudaLaunchCount() - before >= 2
assert np.array_equal(yh.numpy().view(np.uint32), yd.cpu().numpy().view(np.uint32))
print("ok")
"""
    env = dict(os.environ, CKFFT_CUDA_ZERO_COPY="0")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600,
                       cwd=str(pathlib.Path(__file__).resolve().parents[1]))
    assert r.returncode == 0 and "ok" in r.stdout, r.stdout + r.stderr


def test_zero_count_is_noop(torch_cuda, ctx_cache):
    ctx = ctx_cache(64)
    a = torch_cuda.zeros(64, dtype=torch_cuda.complex64, device="cuda")
    b = torch_cuda.ones(64, dtype=torch_cuda.complex64, device="cuda")
    assert ctx.batch("cfwd", 64, 0, a, b) == 1
    assert torch_cuda.all(b == 1)
    assert ctx.batch("cfwd", 64, -1, a, b) == 0


# ------------------------------------------------------------ API contract

def test_argument_checks_with_context(torch_cuda, lib, ctx_cache):
    """src/ckfft/ckfft.cpp:38-110 return codes on a live context."""
    ctx = ctx_cache(64)
    a = torch_cuda.zeros(256, dtype=torch_cuda.complex64, device="cuda")
    b = torch_cuda.zeros(256, dtype=torch_cuda.complex64, device="cuda")
    t = torch_cuda.zeros(256, dtype=torch_cuda.complex64, device="cuda")
    for n in (0, -1, -(2 ** 31), 3, 48, 128):
        assert ctx.complex_forward(n, a, b) == 0, n
        assert ctx.real_forward(n, a, b) == 0, n
        assert ctx.real_inverse(n, a, b, t) == 0, n
    assert ctx.complex_forward(64, a, a) == 0
    assert ctx.complex_forward(64, None, b) == 0
    assert ctx.complex_forward(64, a, None) == 0
    assert ctx.real_inverse(64, a, b, None) == 0
    assert ctx.complex_forward(64, a, b) == 1
    from ckfft_gb300 import binding

    fwd_only = binding.Context(64, binding.FORWARD)
    assert fwd_only.complex_forward(64, a, b) == 1
    assert fwd_only.complex_inverse(64, a, b) == 0
    assert fwd_only.real_inverse(64, a, b, t) == 0
    fwd_only.close()
    inv_only = binding.Context(64, binding.INVERSE)
    assert inv_only.complex_forward(64, a, b) == 0
    assert inv_only.real_forward(64, a, b) == 0
    assert inv_only.complex_inverse(64, a, b) == 1
    inv_only.close()


def test_user_buffer_context(torch_cuda, lib):
    """context.cpp:68-88,132: size query, caller memory, Shutdown leaves it alone."""
    size = C.c_size_t(0)
    assert not lib.CkFftInit(1024, 3, None, C.byref(size))
    buf = (C.c_char * size.value)()
    h = lib.CkFftInit(1024, 3, buf, C.byref(size))
    assert h == C.addressof(buf)
    x = np.ones(1024, np.complex64)
    y = np.zeros(1024, np.complex64)
    assert lib.CkFftComplexForward(h, 1024, x.ctypes.data, y.ctypes.data) == 1
    assert abs(y[0] - 1024) < 1e-3 and np.max(np.abs(y[1:])) < 1e-3
    lib.CkFftShutdown(h)


def test_threads_share_one_context(torch_cuda, ctx_cache, oracle_mod):
    """Contexts are usable from many threads at once (inc/ckfft/ckfft.h:39-41)."""
    n = 2048
    ctx = ctx_cache(n)
    rng = np.random.default_rng(3)
    xs = [(rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64) for _ in range(8)]
    refs = [run_single(torch_cuda, ctx, "cfwd", n, x, where="host") for x in xs]
    errors = []

    def worker(i):
        try:
            for _ in range(20):
                got = run_single(torch_cuda, ctx, "cfwd", n, xs[i], where="host")
                if not bits_equal(got, refs[i]):
                    errors.append(i)
        except Exception as e:  # noqa: BLE001
            errors.append(repr(e))

    th = [threading.Thread(target=worker, args=(i,)) for i in range(8)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors


def test_deterministic(torch_cuda, ctx_cache):
    n = 1 << 16
    ctx = ctx_cache(n)
    rng = np.random.default_rng(1)
    x = (rng.uniform(-1, 1, (2, n)) + 1j * rng.uniform(-1, 1, (2, n))).astype(np.complex64)
    a = run_batch(torch_cuda, ctx, "cfwd", n, x)
    b = run_batch(torch_cuda, ctx, "cfwd", n, x)
    assert bits_equal(a, b)


def test_launch_counter_counts(torch_cuda, ctx_cache, lib):
    ctx = ctx_cache(1024)
    x = torch_cuda.zeros((4, 1024), dtype=torch_cuda.complex64, device="cuda")
    y = torch_cuda.zeros((4, 1024), dtype=torch_cuda.complex64, device="cuda")
    before = lib.CkFftCudaLaunchCount()
    ctx.check(ctx.batch("cfwd", 1024, 4, x, y))
    assert lib.CkFftCudaLaunchCount() == before + 1
