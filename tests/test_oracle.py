"""CPU tests pinning the oracle to the reference.

The oracle (oracle/ckfft_oracle.c) must reproduce the reference's outputs bit
for bit: against the committed golden vectors (generated by the reference
build, tests/golden/make_golden.py) everywhere, and against the reference
build itself (oracle/_ref) where the reference tree is present.
"""
import os

import numpy as np
import pytest

from conftest import rel_l2


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint32 if a.dtype in (np.float32, np.complex64) else np.uint64)


def same(a, b):
    return a is not None and b is not None and a.shape == b.shape and np.array_equal(bits(a), bits(b))


def test_golden_matrix_bit_exact(golden, oracle_mod):
    """The reference regression matrix (src/test/test.cpp:866-921) on input.txt."""
    x = golden["input_txt"]
    n = 4096
    while n >= 1:
        for nmax in (n, 8192):
            o = oracle_mod.Oracle(nmax)
            sfx = f"{n}_{nmax}" if f"c_fwd_{n}_{nmax}" in golden.files else f"{n}_{n}"
            assert same(o.complex(n, x[:n], False), golden[f"c_fwd_{sfx}"]), ("c_fwd", n, nmax)
            assert same(o.complex(n, x[:n], True), golden[f"c_inv_{sfx}"]), ("c_inv", n, nmax)
            xr = x[:n].real.copy()
            fwd = o.real_forward(n, xr)
            assert same(fwd, golden[f"r_fwd_{sfx}"]), ("r_fwd", n, nmax)
            cf = o.complex(n, xr.astype(np.complex64), False)
            assert same(o.real_inverse(n, cf[: n // 2 + 1]), golden[f"r_inv_{sfx}"]), ("r_inv", n, nmax)
            assert same(o.real_inverse(n, fwd), golden[f"r_rt_{sfx}"]), ("r_rt", n, nmax)
        n //= 2
    assert int(golden["nmax_invariant"][0]) == 1


def test_golden_workloads_bit_exact(golden, oracle_mod):
    o = oracle_mod.Oracle(1 << 13)
    for f in range(4):
        assert same(o.complex(1024, golden["w1_in"][f], False), golden["w1_fwd"][f])
        assert same(o.complex(1024, golden["w1_fwd"][f], True), golden["w1_rt"][f])
        assert same(o.real_forward(4096, golden["w2_in"][f]), golden["w2_fwd"][f])
        assert same(o.real_inverse(4096, golden["w2_fwd"][f]), golden["w2_rt"][f])
    for l2 in range(6, 14):
        n = 1 << l2
        assert same(o.complex(n, golden[f"w4_cin_{l2}"], False), golden[f"w4_cfwd_{l2}"])
        assert same(o.complex(n, golden[f"w4_cin_{l2}"], True), golden[f"w4_cinv_{l2}"])
        assert same(o.real_forward(n, golden[f"w4_rin_{l2}"]), golden[f"w4_rfwd_{l2}"])
        assert same(o.real_inverse(n, golden[f"w4_hin_{l2}"]), golden[f"w4_rinv_{l2}"])


def test_example_round_trip(golden, oracle_mod):
    """src/example/main.cpp:55-76: forward then inverse returns 2n * x."""
    x = golden["example_input"]
    o = oracle_mod.Oracle(1024)
    y = o.real_inverse(1024, o.real_forward(1024, x))
    assert same(y, golden["example_rt"])
    err = float(np.sum((y / 2048.0 - x) ** 2))
    assert err < 1e-9


def test_oracle_vs_fp64(oracle_mod):
    rng = np.random.default_rng(7)
    for l2 in (3, 6, 10, 13, 16):
        n = 1 << l2
        o = oracle_mod.Oracle(n)
        x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
        assert rel_l2(o.complex(n, x, False), oracle_mod.fp64_complex(x)) < 1e-6
        assert rel_l2(o.complex(n, x, True), oracle_mod.fp64_complex(x, True)) < 1e-6
        xr = x.real.copy()
        assert rel_l2(o.real_forward(n, xr), oracle_mod.fp64_real_forward(xr)) < 1e-6
        h = (rng.uniform(-1, 1, n // 2 + 1) + 1j * rng.uniform(-1, 1, n // 2 + 1)).astype(np.complex64)
        assert rel_l2(o.real_inverse(n, h), oracle_mod.fp64_real_inverse(h, n)) < 1e-6


def test_oracle_argument_checks(oracle_mod):
    """Return codes of src/ckfft/ckfft.cpp:16-110 as restated by the oracle."""
    import ctypes as C

    lib = oracle_mod.Oracle.lib()
    assert not lib.ock_init(0, 3)
    assert not lib.ock_init(-4, 3)
    assert not lib.ock_init(12, 3)
    assert not lib.ock_init(16, 0)
    assert not lib.ock_init(16, 4)
    fwd_only = lib.ock_init(16, 1)
    buf = (C.c_float * 64)()
    out = (C.c_float * 64)()
    tmp = (C.c_float * 64)()
    p = C.cast(buf, C.c_void_p)
    q = C.cast(out, C.c_void_p)
    t = C.cast(tmp, C.c_void_p)
    assert lib.ock_complex(None, 8, p, q, 0) == 0
    assert lib.ock_complex(fwd_only, 8, p, q, 1) == 0          # no inverse table
    assert lib.ock_complex(fwd_only, 12, p, q, 0) == 0         # not a power of two
    assert lib.ock_complex(fwd_only, 32, p, q, 0) == 0         # > nmax
    assert lib.ock_complex(fwd_only, 8, p, p, 0) == 0          # in place
    assert lib.ock_complex(fwd_only, 8, None, q, 0) == 0
    assert lib.ock_complex(fwd_only, 8, p, q, 0) == 1
    assert lib.ock_real_inverse(fwd_only, 8, p, q, None) == 0  # tmp checked first
    assert lib.ock_real_inverse(fwd_only, 8, p, q, t) == 0     # no inverse table
    lib.ock_free(fwd_only)


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(__file__)),
                                                    "oracle", "_ref", "libckfft_ref.so")),
                    reason="reference build (oracle/_ref) only exists where the reference tree is")
def test_oracle_matches_reference_build(oracle_mod):
    rng = np.random.default_rng(11)
    for l2 in range(0, 17):
        n = 1 << l2
        for nmax in {n, 4 * n}:
            o = oracle_mod.Oracle(nmax)
            r = oracle_mod.Reference(nmax)
            x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
            assert same(o.complex(n, x, False), r.complex(n, x, False))
            assert same(o.complex(n, x, True), r.complex(n, x, True))
            xr = rng.uniform(-1, 1, n).astype(np.float32)
            assert same(o.real_forward(n, xr), r.real_forward(n, xr))
            h = (rng.uniform(-1, 1, n // 2 + 1) + 1j * rng.uniform(-1, 1, n // 2 + 1)).astype(np.complex64)
            assert same(o.real_inverse(n, h), r.real_inverse(n, h))


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(__file__)),
                                                    "oracle", "_ref", "libkissfft_ref.so")),
                    reason="kiss_fft build (oracle/_ref) only exists where the reference tree is")
def test_kiss_third_opinion(oracle_mod, golden):
    """kiss_fft agrees within the reference harness's RMS threshold 1e-3 (test.cpp:776)."""
    k = oracle_mod.Kiss()
    x = golden["input_txt"]
    for n in (16, 256, 4096):
        o = oracle_mod.Oracle(n)
        d = o.complex(n, x[:n]) - k.complex(n, x[:n])
        assert np.sqrt(np.mean(np.concatenate([d.real, d.imag]) ** 2)) < 1e-3
        xr = x[:n].real.copy()
        d = o.real_forward(n, xr) - k.real_forward(n, xr)
        assert np.sqrt(np.mean(np.concatenate([d.real, d.imag]) ** 2)) < 1e-3


def test_kiss_fixtures(kiss_golden, oracle_mod):
    """The kiss_fft fixtures are unscaled DFTs (FP64 check), kiss_fftri of
    kiss_fftr is the round trip with gain n, and the oracle's real forward is
    twice kiss_fftr (src/test/test.cpp:368-372) within the harness's RMS 1e-3."""
    g = kiss_golden
    for l2 in range(0, 12):
        n = 1 << l2
        x = g[f"cin_{l2}"].astype(np.complex128)
        assert rel_l2(g[f"cfwd_{l2}"], np.fft.fft(x)) < 1e-6
        assert rel_l2(g[f"cinv_{l2}"], np.fft.ifft(x) * n) < 1e-6
        if l2 >= 1:
            r = g[f"rin_{l2}"]
            assert rel_l2(g[f"rfwd_{l2}"], np.fft.rfft(r.astype(np.float64))) < 1e-6
            assert rel_l2(g[f"rinv_{l2}"], r * n) < 1e-6
            o = oracle_mod.Oracle(max(n, 2))
            d = o.real_forward(n, r) - 2 * g[f"rfwd_{l2}"]
            assert np.sqrt(np.mean(np.abs(d) ** 2)) < 1e-3


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "oracle",
                                                    "_ref", "libkissfft_ref.so")),
                    reason="needs the reference's kiss_fft build (oracle/_ref)")
def test_kiss_fixtures_regenerate(kiss_golden, oracle_mod):
    """The committed kiss fixtures are kiss_fft's own outputs, bit for bit."""
    k = oracle_mod.Kiss()
    for l2 in (0, 3, 7, 11):
        n = 1 << l2
        assert same(k.complex(n, kiss_golden[f"cin_{l2}"]), kiss_golden[f"cfwd_{l2}"])
        assert same(k.complex(n, kiss_golden[f"cin_{l2}"], True), kiss_golden[f"cinv_{l2}"])
        if l2:
            assert same(k.real_forward(n, kiss_golden[f"rin_{l2}"]), 2 * kiss_golden[f"rfwd_{l2}"])


def test_batch_runner_matches_single(oracle_mod):
    rng = np.random.default_rng(5)
    n, frames = 256, 37
    o = oracle_mod.Oracle(n)
    x = (rng.uniform(-1, 1, (frames, n)) + 1j * rng.uniform(-1, 1, (frames, n))).astype(np.complex64)
    y = o.batch(oracle_mod.KIND_CFWD, n, frames, x, threads=4)
    for f in (0, 17, 36):
        assert same(y[f], o.complex(n, x[f]))
    xr = rng.uniform(-1, 1, (frames, n)).astype(np.float32)
    yr = o.batch(oracle_mod.KIND_RFWD, n, frames, xr, threads=3)
    zr = o.batch(oracle_mod.KIND_RINV, n, frames, yr, threads=2)
    assert same(zr[5], o.real_inverse(n, yr[5]))
    assert np.allclose(zr / (2 * n), xr, atol=1e-5)
