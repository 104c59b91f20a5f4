"""CPU tests of the C-ABI library: it builds, loads, exports what the header
declares, compiles as C, and rejects invalid arguments with the reference's
return codes before touching a GPU.  No transform runs here."""
import ctypes as C
import os
import re
import subprocess

import pytest

from conftest import ROOT
from ckfft_gb300 import binding

LIB = binding.LIB_PATH


@pytest.fixture(scope="module")
def built():
    from ckfft_gb300 import build

    build.build()
    return binding.load()


def gpu_present():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def test_exports_every_declared_function(built):
    names = binding.header_functions()
    assert {"CkFftInit", "CkFftShutdown", "CkFftComplexForward", "CkFftComplexInverse",
            "CkFftRealForward", "CkFftRealInverse"} <= set(names)
    out = subprocess.run(["nm", "-D", "--defined-only", LIB], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        getattr(built, n)


def test_exports_every_kiss_function(built):
    """The kiss_fft-compatible boundary: every function of kiss_fft_cuda.h."""
    names = binding.header_functions(os.path.join(ROOT, "include", "kiss_fft_cuda.h"), "kiss_")
    assert {"kiss_fft_alloc", "kiss_fft", "kiss_fft_stride", "kiss_fft_free", "kiss_fft_cleanup",
            "kiss_fft_next_fast_size", "kiss_fftr_alloc", "kiss_fftr", "kiss_fftri", "kiss_fftr_free"} == set(names)
    out = subprocess.run(["nm", "-D", "--defined-only", LIB], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (\w+)", out))
    assert not [n for n in names if n not in exported]


def test_kiss_host_logic_without_gpu(built):
    """Size query, size rules and NULL cfg, none of which needs a device."""
    lib = built
    lib.kiss_fft_alloc.restype = C.c_void_p
    lib.kiss_fft_alloc.argtypes = [C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_size_t)]
    lib.kiss_fftr_alloc.restype = C.c_void_p
    lib.kiss_fftr_alloc.argtypes = [C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_size_t)]
    lib.kiss_fft.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    lib.kiss_fft_free.argtypes = [C.c_void_p]
    n = C.c_size_t(0)
    assert lib.kiss_fft_alloc(1024, 0, None, C.byref(n)) is None and n.value > 0
    small = C.c_size_t(1)
    buf = (C.c_char * 8)()
    assert lib.kiss_fft_alloc(1024, 0, buf, C.byref(small)) is None and small.value == n.value
    big = (C.c_char * 4096)()
    assert lib.kiss_fft_alloc(1000, 0, big, C.byref(C.c_size_t(4096))) is None
    assert "power of two" in binding.last_error()
    assert lib.kiss_fftr_alloc(1, 0, None, None) is None
    a, b = (C.c_float * 16)(), (C.c_float * 16)()
    lib.kiss_fft(None, a, b)
    assert "cfg" in binding.last_error()
    lib.kiss_fft_free(None)
    assert lib.kiss_fft_next_fast_size(1000) == 1024 and lib.kiss_fft_next_fast_size(1) == 1
    assert lib.kiss_fft_next_fast_size(4096) == 4096


def test_no_oracle_or_fallback_in_product():
    """The product library neither links nor names the oracle."""
    out = subprocess.run(["nm", "-D", LIB], capture_output=True, text=True, check=True).stdout
    assert not re.search(r"\bock_\w+", out)
    deps = subprocess.run(["readelf", "-d", LIB], capture_output=True, text=True, check=True).stdout
    assert "oracle" not in deps and "ckfft_ref" not in deps
    for dirpath, _, files in os.walk(os.path.join(ROOT, "ckfft_gb300")):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                text = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in text and "from oracle" not in text, f


@pytest.mark.parametrize("std,lang", [("c99", "c"), ("c11", "c"), ("c++11", "c++")])
def test_header_compiles(tmp_path, std, lang):
    """The header must compile as C (cf. src/test/test.c:1-3) and as C++."""
    src = tmp_path / ("t.c" if lang == "c" else "t.cpp")
    src.write_text('#include "ckfft_cuda.h"\nint f(void) { CkFftComplex c; c.real = 1; c.imag = 2;'
                   ' return (int)(c.real + c.imag) + (int)kCkFftDirection_Both; }\n')
    cc = "gcc" if lang == "c" else "g++"
    subprocess.run([cc, f"-std={std}", "-pedantic", "-Wall", "-Werror", "-fsyntax-only",
                    f"-I{os.path.join(ROOT, 'include')}", str(src)], check=True)


@pytest.mark.parametrize("std,lang", [("c99", "c"), ("c++11", "c++")])
def test_kiss_header_compiles(tmp_path, std, lang):
    """kiss_fft_cuda.h compiles as C and C++, alone and with ckfft_cuda.h."""
    src = tmp_path / ("k.c" if lang == "c" else "k.cpp")
    src.write_text('#include "ckfft_cuda.h"\n#include "kiss_fft_cuda.h"\n'
                   'int f(void) { kiss_fft_cpx c; c.r = 1; c.i = 2; kiss_fft_cfg g = 0; kiss_fftr_cfg h = 0;'
                   ' (void)g; (void)h; return (int)(c.r + c.i) + kiss_fftr_next_fast_size_real(5); }\n')
    cc = "gcc" if lang == "c" else "g++"
    subprocess.run([cc, f"-std={std}", "-pedantic", "-Wall", "-Werror", "-fsyntax-only",
                    f"-I{os.path.join(ROOT, 'include')}", str(src)], check=True)


def test_struct_layout(built):
    """CkFftComplex is {float real; float imag} with no padding."""
    class Cx(C.Structure):
        _fields_ = [("real", C.c_float), ("imag", C.c_float)]

    assert C.sizeof(Cx) == 8


def test_init_argument_checks_without_gpu(built):
    """src/ckfft/ckfft.cpp:16-31 and context.cpp:68-72, all decided on the host."""
    lib = built
    assert not lib.CkFftInit(0, 3, None, None)
    assert not lib.CkFftInit(-8, 3, None, None)
    assert not lib.CkFftInit(24, 3, None, None)
    assert not lib.CkFftInit(16, 0, None, None)
    assert not lib.CkFftInit(16, 7, None, None)
    buf = (C.c_char * 256)()
    assert not lib.CkFftInit(16, 3, buf, None)            # buf without bufSize
    size = C.c_size_t(0)
    assert not lib.CkFftInit(16, 3, None, C.byref(size))  # size query
    assert size.value > 0
    need = size.value
    small = C.c_size_t(need - 1)
    assert not lib.CkFftInit(16, 3, buf, C.byref(small))   # too small: size reported
    assert small.value == need
    assert "size" in binding.last_error()


def test_transform_argument_checks_without_gpu(built):
    lib = built
    a = (C.c_float * 64)()
    b = (C.c_float * 64)()
    for f in (lib.CkFftComplexForward, lib.CkFftComplexInverse, lib.CkFftRealForward):
        assert f(None, 8, a, b) == 0
    assert lib.CkFftRealInverse(None, 8, a, b, None) == 0
    assert "tmpBuf" in binding.last_error()                # checked before the context
    assert lib.CkFftRealInverse(None, 8, a, b, a) == 0
    assert "context" in binding.last_error()
    for f in (lib.CkFftCudaComplexForwardBatch, lib.CkFftCudaComplexInverseBatch,
              lib.CkFftCudaRealForwardBatch, lib.CkFftCudaRealInverseBatch):
        assert f(None, 8, 1, a, b, None) == 0
    for f in (lib.CkFftCudaComplexForwardStrided, lib.CkFftCudaComplexInverseStrided,
              lib.CkFftCudaRealForwardStrided, lib.CkFftCudaRealInverseStrided):
        assert f(None, 8, 1, a, 1, 8, b, 1, 8, None) == 0
        assert "context" in binding.last_error()
    lib.CkFftShutdown(None)


@pytest.mark.skipif(gpu_present(), reason="checks the no-device failure path")
def test_init_without_device_fails_cleanly(built):
    assert not built.CkFftInit(16, 3, None, None)
    msg = binding.last_error()
    assert msg, "an error message is expected"


def test_launch_counter_starts_at_zero_without_gpu(built):
    if gpu_present():
        pytest.skip("counter may be nonzero after GPU work in this process")
    assert built.CkFftCudaLaunchCount() == 0
