"""An unmodified C99 program written against the reference's six calls
(tests/c_caller/reference_calls.c: host buffers, CkFftInit / RealForward /
RealInverse / ComplexForward / ComplexInverse / Shutdown) compiled with gcc
against include/ckfft_cuda.h and linked to libckfft_cuda.so; on the GPU its
outputs on the reference example's input (src/example/main.cpp) match the
reference's own outputs from the golden fixture."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, assert_close

SRC = os.path.join(ROOT, "tests", "c_caller", "reference_calls.c")
LIBDIR = os.path.join(ROOT, "ckfft_gb300")


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    from ckfft_gb300 import build
    build.build()
    cc = shutil.which("gcc") or shutil.which("cc")
    assert cc, "a C compiler is required"
    exe = str(tmp_path_factory.mktemp("c_caller") / "reference_calls")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-O2",
                        f"-I{os.path.join(ROOT, 'include')}", SRC, "-o", exe, f"-L{LIBDIR}", "-l:libckfft_cuda.so",
                        f"-Wl,-rpath,{LIBDIR}", "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_c99_caller_builds_against_the_header_and_library(program):
    assert os.access(program, os.X_OK)
    r = subprocess.run(["nm", "-D", "--undefined-only", program], capture_output=True, text=True)
    used = {l.split()[-1] for l in r.stdout.splitlines() if l.strip()}
    ckfft = {u for u in used if u.startswith("CkFft")}
    assert ckfft == {"CkFftInit", "CkFftShutdown", "CkFftRealForward", "CkFftRealInverse",
                     "CkFftComplexForward", "CkFftComplexInverse"}, ckfft


@pytest.mark.gpu
def test_c99_caller_matches_the_reference_outputs(program, golden, tmp_path):
    x = golden["example_input"].astype(np.float32)
    n, m = x.size, x.size // 2
    fin, fout = tmp_path / "in.f32", tmp_path / "out.bin"
    x.tofile(fin)
    r = subprocess.run([program, str(fin), str(fout)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    errs = [float(l.split(":")[1]) for l in r.stdout.splitlines() if "round trip error" in l]
    assert len(errs) == 2 and max(errs) < 1e-8, r.stdout
    raw = np.fromfile(fout, np.uint8)
    spec = raw[: 8 * (m + 1)].view(np.complex64)
    back = raw[8 * (m + 1): 8 * (m + 1) + 4 * n].view(np.float32)
    assert_close(spec, golden["example_fwd"], n, "real forward vs the reference")
    assert_close(back, golden["example_rt"], n, "real round trip vs the reference")
