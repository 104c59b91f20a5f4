"""The Linux timing harness (ckfft_gb300/harness/ckfft_timing.cpp): the
reference's timing test matrix (src/test/test.cpp:610-721) written as
results_linux_<machine>.xml in the reference's layout."""
import os
import platform
import subprocess
import xml.etree.ElementTree as ET

import pytest

from conftest import ROOT

HARNESS = os.path.join(ROOT, "ckfft_gb300", "_build", "ckfft_timing")
TESTERS = ["ckfft", "ckfft_device", "ckfft_kiss_api", "ckfft_batch"]


def _gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="module")
def harness():
    from ckfft_gb300 import build
    build.build()
    assert os.access(HARNESS, os.X_OK)
    return HARNESS


@pytest.mark.skipif(_gpu(), reason="checks the no-device failure path")
def test_harness_fails_cleanly_without_gpu(harness, tmp_path):
    r = subprocess.run([harness, "--reps", "2", "--out", str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 1 and "ckfft_timing:" in r.stderr
    assert not list(tmp_path.iterdir())


def test_harness_usage(harness, tmp_path):
    r = subprocess.run([harness, "--bogus"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage" in r.stderr
    short = tmp_path / "short.txt"
    short.write_text("1 2\n3 4\n")
    r = subprocess.run([harness, "--input", str(short)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "256" in r.stderr


@pytest.mark.gpu
def test_harness_writes_reference_layout(harness, tmp_path, golden):
    inp = tmp_path / "input.txt"
    inp.write_text("\n".join(f"{float(z.real)!r} {float(z.imag)!r}" for z in golden["input_txt"]) + "\n")
    r = subprocess.run([harness, "--reps", "5", "--out", str(tmp_path), "--input", str(inp)], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    path = tmp_path / f"results_linux_{platform.machine().replace(',', '_')}.xml"
    root = ET.parse(path).getroot()
    assert root.tag == "ckfft_test"
    names = [e.tag for e in root]
    want = []
    n = 4096
    while n > 128:
        want += [f"fft_{n}", f"fft_inv_{n}", f"fft_real_{n}", f"fft_inv_real_{n}"]
        n //= 2
    assert names == want
    for test in root:
        assert [t.tag for t in test] == TESTERS
        for t in test:
            assert float(t.get("time")) > 0
    # a second run reads the first as the previous results
    r2 = subprocess.run([harness, "--reps", "3", "--out", str(tmp_path), "--prev", str(path)],
                        capture_output=True, text=True, timeout=600)
    assert r2.returncode == 0 and "%" in r2.stdout
