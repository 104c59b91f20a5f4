"""Generates tests/golden/ckfft_golden.npz from the reference itself.

    python tests/golden/make_golden.py

Needs the reference tree (read-only) and its build in oracle/_ref
(`make -C oracle ref`).  Runs only where the reference tree exists; the
committed .npz is what travels with the tests.

Contents (all outputs are the reference library's own results):
  input_txt          the 4096 complex values of src/test/input.txt, the
                     reference regression suite's fixture (src/test/test.cpp:866-921)
  example_input      the 1024 reals of src/example/main.cpp:39-42
  c_{fwd,inv}_{n}_{nmax}  complex forward / inverse of input_txt[:n] for
                     n = 4096 .. 1 and nmax in {n, 8192}, the matrix of
                     src/test/test.cpp:878-894 (nmax = 8192 kept only where
                     it differs; see nmax_invariant)
  r_fwd_{n}_{nmax}   real forward of Re(input_txt[:n])  (test.cpp:896-919)
  r_inv_{n}_{nmax}   real inverse of the first n/2+1 bins of the complex
                     forward of Re(input_txt[:n])         (test.cpp:836-854)
  r_rt_{n}_{nmax}    real inverse of r_fwd (round trip, gain 2n)
  example_fwd / example_rt  the example's real forward and round trip
  w1_in / w1_fwd / w1_rt    4 frames of workload 1 (N = 1024 complex)
  w2_in / w2_fwd / w2_rt    4 frames of workload 2 (N = 4096 real sinusoids)
  w4_{kind}_{log2}          one transform per kind for log2 n = 6..13
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from ckfft_gb300 import workloads  # noqa: E402
from oracle import oracle as orc  # noqa: E402

REF_TREE = os.environ.get("CKFFT_REFERENCE_TREE", "/root/reference")


def read_input_txt():
    vals = np.loadtxt(os.path.join(REF_TREE, "src", "test", "input.txt"), dtype=np.float64)
    vals = vals.astype(np.float32)
    return (vals[0::2] + 1j * vals[1::2]).astype(np.complex64)


def read_example_input():
    src = open(os.path.join(REF_TREE, "src", "example", "main.cpp")).read()
    body = re.search(r"float input\[\]\s*=\s*\{(.*?)\};", src, re.S).group(1)
    vals = [float(tok.rstrip("f")) for tok in re.findall(r"-?[0-9.]+(?:e-?[0-9]+)?f", body)]
    return np.array(vals, np.float32)


def main():
    orc.build(with_reference=True)
    out = {}
    x = read_input_txt()
    assert x.shape == (4096,), x.shape
    out["input_txt"] = x
    ex = read_example_input()
    assert ex.shape == (1024,), ex.shape
    out["example_input"] = ex

    refs = {}

    def ref(nmax):
        if nmax not in refs:
            refs[nmax] = orc.Reference(nmax)
        return refs[nmax]

    # The reference's outputs do not depend on nmax (table subsampling by a
    # power of two is exact), so the nmax = 8192 results are stored only if
    # they differ bit-wise from the nmax = n ones; `nmax_invariant` records it.
    invariant = True
    n = 4096
    while n >= 1:
        per = {}
        for nmax in sorted({n, 8192}):
            r = ref(nmax)
            xr = x[:n].real.copy()
            fwd = r.real_forward(n, xr)
            cf = r.complex(n, xr.astype(np.complex64), False)
            per[nmax] = {
                f"c_fwd_{n}": r.complex(n, x[:n], False),
                f"c_inv_{n}": r.complex(n, x[:n], True),
                f"r_fwd_{n}": fwd,
                f"r_inv_{n}": r.real_inverse(n, cf[: n // 2 + 1]),
                f"r_rt_{n}": r.real_inverse(n, fwd),
            }
        for k, v in per[n].items():
            out[f"{k}_{n}"] = v
            if 8192 in per and 8192 != n:
                w = per[8192][k]
                if not np.array_equal(v.view(np.uint32), w.view(np.uint32)):
                    invariant = False
                    out[f"{k}_8192"] = w
        n //= 2
    out["nmax_invariant"] = np.array([1 if invariant else 0], np.int32)

    r = ref(1024)
    out["example_fwd"] = r.real_forward(1024, ex)
    out["example_rt"] = r.real_inverse(1024, out["example_fwd"])

    w1 = workloads.complex_uniform(4, workloads.W1_N, workloads.W1_SEED)
    r = ref(workloads.W1_N)
    out["w1_in"] = w1
    out["w1_fwd"] = np.stack([r.complex(workloads.W1_N, f, False) for f in w1])
    out["w1_rt"] = np.stack([r.complex(workloads.W1_N, f, True) for f in out["w1_fwd"]])

    w2 = workloads.sine_frames(4, workloads.W2_N, workloads.W2_SEED)
    r = ref(workloads.W2_N)
    out["w2_in"] = w2
    out["w2_fwd"] = np.stack([r.real_forward(workloads.W2_N, f) for f in w2])
    out["w2_rt"] = np.stack([r.real_inverse(workloads.W2_N, f) for f in out["w2_fwd"]])

    rng = np.random.default_rng(44)
    r = ref(1 << 13)
    for l2 in range(6, 14):
        n = 1 << l2
        c = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
        xr = rng.uniform(-1, 1, n).astype(np.float32)
        xh = (rng.uniform(-1, 1, n // 2 + 1) + 1j * rng.uniform(-1, 1, n // 2 + 1)).astype(np.complex64)
        out[f"w4_cin_{l2}"] = c
        out[f"w4_cfwd_{l2}"] = r.complex(n, c, False)
        out[f"w4_cinv_{l2}"] = r.complex(n, c, True)
        out[f"w4_rin_{l2}"] = xr
        out[f"w4_rfwd_{l2}"] = r.real_forward(n, xr)
        out[f"w4_hin_{l2}"] = xh
        out[f"w4_rinv_{l2}"] = r.real_inverse(n, xh)

    for k, v in out.items():
        assert v is not None, k
    path = os.path.join(HERE, "ckfft_golden.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}: {len(out)} arrays, {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
