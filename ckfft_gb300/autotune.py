"""Autotuner for the single-CTA kernels: picks, per transform kind and size,
which kernel variant runs, and writes the choice as a C++ table.

    python -m ckfft_gb300.autotune [--out-dir DIR] [--mb 256] [--reps 20]

Variants: 0 = plain kernel (one CTA launch per frame group, inputs loaded to
registers), 2 / 3 = persistent kernel with 2 / 3 bulk-copy (TMA) buffers.
Each variant is measured in its own process (the library reads
CKFFT_CUDA_PIPE_NBUF once), on batches of about --mb MiB of input per launch,
with CUDA events around --reps launches after warm-up.  The winner must beat
the plain kernel by 1% to be chosen.  Outputs in --out-dir:
  tuning_table.h   -> copy to ckfft_gb300/csrc/tuning_table.h and rebuild
  autotune.md      -> the measured table (GB/s of algorithmic bytes)
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
KINDS = ["cfwd", "cinv", "rfwd", "rinv"]   # index = ckg::Kind
VARIANTS = [0, 2, 3]
LOG2_RANGE = range(0, 15)                  # complex (half) length 2^L


def measure(mb: int, reps: int) -> dict:
    import torch

    sys.path.insert(0, ROOT)
    from ckfft_gb300 import binding
    from ckfft_gb300.workloads import algorithmic_bytes

    ctx = binding.Context(1 << 15)
    stream = torch.cuda.Stream()
    res = {}
    for kind in KINDS:
        res[kind] = {}
        for L in LOG2_RANGE:
            real = kind in ("rfwd", "rinv")
            n = 1 << (L + 1) if real else 1 << L
            if real and n < 8:
                continue
            per = algorithmic_bytes(real, n)
            frames = max(64, (mb << 20) // (per // 2))
            if kind == "rfwd":
                x = torch.randn((frames, n), device="cuda")
                y = torch.empty((frames, n // 2 + 1), dtype=torch.complex64, device="cuda")
            elif kind == "rinv":
                x = torch.randn((frames, n // 2 + 1), dtype=torch.complex64, device="cuda")
                y = torch.empty((frames, n), device="cuda")
            else:
                x = torch.randn((frames, n), dtype=torch.complex64, device="cuda")
                y = torch.empty_like(x)
            for _ in range(3):
                ctx.check(ctx.batch(kind, n, frames, x, y, stream))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record(stream)
            for _ in range(reps):
                ctx.batch(kind, n, frames, x, y, stream)
            b.record(stream)
            torch.cuda.synchronize()
            sec = a.elapsed_time(b) / 1e3 / reps
            res[kind][L] = frames * per / sec / 1e9
            del x, y
    ctx.close()
    return res


def write_outputs(results: dict, out_dir: str, gpu: str) -> None:
    table = []
    for kind in KINDS:
        row = []
        for L in LOG2_RANGE:
            plain = results[0][kind].get(str(L))
            best, best_v = plain, 0
            for v in VARIANTS[1:]:
                g = results[v][kind].get(str(L))
                if g is not None and plain is not None and g > 1.01 * plain and g > best:
                    best, best_v = g, v
            row.append(best_v)
        table.append(row)
    stamp = time.strftime("%Y-%m-%d")
    lines = [
        "// tuning_table.h -- generated by ckfft_gb300/autotune.py; do not edit by hand.",
        f"// Measured on {gpu}, {stamp}.  kTunedVariant[kind][L]: kernel variant for",
        "// kind (0 complex forward, 1 complex inverse, 2 real forward, 3 real inverse)",
        "// and complex (half-)length 2^L: 0 plain, 2 / 3 pipelined with 2 / 3 buffers.",
        "#pragma once",
        "namespace ckg {",
        f"constexpr signed char kTunedVariant[4][{len(LOG2_RANGE)}] = {{",
    ]
    for kind, row in zip(KINDS, table):
        lines.append("    {" + ", ".join(str(v) for v in row) + "},   // " + kind)
    lines += ["};", "}  // namespace ckg", ""]
    with open(os.path.join(out_dir, "tuning_table.h"), "w") as f:
        f.write("\n".join(lines))
    md = [f"# Autotune of the single-CTA kernels ({gpu}, {stamp})", "",
          "GB/s of algorithmic bytes per launch (complex 16n, real 4n + 8(n/2+1)); "
          "L is log2 of the complex length (real n = 2^(L+1)).", "",
          "| kind | L | plain | pipe x2 | pipe x3 | chosen |", "|---|---|---|---|---|---|"]
    for ki, kind in enumerate(KINDS):
        for li, L in enumerate(LOG2_RANGE):
            vals = [results[v][kind].get(str(L)) for v in VARIANTS]
            if vals[0] is None:
                continue
            cells = ["%.0f" % x if x is not None else "-" for x in vals]
            md.append(f"| {kind} | {L} | " + " | ".join(cells) + f" | {table[ki][li]} |")
    with open(os.path.join(out_dir, "autotune.md"), "w") as f:
        f.write("\n".join(md) + "\n")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out-dir", default=".", help="where autotune.json / autotune.md are written")
    ap.add_argument("--mb", type=int, default=256)
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--measure", action="store_true", help=argparse.SUPPRESS)
    a = ap.parse_args()
    if a.measure:
        print(json.dumps(measure(a.mb, a.reps)))
        return
    os.makedirs(a.out_dir, exist_ok=True)
    results = {}
    for v in VARIANTS:
        env = dict(os.environ, CKFFT_CUDA_PIPE_NBUF=str(v))
        out = subprocess.run([sys.executable, "-m", "ckfft_gb300.autotune", "--measure", "--mb", str(a.mb),
                              "--reps", str(a.reps)], cwd=ROOT, env=env, capture_output=True, text=True)
        if out.returncode != 0:
            sys.stderr.write(out.stderr)
            raise SystemExit(f"measurement for variant {v} failed")
        results[v] = json.loads(out.stdout.strip().splitlines()[-1])
    import torch

    write_outputs(results, a.out_dir, torch.cuda.get_device_name(0))
    print(open(os.path.join(a.out_dir, "autotune.md")).read())


if __name__ == "__main__":
    main()
