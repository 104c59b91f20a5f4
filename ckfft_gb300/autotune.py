"""Autotuner for the single-CTA kernels: picks, per transform kind and size,
which kernel variant runs, and writes the choice as a C++ table.

    python -m ckfft_gb300.autotune [--out-dir DIR] [--mb 256] [--reps 20]

Variants (the dimensions searched):
  0    plain kernel in the default shape (16 values per thread, 32 at 2^14;
       transforms per CTA filling 256 threads; radix 16 first, the remainder
       radix last), inputs loaded to registers;
  2, 3 persistent kernel with 2 / 3 bulk-copy (TMA) buffers, default shape;
  4, 5 half / twice the values per thread (radix 8 / 32 stages: threads per
       transform x2 / x0.5, so the radix order changes with it);
  6, 7 transforms per CTA filling 512 / 128 threads;
  8    persistent kernel with one bulk-copy landing buffer and a separate
       exchange area that moves the x parts, then the y parts (complex kinds;
       the form that fits complex 2^14).
Each variant is measured in its own process (the library reads
CKFFT_CUDA_VARIANT once), on batches of about --mb MiB of input per launch,
with CUDA events around --reps launches after warm-up; a variant that does not
exist for a size runs (and measures) the plain kernel.  The winner must beat
the plain kernel by 1% to be chosen.  Outputs in --out-dir:
  tuning_table.h   -> copy to ckfft_gb300/csrc/tuning_table.h and rebuild
  autotune.md      -> the measured table (GB/s of algorithmic bytes)
  autotune.json    -> the raw measurements
The values per thread of a size are chosen for every kernel family at once
(they change the radices, hence the rounding); a size whose values per
thread change runs the plain launch until the next tuning pass, which
measures the launch variants with the new shape.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
KINDS = ["cfwd", "cinv", "rfwd", "rinv"]   # index = ckg::Kind
VARIANTS = [0, 2, 3, 4, 5, 6, 7, 8]
NAMES = ["plain", "pipe x2", "pipe x3", "R/2", "2R", "512 thr", "128 thr", "pipe sx"]
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


def current_log2r() -> list:
    """Values per thread (log2) per size compiled into the library now
    (kTunedLog2R of csrc/tuning_table.h)."""
    text = open(os.path.join(HERE, "csrc", "tuning_table.h")).read()
    m = re.search(r"kTunedLog2R\[\d+\]\s*=\s*\{([0-9, ]+)\}", text)
    return [int(v) for v in m.group(1).split(",")]


# Variants that keep a frame's arithmetic (same radices, so the same bits as
# every other kernel family of the size): pipelined loads, CTA size.
SAME_BITS = [2, 3, 6, 7, 8]


def choose(results: dict, lr0: list):
    """Per size: the values per thread (log2) every kernel family of that size
    uses -- the variant among default / half / twice with the best summed
    GB/s over the four kinds, if it beats the default by 1%.  Per kind and
    size: the launch variant (pipelined loads, CTA size) that beats the plain
    kernel by 1%; none where the values per thread change (the other
    variants were measured with the old ones)."""
    lr, table = list(lr0), [[0] * len(LOG2_RANGE) for _ in KINDS]
    for L in LOG2_RANGE:
        score = {v: sum(results[v][k].get(str(L), 0.0) or 0.0 for k in KINDS) for v in (0, 4, 5)}
        best = max((4, 5), key=lambda v: score[v])
        if score[0] > 0 and score[best] > 1.01 * score[0]:
            lr[L] = lr0[L] - 1 if best == 4 else lr0[L] + 1
    for ki, kind in enumerate(KINDS):
        for L in LOG2_RANGE:
            plain = results[0][kind].get(str(L))
            if plain is None or lr[L] != lr0[L]:
                continue
            best, best_v = plain, 0
            for v in SAME_BITS:
                g = results[v][kind].get(str(L))
                if g is not None and g > 1.01 * plain and g > best:
                    best, best_v = g, v
            table[ki][L] = best_v
    return lr, table


def write_outputs(results: dict, out_dir: str, gpu: str) -> None:
    lr0 = current_log2r()
    lr, table = choose(results, lr0)
    stamp = time.strftime("%Y-%m-%d")
    lines = [
        "// tuning_table.h -- generated by ckfft_gb300/autotune.py; do not edit by hand.",
        f"// Measured on {gpu}, {stamp}.",
        "// kTunedLog2R[L]: values per thread (log2) of every single-CTA kernel family",
        "// (batched, pipelined, strided, fused, grouped, job kernel) for complex",
        "// (half-)length 2^L, so that all of them compute a size with the same radices.",
        "// kTunedVariant[kind][L]: batched kernel variant for kind (0 complex forward,",
        "// 1 complex inverse, 2 real forward, 3 real inverse): 0 plain, 2 / 3 pipelined",
        "// with 2 / 3 bulk-copy buffers, 6 / 7 CTAs of about 512 / 128 threads, 8",
        "// pipelined with one buffer and a split exchange area (the same arithmetic",
        "// as plain).",
        "#pragma once",
        "namespace ckg {",
        f"constexpr signed char kTunedLog2R[{len(LOG2_RANGE)}] = {{" + ", ".join(str(v) for v in lr) + "};",
        f"constexpr signed char kTunedVariant[4][{len(LOG2_RANGE)}] = {{",
    ]
    for kind, row in zip(KINDS, table):
        lines.append("    {" + ", ".join(str(v) for v in row) + "},   // " + kind)
    lines += ["};", "}  // namespace ckg", ""]
    with open(os.path.join(out_dir, "tuning_table.h"), "w") as f:
        f.write("\n".join(lines))
    md = [f"# Autotune of the single-CTA kernels ({gpu}, {stamp})", "",
          "GB/s of algorithmic bytes per launch (complex 16n, real 4n + 8(n/2+1)); "
          "L is log2 of the complex length (real n = 2^(L+1)).  R/2 and 2R are relative to the "
          "values per thread compiled in when measured (log2 R column).", "",
          "| kind | L | log2 R | " + " | ".join(NAMES) + " | chosen variant | chosen log2 R |",
          "|---|---|---|" + "---|" * (len(NAMES) + 2)]
    for ki, kind in enumerate(KINDS):
        for L in LOG2_RANGE:
            vals = [results[v][kind].get(str(L)) for v in VARIANTS]
            if vals[0] is None:
                continue
            cells = ["%.0f" % x if x is not None else "-" for x in vals]
            md.append(f"| {kind} | {L} | {lr0[L]} | " + " | ".join(cells) + f" | {table[ki][L]} | {lr[L]} |")
    with open(os.path.join(out_dir, "autotune.md"), "w") as f:
        f.write("\n".join(md) + "\n")
    with open(os.path.join(out_dir, "autotune.json"), "w") as f:
        json.dump({"gpu": gpu, "date": stamp, "log2r_measured_with": lr0, "results": results}, f)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out-dir", default=".", help="where autotune.json / autotune.md are written")
    ap.add_argument("--mb", type=int, default=256)
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--measure", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--from-json", help="re-derive the table from an earlier autotune.json")
    a = ap.parse_args()
    if a.measure:
        print(json.dumps(measure(a.mb, a.reps)))
        return
    os.makedirs(a.out_dir, exist_ok=True)
    if a.from_json:
        d = json.load(open(a.from_json))
        write_outputs({int(k): v for k, v in d["results"].items()}, a.out_dir, d["gpu"])
        print(open(os.path.join(a.out_dir, "autotune.md")).read())
        return
    results = {}
    for v in VARIANTS:
        env = dict(os.environ, CKFFT_CUDA_VARIANT=str(v))
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
