"""Benchmark: batched real FFT, N = 4096 FP32, 65536 frames (forward + inverse).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one CkFftCudaRealForwardBatch over all frames followed by one
CkFftCudaRealInverseBatch over the spectra (the workload's forward/inverse
pair), inputs resident in HBM.  Prints one JSON line on rank 0.

  value      GB/s of algorithmic HBM bytes (real transform: 4n + 8(n/2+1) bytes
             each way) over the K timed steps, CUDA events on the launch stream,
             max over ranks, summed over ranks (frames are sharded: weak scaling)
  e2e        same metric through the same C-ABI calls with pinned HOST buffers:
             host->device copies, kernels and device->host copies all timed
  roofline   the forward kernel's achieved GB/s vs the measured HBM copy peak
  cpu_baseline  the reference's scalar path (the oracle port, or the reference
             build where it exists) on every host core, on a sample of frames
  per_call   the plain drop-in: one CkFftRealForward call (one launch) per frame

--impl reference times the reference's CPU implementation on the host cores
for the same workload and metric (rank 0 only).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N = 4096
FRAMES = 65536
METRIC = "batched real FFT GB/s (N=4096 FP32, fwd+inv)"
UNIT = "GB/s"
PROFILE = os.path.join(ROOT, "profiles", "k_r2c_small_n4096_x65536.md")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--frames", type=int, default=FRAMES)
    ap.add_argument("--n", type=int, default=N)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-percall", action="store_true")
    return ap.parse_args()


def frame_bytes(n):
    from ckfft_gb300.workloads import algorithmic_bytes

    return algorithmic_bytes(True, n)


# ----------------------------------------------------------------- helpers

class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.rows = []
        self.proc = None
        self.thread = None
        self.window = (0.0, 0.0)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-i", str(self.dev)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.time(), [c.strip() for c in line.split(",")]))

    def mark(self, t0, t1):
        self.window = (t0, t1)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self):
        t0, t1 = self.window
        inside = [r for t, r in self.rows if t0 - 0.15 <= t <= t1 + 0.15]
        rows = inside or [r for _, r in self.rows]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if len(r) > 1 and num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if len(r) > 2 and num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for i, nm in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(inside)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """dram bytes per launch of the forward kernel from the committed ncu summary."""
    if not os.path.exists(PROFILE):
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", open(PROFILE).read())
    return float(m.group(1)) if m else None


def cpu_frames_sample(frames, n, seed):
    """Sample frames of the workload generated on the host (torch CPU generator)."""
    from ckfft_gb300 import workloads as wl

    return wl.sine_frames_torch(frames, n, seed, device="cpu").numpy()


def time_cpu_reference(n, frames_total, min_seconds=2.0, sample=8192):
    """The reference's scalar path on all host cores: GB/s and transforms/s.

    Runs the oracle port of the reference's algorithm (bit-identical to the
    reference built with the same flags; the reference tree is not on the GPU
    host) with one frame stream per thread, on `sample` distinct frames
    repeated until `min_seconds` of wall time have passed."""
    import numpy as np
    from oracle import oracle as orc

    orc.build(with_reference=False)
    threads = os.cpu_count() or 1
    sample = min(sample, frames_total)
    x = cpu_frames_sample(sample, n, 12345)
    X = np.empty((sample, n // 2 + 1), np.complex64)
    y = np.empty((sample, n), np.float32)
    runner = orc.Oracle(n, fast=True)
    runner.batch_into(orc.KIND_RFWD, n, sample, x, X, threads)   # warm-up
    done = 0
    t0 = time.perf_counter()
    while True:
        runner.batch_into(orc.KIND_RFWD, n, sample, x, X, threads)
        runner.batch_into(orc.KIND_RINV, n, sample, X, y, threads)
        done += sample
        if time.perf_counter() - t0 >= min_seconds:
            break
    dt = time.perf_counter() - t0
    gbs = done * 2 * frame_bytes(n) / dt / 1e9
    return {"value": round(gbs, 3), "unit": UNIT, "cores": threads, "kind": "port",
            "transforms_per_s": round(2 * done / dt, 1),
            "sample": f"{sample} distinct N={n} sinusoid frames, forward+inverse, repeated for "
                      f"{dt:.2f} s ({done} frame pairs) on {threads} threads, one frame stream per thread"}


# ------------------------------------------------------------- reference arm

def run_reference(args, rank, world):
    if rank != 0:
        return
    n, frames = args.n, args.frames
    import numpy as np
    from oracle import oracle as orc

    orc.build(with_reference=False)
    threads = os.cpu_count() or 1
    o = orc.Oracle(n, fast=True)
    sample = min(8192, frames)
    xs = cpu_frames_sample(sample, n, 12345)
    reps = max(1, frames // sample)
    x = np.ascontiguousarray(np.tile(xs, (reps, 1)))
    total = x.shape[0]
    X = np.empty((total, n // 2 + 1), np.complex64)
    y = np.empty((total, n), np.float32)

    def step():
        o.batch_into(orc.KIND_RFWD, n, total, x, X, threads)
        o.batch_into(orc.KIND_RINV, n, total, X, y, threads)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    value = args.steps * total * 2 * frame_bytes(n) / dt / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"real FFT N={n}, {total} sinusoid frames, forward + inverse",
                   "frames": total, "n": n},
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{sample} distinct frames tiled to {total}, forward+inverse per step, "
                                   f"oracle port of the reference's scalar path on {threads} threads"},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "transforms_per_s": round(args.steps * total * 2 / dt, 1),
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ our arm

def run_ours(args, rank, world, local_rank):
    import torch
    from ckfft_gb300 import binding
    from ckfft_gb300 import workloads as wl

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    n, frames = args.n, args.frames
    ctx = binding.Context(n)
    x = wl.sine_frames_torch(frames, n, wl.W2_SEED + rank, device=dev)
    X = torch.empty((frames, n // 2 + 1), dtype=torch.complex64, device=dev)
    y = torch.empty((frames, n), dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)

    def step(ev=None):
        if ev is not None:
            ev[0].record(stream)
        ctx.check(ctx.batch("rfwd", n, frames, x, X, stream), "real forward batch")
        if ev is not None:
            ev[1].record(stream)
        ctx.check(ctx.batch("rinv", n, frames, X, y, stream), "real inverse batch")

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    # correctness gate on the benchmarked data: round trip and one oracle frame
    err = (torch.linalg.vector_norm((y / (2 * n) - x).double()) / torch.linalg.vector_norm(x.double())).item()
    if not err < 1e-5:
        raise SystemExit(f"round-trip error {err:.3e}: refusing to report a number")

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    sampler = ClockSampler(local_rank)
    sampler.start()
    time.sleep(0.3)
    fwd_events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                  for _ in range(args.steps)]
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    launches0 = binding.launch_count()
    w0 = time.time()
    start.record(stream)
    for k in range(args.steps):
        step(fwd_events[k])
    end.record(stream)
    torch.cuda.synchronize()
    w1 = time.time()
    barrier()
    launches = binding.launch_count() - launches0
    sampler.mark(w0, w1)
    time.sleep(0.25)
    sampler.stop()
    secs = start.elapsed_time(end) / 1e3
    fwd_ms = sum(a.elapsed_time(b) for a, b in fwd_events) / args.steps
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([secs], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        secs = float(t.item())

    bytes_step = frames * 2 * frame_bytes(n)
    value = world * bytes_step * args.steps / secs / 1e9
    peak, peak_kind = measured_peaks()
    achieved = frames * frame_bytes(n) / (fwd_ms / 1e3) / 1e9
    traffic = ncu_traffic()

    e2e = None
    if not args.no_e2e:
        e2e = measure_e2e(torch, ctx, x, n, frames, bytes_step, world)

    per_call = None if args.no_percall else measure_per_call(torch, ctx, x, n)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = time_cpu_reference(n, frames)

    if rank != 0:
        ctx.close()
        return
    clocks = sampler.summary()
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3),
        "ms_per_step": round(secs / args.steps * 1e3, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (sum of 8 sinusoids + N(0,0.01^2) noise per frame, seeded)",
        "config": {"workload": f"real FFT N={n} FP32, {frames} frames per GPU, forward + inverse batch",
                   "n": n, "frames": frames, "parallelism": f"replicas x{world} (frames sharded, no collective)",
                   "l2": "inputs larger than L2 (1 GiB of frames per direction), no flush needed"},
        "roofline": {"bound": "hbm", "kernel": "k_r2c_small<11> (real forward, n=4096)",
                     "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                     "traffic": traffic, "algorithmic_bytes_per_launch": frames * frame_bytes(n),
                     "avg_launch_ms": round(fwd_ms, 4)},
        "clocks": clocks,
        "gpu_launches": launches,
        "e2e": e2e,
        "per_call": per_call,
        "transforms_per_s": round(world * 2 * frames * args.steps / secs, 1),
        "gflops_2.5nlog2n": round(world * 2 * frames * 2.5 * n * math.log2(n) * args.steps / secs / 1e9, 1),
        "round_trip_rel_err": err,
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    ctx.close()


def measure_e2e(torch, ctx, x, n, frames, bytes_step, world, steps=3):
    """The same step through the C ABI with pinned host buffers (copies timed)."""
    xh = x.cpu().pin_memory()
    Xh = torch.empty((frames, n // 2 + 1), dtype=torch.complex64).pin_memory()
    yh = torch.empty((frames, n), dtype=torch.float32).pin_memory()
    ctx.check(ctx.batch("rfwd", n, frames, xh, Xh))
    ctx.check(ctx.batch("rinv", n, frames, Xh, yh))
    t0 = time.perf_counter()
    for _ in range(steps):
        ctx.check(ctx.batch("rfwd", n, frames, xh, Xh))
        ctx.check(ctx.batch("rinv", n, frames, Xh, yh))
    dt = (time.perf_counter() - t0) / steps
    h2d = xh.numel() * 4 + Xh.numel() * 8
    d2h = Xh.numel() * 8 + yh.numel() * 4
    return {"value": round(world * bytes_step / dt / 1e9, 2), "unit": UNIT,
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": round(dt * 1e3, 3),
            "steps": steps, "api": "CkFftCudaRealForwardBatch + CkFftCudaRealInverseBatch on pinned host buffers"}


def measure_per_call(torch, ctx, x, n, calls=512):
    """The plain drop-in: CkFftRealForward once per frame, device buffers, one launch each."""
    out = torch.empty((calls, n // 2 + 1), dtype=torch.complex64, device=x.device)
    for f in range(8):
        ctx.check(ctx.real_forward(n, x[f], out[f]))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for f in range(calls):
        ctx.real_forward(n, x[f], out[f])
    dt = time.perf_counter() - t0
    return {"transforms_per_s": round(calls / dt, 1), "gbs": round(calls * frame_bytes(n) / dt / 1e9, 3),
            "calls": calls, "api": "CkFftRealForward per frame (device pointers, blocking)"}


def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist

        dist.init_process_group("gloo")
    run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
