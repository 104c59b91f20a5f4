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
  w4         the uneven batch (10000 transforms, log2 n 6..16, mixed kinds) in
             one graph replay: GB/s, fraction of HBM, transforms/s against one
             drop-in call per transform, and its CPU baseline
  w5         serving: Poisson request streams at 10-90% of the batched peak of
             the same request mix, p50 / p99 / p99.9 through the server and
             through one call per request, device- and host-resident requests

--gpus N must equal the launcher's WORLD_SIZE (torchrun --nproc-per-node N):
one rank per GPU, each transforming its own shard of frames (replicas, no
collective besides the barrier and the max of the timing).

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
# complex sizes from 2^21 on run as three HBM passes (fft_large.cu), below as two
THREE_PASS_MIN_LOG2 = 21
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
    ap.add_argument("--no-w4", action="store_true", help="default line: leave out the uneven-batch sub-object")
    ap.add_argument("--no-w5", action="store_true", help="default line: leave out the serving sub-object")
    ap.add_argument("--requests", type=int, default=10000, help="w5: requests per offered load")
    ap.add_argument("--direct-mb", type=int, default=8, help="w5: requests this large skip batching")
    ap.add_argument("--workload", choices=["w1", "w2", "w3", "w4", "w5", "sizes", "layouts"], default="w2",
                    help="w2 (default): real n=4096 x 65536 frames; w1: complex n=1024 x 4096 round trip; "
                         "w3: large single complex transforms; w4: uneven mixed batch; w5: serving; "
                         "sizes: batched GB/s per size and kind; layouts: distance-1 advanced layouts")
    ap.add_argument("--sizes", default=",".join(str(i) for i in range(25)),
                    help="sizes workload: comma-separated log2 n")
    ap.add_argument("--kinds", default="cfwd,cinv,rfwd,rinv", help="sizes workload: comma-separated kinds")
    return ap.parse_args()


VARIANT_SHAPE = {0: "", 2: "pipelined, 2 bulk-copy buffers", 3: "pipelined, 3 bulk-copy buffers",
                 4: "half the values per thread", 5: "twice the values per thread",
                 6: "CTAs of about 512 threads", 7: "CTAs of about 128 threads"}


def kernel_label(kind, n):
    """The single-CTA kernel (and tuned variant) the library runs for a batch
    of this kind and size, from the committed tuning table."""
    kinds = ["cfwd", "cinv", "rfwd", "rinv"]
    lc = int(math.log2(n)) - (1 if kind[0] == "r" else 0)
    v = 0
    path = os.path.join(ROOT, "ckfft_gb300", "csrc", "tuning_table.h")
    if os.path.exists(path):
        rows = re.findall(r"\{([0-9, ]+)\},\s*//\s*(\w+)", open(path).read())
        table = {name: [int(x) for x in row.split(",")] for row, name in rows}
        if kind in table and lc < len(table[kind]):
            v = table[kind][lc]
    name = {"cfwd": "k_c2c_small", "cinv": "k_c2c_small", "rfwd": "k_r2c_small", "rinv": "k_c2r_small"}[kind]
    if v in (2, 3):
        name = "k_pipe"
    shape = VARIANT_SHAPE.get(v, "")
    return f"{name}<{lc}>" + (f" ({shape})" if shape else "")


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
    shard = frame_shard(rank, world, frames)
    ctx = binding.Context(n)
    x = wl.sine_frames_torch(frames, n, shard["seed"], device=dev)
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
    # correctness gate on the benchmarked data: the round trip, and one frame
    # of each direction against the oracle (the inverse on the GPU's spectrum)
    err = (torch.linalg.vector_norm((y / (2 * n) - x).double()) / torch.linalg.vector_norm(x.double())).item()
    if not err < 1e-5:
        raise SystemExit(f"round-trip error {err:.3e}: refusing to report a number")
    gate = oracle_gate(n, x[frames // 2].cpu().numpy(), X[frames // 2].cpu().numpy(), y[frames // 2].cpu().numpy())

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
    bytes_step = frames * 2 * frame_bytes(n)
    secs, value = combine_ranks(secs, bytes_step * args.steps, world)
    peak, peak_kind = measured_peaks()
    achieved = frames * frame_bytes(n) / (fwd_ms / 1e3) / 1e9
    traffic = ncu_traffic()

    e2e = None
    if not args.no_e2e:
        e2e = measure_e2e(torch, ctx, x, n, frames, bytes_step, world, steps=args.steps)

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
        "roofline": {"bound": "hbm", "kernel": kernel_label("rfwd", n) + f", real forward n={n}",
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
        "oracle_gate": gate,
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    ctx.close()
    if world == 1 and not args.no_w4:
        line["w4"] = measure_w4(args)
    if world == 1 and not args.no_w5:
        line["w5"] = measure_w5(args)
    print(json.dumps(line), flush=True)


def oracle_gate(n, x, X, y):
    """One frame of the benchmarked data against the oracle: the forward
    spectrum of x, and the inverse of the GPU's own spectrum X."""
    from oracle import oracle as orc

    orc.build(with_reference=False)
    o = orc.Oracle(n)
    ef = orc.rel_l2(X, o.real_forward(n, x))
    ei = orc.rel_l2(y, o.real_inverse(n, X))
    if not (ef <= 1e-5 and ei <= 1e-5):
        raise SystemExit(f"oracle gate failed: forward {ef:.3e}, inverse {ei:.3e}: refusing to report a number")
    return {"forward_rel_l2": ef, "inverse_rel_l2": ei}


def measure_e2e(torch, ctx, x, n, frames, bytes_step, world, steps=20):
    """The same step through the C ABI with pinned host buffers (copies timed),
    over as many steps as the device-timed value."""
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
            "steps": steps, "api": "CkFftCudaRealForwardBatch + CkFftCudaRealInverseBatch on pinned host buffers",
            "route": "real inverse read and written in place by the kernel over the CPU-GPU link; "
                     "real forward (ragged n/2+1 rows, > 128 MiB) staged by copy engines"}


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


def frame_shard(rank, world, frames_per_rank, seed=None):
    """Rank `rank`'s share of a weak-scaling run: frames [start, start + count)
    of the job's world * frames_per_rank frames, generated from its own seed."""
    if not (0 <= rank < world) or frames_per_rank < 0:
        raise ValueError(f"bad shard: rank {rank} of {world}, {frames_per_rank} frames")
    from ckfft_gb300 import workloads as wl

    base = wl.W2_SEED if seed is None else seed
    return {"start": rank * frames_per_rank, "count": frames_per_rank, "seed": base + rank}


def combine_ranks(secs, bytes_local, world):
    """Whole-job figures from each rank's timed region: the slowest rank's time
    (max over ranks, a collective on the timing only) and the bytes of all
    ranks (every rank processes its own frames: weak scaling)."""
    if world > 1:
        import torch
        import torch.distributed as dist

        t = torch.tensor([secs], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        secs = float(t.item())
    return secs, world * bytes_local / secs / 1e9


# ------------------------------------------------------------ other workloads

def l2_flusher(torch, dev):
    """Between timed steps, outside the events: writes a buffer twice the L2 size,
    then reads another one, so L2 holds clean lines (no write-back of the flush
    buffer lands inside the next timed step)."""
    wbuf = torch.empty(64 << 20, dtype=torch.float32, device=dev)     # 256 MiB
    rbuf = torch.ones(64 << 20, dtype=torch.float32, device=dev)

    def flush():
        wbuf.fill_(1.0)
        rbuf.sum()
    return flush


def timed_steps(torch, stream, step, steps, flush=None):
    """Sum of per-step CUDA-event times on `stream`.  Every step and every L2
    flush (between steps, outside the events) is enqueued on `stream` ahead
    of time, so the events time the GPU's work rather than the host's calls;
    one synchronize closes the run."""
    torch.cuda.synchronize()
    events = []
    with torch.cuda.stream(stream):
        for _ in range(steps):
            if flush:
                flush()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step()
            b.record(stream)
            events.append((a, b))
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in events) / 1e3


def base_line(args, metric, value, unit, secs, config, world=1):
    return {"metric": metric, "value": round(value, 2), "unit": unit, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": round(secs / args.steps * 1e3, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "config": config}


def run_w1(args):
    """Workload 1: complex forward then inverse, n = 1024, 4096 frames, U[-1,1) seed 0."""
    import torch
    from ckfft_gb300 import binding
    from ckfft_gb300 import workloads as wl

    n, frames = wl.W1_N, wl.W1_FRAMES
    ctx = binding.Context(n)
    x = torch.from_numpy(wl.complex_uniform(frames, n, wl.W1_SEED)).cuda()
    X, y = torch.empty_like(x), torch.empty_like(x)
    stream = torch.cuda.Stream()
    fwd_ev = []

    def step():
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.check(ctx.batch("cfwd", n, frames, x, X, stream))
        b.record(stream)
        fwd_ev.append((a, b))
        ctx.check(ctx.batch("cinv", n, frames, X, y, stream))

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    err = (torch.linalg.vector_norm(y / n - x) / torch.linalg.vector_norm(x)).item()
    fwd_ev.clear()
    flush = l2_flusher(torch, x.device)
    launches0 = binding.launch_count()
    secs = timed_steps(torch, stream, step, args.steps, flush)
    launches = binding.launch_count() - launches0
    per = 16 * n
    value = args.steps * 2 * frames * per / secs / 1e9
    fwd_ms = sum(a.elapsed_time(b) for a, b in fwd_ev) / len(fwd_ev)
    peak, src = measured_peaks()
    line = base_line(args, "batched complex FFT GB/s (N=1024 FP32, fwd+inv)", value, "GB/s", secs,
                     {"workload": f"complex FFT n={n}, {frames} frames, forward then inverse (round trip)",
                      "n": n, "frames": frames, "l2": "256 MiB buffer written between timed steps (outside the events)"})
    line["roofline"] = {"bound": "hbm", "kernel": kernel_label("cfwd", n) + f", complex forward n={n}",
                        "achieved": round(frames * per / (fwd_ms / 1e3) / 1e9, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(frames * per / (fwd_ms / 1e3) / 1e9 / peak, 4), "peak_source": src,
                        "traffic": None, "avg_launch_ms": round(fwd_ms, 4)}
    line["gpu_launches"] = launches
    line["round_trip_rel_err"] = err
    line["transforms_per_s"] = round(args.steps * 2 * frames / secs, 1)
    if not args.no_e2e:
        xh = x.cpu().pin_memory()
        Xh = torch.empty_like(xh).pin_memory()
        yh = torch.empty_like(xh).pin_memory()
        ctx.check(ctx.batch("cfwd", n, frames, xh, Xh))
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ctx.check(ctx.batch("cfwd", n, frames, xh, Xh))
            ctx.check(ctx.batch("cinv", n, frames, Xh, yh))
        dt = (time.perf_counter() - t0) / args.steps
        line["e2e"] = {"value": round(2 * frames * per / dt / 1e9, 2), "unit": "GB/s",
                       "h2d_bytes_per_step": 2 * frames * n * 8, "d2h_bytes_per_step": 2 * frames * n * 8,
                       "ms_per_step": round(dt * 1e3, 3)}
    if not args.no_cpu:
        line["cpu_baseline"] = time_cpu_complex(n, frames)
    print(json.dumps(line), flush=True)
    ctx.close()


# (name, kind, n, transforms, distance-1 side: "both" / "in" / "out")
LAYOUT_CASES = [
    ("interleaved channels, complex n=4096 x 16384, both sides", "cfwd", 4096, 16384, "both"),
    ("interleaved channels, complex n=4096 x 16384, input side", "cfwd", 4096, 16384, "in"),
    ("interleaved reals -> spectra, n=4096 x 16384", "rfwd", 4096, 16384, "in"),
    ("spectra -> interleaved reals, n=4096 x 16384", "rinv", 4096, 16384, "out"),
    ("matrix columns, complex 1024 x 65536", "cfwd", 1024, 65536, "both"),
    ("interleaved channels, complex n=2^16 x 1024, both sides", "cfwd", 1 << 16, 1024, "both"),
]


def run_layouts(args):
    """Distance-1 advanced layouts through CkFftCuda*Strided (device buffers,
    CUDA events on the launching stream) against the contiguous batch of the
    same work; GB/s of algorithmic bytes (each element read or written once)."""
    import torch
    from ckfft_gb300 import binding
    from ckfft_gb300.workloads import algorithmic_bytes

    ctx = binding.Context(max(c[2] for c in LAYOUT_CASES))
    stream = torch.cuda.Stream()
    g = torch.Generator(device="cuda")
    g.manual_seed(11)
    steps = max(3, min(args.steps, 20))
    table = {}

    def timed(call):
        for _ in range(3):
            ctx.check(call())
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        for _ in range(steps):
            call()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3 / steps

    for name, kind, n, count, side in LAYOUT_CASES:
        real = kind in ("rfwd", "rinv")
        nin = n if kind != "rinv" else n // 2 + 1
        nout = n if kind != "rfwd" else n // 2 + 1
        tin = torch.float32 if kind == "rfwd" else torch.complex64
        tout = torch.float32 if kind == "rinv" else torch.complex64
        mk = (lambda rows, cols, dt: torch.randn((rows, cols), generator=g, device="cuda", dtype=dt))
        din, dout = side in ("both", "in"), side in ("both", "out")
        x = mk(nin, count, tin) if din else mk(count, nin, tin)
        y = torch.empty((nout, count) if dout else (count, nout), device="cuda", dtype=tout)
        isd = (count, 1) if din else (1, nin)
        osd = (count, 1) if dout else (1, nout)
        t_lay = timed(lambda: ctx.strided(kind, n, count, x, isd[0], isd[1], y, osd[0], osd[1], stream))
        xc = torch.empty((count, nin), device="cuda", dtype=tin)
        yc = torch.empty((count, nout), device="cuda", dtype=tout)
        t_con = timed(lambda: ctx.batch(kind, n, count, xc, yc, stream))
        per = count * algorithmic_bytes(real, n)
        table[name] = {"gbs": round(per / t_lay / 1e9, 1), "contiguous_gbs": round(per / t_con / 1e9, 1),
                       "ms": round(t_lay * 1e3, 4)}
        del x, y, xc, yc
    first = table[LAYOUT_CASES[0][0]]
    peak, src = measured_peaks()
    line = base_line(args, "advanced-layout batch GB/s (" + LAYOUT_CASES[0][0] + ")", first["gbs"], "GB/s",
                     first["ms"] / 1e3 * args.steps,
                     {"workload": "distance-1 layouts through CkFftCuda*Strided, device buffers",
                      "l2": "every case larger than L2", "steps": steps})
    line["table"] = table
    line["roofline"] = {"bound": "hbm", "kernel": "transposes + contiguous batched kernels", "achieved": first["gbs"],
                        "peak": peak, "unit": "GB/s", "frac": round(first["gbs"] / peak, 4), "peak_source": src,
                        "traffic": None}
    print(json.dumps(line), flush=True)
    ctx.close()


def time_cpu_complex(n, frames, min_seconds=2.0):
    import numpy as np
    from oracle import oracle as orc
    from ckfft_gb300 import workloads as wl

    orc.build(with_reference=False)
    threads = os.cpu_count() or 1
    x = wl.complex_uniform(frames, n, 0)
    X = np.empty_like(x)
    y = np.empty_like(x)
    o = orc.Oracle(n, fast=True)
    o.batch_into(orc.KIND_CFWD, n, frames, x, X, threads)
    done, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < min_seconds:
        o.batch_into(orc.KIND_CFWD, n, frames, x, X, threads)
        o.batch_into(orc.KIND_CINV, n, frames, X, y, threads)
        done += frames
    dt = time.perf_counter() - t0
    return {"value": round(done * 2 * 16 * n / dt / 1e9, 3), "unit": "GB/s", "cores": threads, "kind": "port",
            "transforms_per_s": round(2 * done / dt, 1),
            "sample": f"{frames} frames of n={n}, forward+inverse, repeated for {dt:.2f} s on {threads} threads"}


def run_w3(args):
    """Workload 3: single complex transforms of 2^20, 2^22, 2^24 points, N(0,1), fwd + inv."""
    import numpy as np
    import torch
    from ckfft_gb300 import binding
    from ckfft_gb300 import workloads as wl
    from oracle import oracle as orc

    ctx = binding.Context(1 << 24)
    stream = torch.cuda.Stream()
    flush = l2_flusher(torch, torch.device("cuda"))
    peak, src = measured_peaks()
    sizes = {}
    for l2 in wl.W3_LOG2:
        n = 1 << l2
        xh = wl.complex_normal(n, seed=l2)
        x = torch.from_numpy(xh).cuda()
        X, y = torch.empty_like(x), torch.empty_like(x)

        def step():
            ctx.check(ctx.batch("cfwd", n, 1, x, X, stream))
            ctx.check(ctx.batch("cinv", n, 1, X, y, stream))

        for _ in range(max(args.warmup, 3)):
            step()
        torch.cuda.synchronize()
        fwd_err = float(np.linalg.norm(X.cpu().numpy() - np.fft.fft(xh.astype(np.complex128))) /
                        np.linalg.norm(np.fft.fft(xh.astype(np.complex128))))
        rt_err = (torch.linalg.vector_norm(y / n - x) / torch.linalg.vector_norm(x)).item()
        secs = timed_steps(torch, stream, step, args.steps, flush)
        gbs = args.steps * 2 * 16 * n / secs / 1e9
        passes = 3 if l2 >= THREE_PASS_MIN_LOG2 else 2      # HBM passes of the multi-pass path
        sizes[f"2^{l2}"] = {"gbs_algorithmic": round(gbs, 1), "passes": passes,
                            "gbs_pass_traffic": round(passes * gbs, 1),
                            "frac_of_peak_pass_traffic": round(passes * gbs / peak, 4),
                            "frac_of_peak_algorithmic": round(gbs / peak, 4),
                            "us_per_transform": round(secs / (2 * args.steps) * 1e6, 2),
                            "rel_err_fwd_vs_fp64": fwd_err, "round_trip_rel_err": rt_err}
        del x, X, y
    top = sizes[f"2^{max(wl.W3_LOG2)}"]
    line = base_line(args, "large complex FFT GB/s (2^24 points, fwd+inv)", top["gbs_algorithmic"], "GB/s",
                     top["us_per_transform"] * 2 * args.steps / 1e6,
                     {"workload": "single complex transforms of 2^20, 2^22, 2^24 points, N(0,1), forward + inverse",
                      "l2": "256 MiB buffer written between timed steps (outside the events)",
                      "passes": {k: v["passes"] for k, v in sizes.items()}})
    line["sizes"] = sizes
    line["roofline"] = {"bound": "hbm",
                        "kernel": "k_cols + k_cols + k_rows3 (three passes, 16 n bytes each) at 2^24",
                        "achieved": top["gbs_pass_traffic"], "peak": peak, "unit": "GB/s",
                        "frac": top["frac_of_peak_pass_traffic"], "peak_source": src, "traffic": None,
                        "algorithmic_frac": top["frac_of_peak_algorithmic"]}
    print(json.dumps(line), flush=True)
    ctx.close()


def run_sizes(args):
    """Batched throughput per size and kind: about 1 GiB of input per call
    (CkFftCuda*Batch on device buffers, larger than L2, so no flush), the
    calls of each (size, kind) enqueued back to back and timed with CUDA
    events; GB/s of algorithmic bytes."""
    import torch
    from ckfft_gb300 import binding
    from ckfft_gb300 import workloads as wl

    sizes = [int(v) for v in args.sizes.split(",")]
    ctx = binding.Context(1 << max(1, max(sizes)))
    stream = torch.cuda.Stream()
    peak, src = measured_peaks()
    table = {}
    total_secs = 0.0
    for l2 in sizes:
        n = 1 << l2
        row = {}
        for kind in args.kinds.split(","):
            real = kind[0] == "r"
            in_b = 4 * n if kind == "rfwd" else 8 * (n // 2 + 1) if kind == "rinv" else 8 * n
            out_b = 8 * (n // 2 + 1) if kind == "rfwd" else 4 * n if kind == "rinv" else 8 * n
            count = max(1, (1 << 30) // in_b)
            x = torch.randn(count * in_b // 4, device="cuda")
            y = torch.empty(count * out_b // 4 + 4, device="cuda")

            def step():
                ctx.check(ctx.batch(kind, n, count, x, y, stream))

            for _ in range(max(args.warmup, 3)):
                step()
            secs = timed_steps(torch, stream, step, args.steps)
            total_secs += secs
            row[kind] = round(args.steps * count * wl.algorithmic_bytes(real, n) / secs / 1e9, 1)
            del x, y
        table[f"2^{l2}"] = row
    top = next(iter(table[f"2^{sizes[-1]}"].values()))
    line = base_line(args, f"batched FFT GB/s per size (value: {args.kinds.split(',')[0]} at 2^{sizes[-1]})", top, "GB/s",
                     total_secs, {"workload": "one batch of about 1 GiB of input per size and kind, device buffers",
                                  "l2": "inputs larger than L2, no flush", "sizes": sizes})
    line["table"] = table
    line["roofline"] = {"bound": "hbm", "kernel": f"batched kernels at 2^{sizes[-1]}", "achieved": top, "peak": peak,
                        "unit": "GB/s", "frac": round(top / peak, 4), "peak_source": src, "traffic": None}
    print(json.dumps(line), flush=True)
    ctx.close()


def w4_jobs(torch, g):
    """The uneven batch's 10000 jobs with U[-1,1) inputs generated on the device."""
    from ckfft_gb300 import workloads as wl

    jobs = []
    for real, inv, l2 in wl.uneven_jobs():
        n = 1 << l2
        if real and not inv:
            x = torch.rand(n, generator=g, device="cuda") * 2 - 1
            y = torch.empty(n // 2 + 1, dtype=torch.complex64, device="cuda")
            kind = "rfwd"
        elif real:
            x = torch.complex(torch.rand(n // 2 + 1, generator=g, device="cuda") * 2 - 1,
                              torch.rand(n // 2 + 1, generator=g, device="cuda") * 2 - 1)
            y = torch.empty(n, device="cuda")
            kind = "rinv"
        else:
            x = torch.complex(torch.rand(n, generator=g, device="cuda") * 2 - 1,
                              torch.rand(n, generator=g, device="cuda") * 2 - 1)
            y = torch.empty_like(x)
            kind = "cinv" if inv else "cfwd"
        jobs.append((kind, n, 1, x, y))
    return jobs


ORACLE_KIND = {"cfwd": 0, "cinv": 1, "rfwd": 2, "rinv": 3}


def time_cpu_jobs(groups, min_seconds=2.0):
    """The reference's scalar path (oracle port) over jobs grouped by (kind, n):
    groups maps (kind, n) -> host input array (rows = transforms).  Every host
    thread runs its own share of each group; repeated until min_seconds."""
    import numpy as np
    from oracle import oracle as orc

    orc.build(with_reference=False)
    threads = os.cpu_count() or 1
    o = orc.Oracle(max(n for _, n in groups), fast=True)
    outs = {}
    for (kind, n), xs in groups.items():
        rows = xs.shape[0]
        outs[(kind, n)] = (np.empty((rows, n // 2 + 1), np.complex64) if kind == "rfwd"
                           else np.empty((rows, n), np.float32) if kind == "rinv"
                           else np.empty((rows, n), np.complex64))
    from ckfft_gb300 import workloads as wl

    algo = sum(xs.shape[0] * wl.algorithmic_bytes(kind in ("rfwd", "rinv"), n) for (kind, n), xs in groups.items())
    count = sum(xs.shape[0] for xs in groups.values())
    reps, t0 = 0, time.perf_counter()
    while True:
        for (kind, n), xs in groups.items():
            o.batch_into(ORACLE_KIND[kind], n, xs.shape[0], xs, outs[(kind, n)], threads)
        reps += 1
        if time.perf_counter() - t0 >= min_seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": round(reps * algo / dt / 1e9, 3), "unit": "GB/s", "cores": threads, "kind": "port",
            "transforms_per_s": round(reps * count / dt, 1), "reps": reps, "seconds": round(dt, 3)}


def measure_w4(args):
    """Workload 4: 10000 transforms of uneven sizes in one graph replay (the persistent job
    kernel plus grouped launches over pointer tables), against the plain path of one CkFft*
    call per transform and against the reference's scalar path on the host cores."""
    import numpy as np
    import torch
    from ckfft_gb300 import binding
    from ckfft_gb300 import workloads as wl

    ctx = binding.Context(1 << 16)
    g = torch.Generator(device="cuda")
    g.manual_seed(wl.W4_SEED)
    jobs = w4_jobs(torch, g)
    plan = ctx.plan(jobs)
    stream = torch.cuda.Stream()
    for _ in range(max(args.warmup, 3)):
        ctx.check(plan.exec(stream))
    torch.cuda.synchronize()
    # gate: every job of two sizes (complex 2^16 forward, real 2^16 inverse) and a
    # spread of others against the oracle
    gate = w4_gate(jobs)
    launches0 = binding.launch_count()
    secs = timed_steps(torch, stream, lambda: ctx.check(plan.exec(stream)), args.steps)
    launches = binding.launch_count() - launches0
    value = args.steps * plan.bytes / secs / 1e9
    tps = args.steps * len(jobs) / secs
    tmp = torch.empty((1 << 15) + 1, dtype=torch.complex64, device="cuda")

    def per_call():
        for kind, n, _, x, y in jobs:
            if kind == "cfwd":
                ctx.complex_forward(n, x, y)
            elif kind == "cinv":
                ctx.complex_inverse(n, x, y)
            elif kind == "rfwd":
                ctx.real_forward(n, x, y)
            else:
                ctx.real_inverse(n, x, y, tmp)
    pc = None
    if not args.no_percall:
        per_call()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        per_call()
        torch.cuda.synchronize()
        pc = time.perf_counter() - t0
    peak, src = measured_peaks()
    out = {"metric": "uneven batch FFT GB/s (10000 transforms, log2 n 6..16, mixed kinds)",
           "value": round(value, 2), "unit": "GB/s", "steps": args.steps, "ms_per_step": round(secs / args.steps * 1e3, 4),
           "frac_of_hbm": round(value / peak, 4), "peak": peak, "peak_source": src,
           "transforms_per_s": round(tps, 1), "gpu_launches": launches, "oracle_gate": gate,
           "config": {"workload": "10000 transforms, log2 n uniform 6..16, 70% complex / 30% real, 50% inverse, "
                                  "U[-1,1) inputs, one CUDA-graph replay per step",
                      "jobs": len(jobs), "bytes_per_step": plan.bytes,
                      "l2": f"{plan.bytes / 1e9:.2f} GB of algorithmic traffic per step (larger than L2)"}}
    if pc is not None:
        out["per_call"] = {"transforms_per_s": round(len(jobs) / pc, 1), "gbs": round(plan.bytes / pc / 1e9, 2),
                           "api": "one CkFftComplex*/CkFftReal* call per transform (device pointers, blocking)",
                           "speedup_of_plan": round(tps / (len(jobs) / pc), 1)}
    if not args.no_cpu:
        groups = {}
        for kind, n, _, x, _ in jobs:
            groups.setdefault((kind, n), []).append(x.cpu().numpy())
        groups = {k: np.ascontiguousarray(np.stack(v)) for k, v in groups.items()}
        cpu = time_cpu_jobs(groups)
        cpu["sample"] = (f"all {len(jobs)} jobs of the batch (inputs copied to the host), grouped by kind and size, "
                         f"repeated {cpu.pop('reps')} times in {cpu.pop('seconds')} s on {cpu['cores']} threads")
        out["cpu_baseline"] = cpu
    plan.close()
    ctx.close()
    return out


def w4_gate(jobs, per_group=4):
    """A few transforms of every (kind, size) of the uneven batch against the oracle."""
    from oracle import oracle as orc

    orc.build(with_reference=False)
    o = orc.Oracle(1 << 16)
    seen, worst = {}, 0.0
    for kind, n, _, x, y in jobs:
        if seen.get((kind, n), 0) >= per_group:
            continue
        seen[(kind, n)] = seen.get((kind, n), 0) + 1
        xh = x.cpu().numpy()
        ref = (o.complex(n, xh, kind == "cinv") if kind in ("cfwd", "cinv")
               else o.real_forward(n, xh) if kind == "rfwd" else o.real_inverse(n, xh))
        e = orc.rel_l2(y.cpu().numpy(), ref)
        if not e <= 1e-5:
            raise SystemExit(f"w4 oracle gate: {kind} n={n} rel L2 {e:.3e}: refusing to report a number")
        worst = max(worst, e)
    return {"checked": sum(seen.values()), "groups": len(seen), "worst_rel_l2": worst}


def run_w4(args):
    out = measure_w4(args)
    line = base_line(args, out["metric"], out["value"], "GB/s", out["ms_per_step"] * args.steps / 1e3, out["config"])
    peak = out["peak"]
    line["roofline"] = {"bound": "hbm", "kernel": "one graph: k_jobs + grouped launches over pointer tables",
                        "achieved": out["value"], "peak": peak, "unit": "GB/s", "frac": out["frac_of_hbm"],
                        "peak_source": out["peak_source"], "traffic": None}
    for k in ("transforms_per_s", "per_call", "gpu_launches", "cpu_baseline", "oracle_gate"):
        if k in out:
            line[k] = out[k]
    print(json.dumps(line), flush=True)


def w5_requests(nreq, seed):
    """(kind, n, frames) of the serving workload: 2^k points, k uniform in 8..20,
    1-64 frames, complex / real and forward / inverse with equal odds."""
    import numpy as np
    from ckfft_gb300 import workloads as wl

    rng = np.random.default_rng(seed)
    lo, hi = wl.W5_LOG2
    l2 = rng.integers(lo, hi + 1, nreq)
    frames = rng.integers(1, 65, nreq)
    real = rng.uniform(size=nreq) < 0.5
    inv = rng.uniform(size=nreq) < 0.5
    kinds = [("rinv" if i else "rfwd") if r else ("cinv" if i else "cfwd") for r, i in zip(real, inv)]
    return [(k, 1 << int(a), int(c)) for k, a, c in zip(kinds, l2, frames)]


def io_bytes(kind, n, c):
    fin = 4 * n if kind == "rfwd" else 8 * (n // 2 + 1) if kind == "rinv" else 8 * n
    fout = 8 * (n // 2 + 1) if kind == "rfwd" else 4 * n if kind == "rinv" else 8 * n
    return c * fin, c * fout


def place(spec, in_base, in_cap, out_base, out_cap):
    """Gives each request its own input and output window in two pools, in
    order, wrapping to the start when a pool is used up (a pool is far larger
    than L2, so no request finds its input in L2 from an earlier one)."""
    reqs, oi, oo = [], 0, 0
    for kind, n, c in spec:
        bi, bo = io_bytes(kind, n, c)
        bi, bo = (bi + 255) // 256 * 256, (bo + 255) // 256 * 256
        if oi + bi > in_cap:
            oi = 0
        if oo + bo > out_cap:
            oo = 0
        reqs.append((kind, n, c, in_base + oi, out_base + oo))
        oi += bi
        oo += bo
    return reqs


def batched_peak(torch, ctx, reqs, host):
    """GB/s of the request mix through the batched entry points, back to back:
    device buffers asynchronously on one stream (CUDA events), host buffers
    with the blocking staged calls (wall clock)."""
    from ckfft_gb300 import workloads as wl

    algo = sum(wl.algorithmic_bytes(k in ("rfwd", "rinv"), n) * c for k, n, c, _, _ in reqs)
    if host:
        for k, n, c, i, o in reqs[:8]:
            ctx.check(ctx.batch(k, n, c, i, o))
        t0 = time.perf_counter()
        for k, n, c, i, o in reqs:
            ctx.check(ctx.batch(k, n, c, i, o))
        return algo / (time.perf_counter() - t0) / 1e9
    stream = torch.cuda.Stream()

    def step():
        for k, n, c, i, o in reqs:
            ctx.check(ctx.batch(k, n, c, i, o, stream))
    step()
    return algo / timed_steps(torch, stream, step, 1) / 1e9


def w5_gate(srv, reqs, src, dst, count=24):
    """The first requests (before any window wraps) through the server, the
    first frame of each against the oracle.  src / dst: the pools (device or
    page-locked host tensors) the requests' pointers point into."""
    import numpy as np
    from oracle import oracle as orc
    from ckfft_gb300 import binding

    orc.build(with_reference=False)
    o = orc.Oracle(1 << 20)
    import torch

    sb, db = src.view(-1).view(torch.uint8), dst.view(-1).view(torch.uint8)
    worst = 0.0
    for k, n, c, i, out in reqs[:count]:
        ok, _ = srv.wait(srv.submit(k, n, c, i, out), 60.0)
        if not ok:
            raise SystemExit(f"w5 gate: server request failed: {binding.last_error()}")
        bi, bo = io_bytes(k, n, c)
        oi, oo = i - src.data_ptr(), out - dst.data_ptr()
        xin = sb[oi:oi + bi // c].cpu().numpy()
        yout = db[oo:oo + bo // c].cpu().numpy()
        if k in ("cfwd", "cinv"):
            ref, got = o.complex(n, xin.view(np.complex64), k == "cinv"), yout.view(np.complex64)
        elif k == "rfwd":
            ref, got = o.real_forward(n, xin.view(np.float32)), yout.view(np.complex64)
        else:
            ref, got = o.real_inverse(n, xin.view(np.complex64)), yout.view(np.float32)
        e = orc.rel_l2(got, ref)
        if not e <= 1e-5:
            raise SystemExit(f"w5 gate: {k} n={n} rel L2 {e:.3e}: refusing to report a number")
        worst = max(worst, e)
    return {"checked": min(count, len(reqs)), "worst_rel_l2": worst}


def serve_sweep(torch, ctx, srv, reqs, peak_gbs, loads, seed):
    """Poisson arrivals at each offered load (fraction of peak_gbs): the server
    replay and the one-call-per-request replay of the same trace."""
    import numpy as np
    from ckfft_gb300 import binding
    from ckfft_gb300 import workloads as wl

    mean_bytes = sum(wl.algorithmic_bytes(k in ("rfwd", "rinv"), n) * c for k, n, c, _, _ in reqs) / len(reqs)
    rows = []
    for f in loads:
        rate = f * peak_gbs * 1e9 / mean_bytes
        t = np.cumsum(np.random.default_rng(seed + int(f * 100)).exponential(1.0 / rate, len(reqs)))
        t -= t[0]
        trace = [(float(ti),) + r for ti, r in zip(t, reqs)]
        ok1, _, s1 = srv.replay(trace)
        ok2, _, s2 = binding.replay_per_request(ctx, trace)
        if not (ok1 and ok2):
            raise SystemExit(f"replay failed: {binding.last_error()}")
        row = {"load": f, "offered_req_per_s": round(rate, 1), "offered_gbs": round(f * peak_gbs, 1)}
        for name, sx in (("server", s1), ("per_request", s2)):
            row[name] = {"p50_ms": round(sx["p50_s"] * 1e3, 4), "p99_ms": round(sx["p99_s"] * 1e3, 4),
                         "p999_ms": round(sx["p999_s"] * 1e3, 4), "max_ms": round(sx["max_s"] * 1e3, 4),
                         "throughput_gbs": round(sx["algo_bytes"] / sx["seconds"] / 1e9, 1)}
        rows.append(row)
    return rows


def time_cpu_requests(spec, min_seconds=2.0):
    """The reference's scalar path (oracle port) on requests of the serving mix,
    taken in order until min_seconds of work: GB/s over those requests."""
    import numpy as np
    from oracle import oracle as orc
    from ckfft_gb300 import workloads as wl

    orc.build(with_reference=False)
    threads = os.cpu_count() or 1
    o = orc.Oracle(1 << 20, fast=True)
    rng = np.random.default_rng(1)
    done_b, done_r, t_work = 0, 0, 0.0
    for kind, n, c in spec:
        if kind == "rfwd":
            x = rng.standard_normal((c, n), dtype=np.float32)
            y = np.empty((c, n // 2 + 1), np.complex64)
        elif kind == "rinv":
            x = (rng.standard_normal((c, n // 2 + 1)) + 1j * rng.standard_normal((c, n // 2 + 1))).astype(np.complex64)
            y = np.empty((c, n), np.float32)
        else:
            x = (rng.standard_normal((c, n)) + 1j * rng.standard_normal((c, n))).astype(np.complex64)
            y = np.empty((c, n), np.complex64)
        t0 = time.perf_counter()
        o.batch_into(ORACLE_KIND[kind], n, c, x, y, threads)
        t_work += time.perf_counter() - t0
        done_b += wl.algorithmic_bytes(kind in ("rfwd", "rinv"), n) * c
        done_r += 1
        if t_work >= min_seconds:
            break
    return {"value": round(done_b / t_work / 1e9, 3), "unit": "GB/s", "cores": threads, "kind": "port",
            "requests_per_s": round(done_r / t_work, 1),
            "sample": f"the first {done_r} requests of the serving mix (N(0,1) inputs), {t_work:.2f} s of transform "
                      f"time on {threads} threads, each request's frames spread over the threads"}


def measure_w5(args, loads=(0.1, 0.3, 0.5, 0.7, 0.9), host_requests=2000):
    """Workload 5: Poisson request streams (2^k points, k in 8..20, 1-64 frames,
    mixed complex/real, N(0,1) inputs) at 10-90% of the peak offered load,
    through the continuous-batching server and through one call per request.
    Peak offered load = the batched throughput of the same request mix through
    CkFftCuda*Batch.  Every request reads its own input window and writes its
    own output window of pools far larger than L2.  Device-resident requests
    at every load; page-locked host requests (staged by the server, every byte
    crossing the CPU-GPU link inside the latency) at 50%."""
    import torch
    from ckfft_gb300 import binding
    from ckfft_gb300 import workloads as wl

    nreq = args.requests
    spec = w5_requests(nreq, wl.W5_SEED)
    ctx = binding.Context(1 << wl.W5_LOG2[1])
    g = torch.Generator(device="cuda")
    g.manual_seed(wl.W5_SEED)
    pool_b = 8 << 30
    src = torch.randn(pool_b // 4, generator=g, device="cuda")
    dst = torch.empty(pool_b // 4, device="cuda")
    reqs = place(spec, src.data_ptr(), pool_b, dst.data_ptr(), pool_b)
    algo = sum(wl.algorithmic_bytes(k in ("rfwd", "rinv"), n) * c for k, n, c in spec)
    srv = binding.Server(ctx, scratch_budget_bytes=4 << 30, max_inflight=2, direct_threshold_bytes=args.direct_mb << 20)
    gate = w5_gate(srv, reqs, src, dst)
    peak = batched_peak(torch, ctx, reqs, host=False)
    srv.replay([(0.0,) + r for r in reqs[:200]])                         # warm-up
    rows = serve_sweep(torch, ctx, srv, reqs, peak, loads, 100)
    srv.close()
    # page-locked host requests at 50% of their own batched peak
    hb = 4 << 30
    hsrc = torch.empty(hb // 4).pin_memory()
    hsrc.copy_(src[: hb // 4])
    hdst = torch.empty(hb // 4).pin_memory()
    del src, dst
    torch.cuda.empty_cache()
    hspec = spec[:host_requests]
    hreqs = place(hspec, hsrc.data_ptr(), hb, hdst.data_ptr(), hb)
    srv = binding.Server(ctx, scratch_budget_bytes=4 << 30, max_inflight=2, direct_threshold_bytes=args.direct_mb << 20)
    hgate = w5_gate(srv, hreqs, hsrc, hdst, count=8)
    hpeak = batched_peak(torch, ctx, hreqs, host=True)
    srv.replay([(0.0,) + r for r in hreqs[:50]])
    hrows = serve_sweep(torch, ctx, srv, hreqs, hpeak, (0.5,), 200)
    srv.close()
    ctx.close()
    mid = next(r for r in rows if r["load"] == 0.5)
    out = {"metric": "served p99 latency at 50% of peak offered load", "value": mid["server"]["p99_ms"], "unit": "ms",
           "higher_is_better": False, "peak_gbs": round(peak, 1), "peak_definition":
               "batched throughput of the same request mix through CkFftCuda*Batch (device buffers, back to back)",
           "mean_request_mb": round(algo / nreq / 1e6, 2), "requests_per_load": nreq, "loads": rows,
           "oracle_gate": gate,
           "host_resident": {"requests": len(hreqs), "peak_gbs": round(hpeak, 1), "loads": hrows, "oracle_gate": hgate,
                             "peak_definition": "batched throughput of the same mix through CkFftCuda*Batch from "
                                                "page-locked host buffers (blocking, staged over the CPU-GPU link)"},
           "config": {"workload": f"{nreq} requests per load, size 2^k with k uniform in {wl.W5_LOG2[0]}..{wl.W5_LOG2[1]}, "
                                  "1-64 frames, 50% real / 50% complex, 50% inverse, N(0,1) inputs, Poisson arrivals",
                      "server": f"2 job-kernel runs in flight, requests >= {args.direct_mb} MiB on 2 direct lanes, "
                                "4 GiB scratch budget",
                      "inputs": "each request reads its own window of an 8 GiB pool (device) / 4 GiB pool (host), "
                                "wrapping only after the pool is used up"}}
    if not args.no_cpu:
        out["cpu_baseline"] = time_cpu_requests(spec)
    return out


def run_w5(args):
    out = measure_w5(args)
    line = {"metric": out["metric"], "value": out["value"], "unit": "ms", "n_gpus": 1, "steps": len(out["loads"]),
            "warmup": 1, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded N(0,1) inputs)", "config": out["config"]}
    for k in ("peak_gbs", "peak_definition", "mean_request_mb", "requests_per_load", "loads", "host_resident",
              "oracle_gate", "cpu_baseline"):
        if k in out:
            line[k] = out[k]
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    world_env = int(os.environ.get("WORLD_SIZE", "1"))
    if args.gpus != world_env:
        sys.stderr.write(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={world_env}; launch one rank per GPU with "
                         f"`python -m torch.distributed.run --nproc-per-node {args.gpus} bench.py --gpus {args.gpus}`\n")
        raise SystemExit(2)
    if args.workload != "w2" and args.impl == "ours":
        {"w1": run_w1, "w3": run_w3, "w4": run_w4, "w5": run_w5, "sizes": run_sizes,
         "layouts": run_layouts}[args.workload](args)
        return
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
