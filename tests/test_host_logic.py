"""CPU tests of host-side logic: workload generators, byte accounting, the
multi-rank combination of the benchmark (gloo, world size 2), and the
replica sharding of frames."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from ckfft_gb300 import workloads as wl


def test_workload_generators_are_seeded_and_shaped():
    a = wl.complex_uniform(3, 64, seed=0)
    b = wl.complex_uniform(3, 64, seed=0)
    assert a.dtype == np.complex64 and a.shape == (3, 64) and np.array_equal(a, b)
    assert np.all(np.abs(a.real) <= 1) and np.all(np.abs(a.imag) <= 1)
    s = wl.sine_frames(4, 256, seed=2)
    assert s.dtype == np.float32 and s.shape == (4, 256)
    assert np.max(np.abs(s)) <= 8.2                     # 8 tones of amplitude <= 1 plus small noise
    t = wl.sine_frames_torch(4, 256, seed=2, device="cpu")
    assert tuple(t.shape) == (4, 256) and t.dtype == torch.float32
    jobs = wl.uneven_jobs(2000, seed=4)
    l2 = np.array([j[2] for j in jobs])
    assert l2.min() == 6 and l2.max() == 16
    assert 0.25 < np.mean([j[0] for j in jobs]) < 0.35   # 30% real
    assert 0.45 < np.mean([j[1] for j in jobs]) < 0.55   # 50% inverse
    reqs = wl.serving_requests(500, 1000.0)
    assert all(8 <= r[3] <= 20 and 1 <= r[4] <= 64 for r in reqs)
    assert all(x <= y for x, y in zip([r[0] for r in reqs], [r[0] for r in reqs][1:]))


def test_algorithmic_bytes():
    assert wl.algorithmic_bytes(False, 1024) == 16 * 1024
    assert wl.algorithmic_bytes(True, 4096) == 4 * 4096 + 8 * 2049


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, secs, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    t, v = bench.combine_ranks(secs[rank], 1e9, world)
    out[rank] = (t, v)
    dist.barrier()
    dist.destroy_process_group()


def test_combine_ranks_takes_the_slowest_rank_gloo():
    """Two gloo ranks with different timed regions agree on max time and total bytes."""
    world, port = 2, _free_port()
    secs = [0.5, 2.0]
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(world, port, secs, out), nprocs=world, start_method="spawn")
    for r in range(world):
        t, v = out[r]
        assert t == 2.0
        assert v == pytest.approx(world * 1e9 / 2.0 / 1e9)


def _shard_main(rank, world, port, frames, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    sh = bench.frame_shard(rank, world, frames)
    mine = torch.tensor([sh["start"], sh["count"], sh["seed"]], dtype=torch.int64)
    every = [torch.zeros(3, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(every, mine)
    out[rank] = [tuple(int(v) for v in t) for t in every]
    dist.barrier()
    dist.destroy_process_group()


def test_frame_shards_are_disjoint_covering_and_seeded_per_rank_gloo():
    """Each of two gloo ranks takes its shard of the weak-scaling run; the
    gathered shards tile the job's frames exactly once, with one seed per rank."""
    world, port, frames = 2, _free_port(), 65536
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_shard_main, args=(world, port, frames, out), nprocs=world, start_method="spawn")
    assert out[0] == out[1]
    shards = sorted(out[0])
    covered = np.zeros(world * frames, np.int32)
    for start, count, _ in shards:
        covered[start:start + count] += 1
    assert np.all(covered == 1)
    assert len({seed for _, _, seed in shards}) == world


def test_bench_refuses_a_gpu_count_it_was_not_launched_with():
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--gpus", "2", "--steps", "1"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 2 and "WORLD_SIZE" in r.stderr, r.stderr
