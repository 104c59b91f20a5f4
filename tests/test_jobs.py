"""GPU tests of mixed runs (CkFftCudaPlanJobs / ExecPlan / RunJobs): many
transforms of different sizes, kinds and directions in one call or graph
replay (the persistent job kernel plus grouped launches over pointer tables).
Each result must equal the oracle within the parity bar, and must be the same
bits alone and in the mix."""
import numpy as np
import pytest

from conftest import assert_close

pytestmark = pytest.mark.gpu

OUT = {"cfwd": lambda n: (n, "c"), "cinv": lambda n: (n, "c"), "rfwd": lambda n: (n // 2 + 1, "c"),
       "rinv": lambda n: (n, "r")}
IN = {"cfwd": lambda n: (n, "c"), "cinv": lambda n: (n, "c"), "rfwd": lambda n: (n, "r"),
      "rinv": lambda n: (n // 2 + 1, "c")}


def make_job(torch, rng, kind, n, count):
    m, t = IN[kind](n)
    if t == "c":
        x = (rng.uniform(-1, 1, (count, m)) + 1j * rng.uniform(-1, 1, (count, m))).astype(np.complex64)
    else:
        x = rng.uniform(-1, 1, (count, m)).astype(np.float32)
    mo, to = OUT[kind](n)
    out = torch.full((count, mo), float("nan"), dtype=torch.complex64 if to == "c" else torch.float32, device="cuda")
    return {"kind": kind, "n": n, "count": count, "x": x, "xd": torch.from_numpy(x).cuda(), "out": out}


def oracle_out(o, j, f):
    kind, n, x = j["kind"], j["n"], j["x"][f]
    if kind == "cfwd":
        return o.complex(n, x, False)
    if kind == "cinv":
        return o.complex(n, x, True)
    if kind == "rfwd":
        return o.real_forward(n, x)
    return o.real_inverse(n, x)


def as_tuple(j):
    return (j["kind"], j["n"], j["count"], j["xd"], j["out"])


def mixed_jobs(torch, seed=0):
    rng = np.random.default_rng(seed)
    jobs = []
    for kind in ("cfwd", "cinv"):
        for l2 in range(0, 21):
            jobs.append(make_job(torch, rng, kind, 1 << l2, 2 if l2 <= 16 else 1))
    for kind in ("rfwd", "rinv"):
        for l2 in range(0, 22):
            jobs.append(make_job(torch, rng, kind, 1 << l2, 2 if l2 <= 16 else 1))
    order = rng.permutation(len(jobs))
    return [jobs[i] for i in order]


def test_mixed_run_matches_oracle(torch_cuda, ctx_cache, oracle_mod):
    jobs = mixed_jobs(torch_cuda)
    ctx = ctx_cache(1 << 21)
    ctx.check(ctx.run_jobs([as_tuple(j) for j in jobs]), "run_jobs")
    o = oracle_mod.Oracle(1 << 21)
    for j in jobs:
        got = j["out"].cpu().numpy()
        for f in range(j["count"]):
            ref = oracle_out(o, j, f)
            assert_close(got[f], ref, j["n"], f"{j['kind']} n={j['n']} frame {f}")


def test_same_alone_and_in_the_mix(torch_cuda, ctx_cache):
    jobs = mixed_jobs(torch_cuda, seed=1)
    ctx = ctx_cache(1 << 21)
    ctx.check(ctx.run_jobs([as_tuple(j) for j in jobs]), "mixed")
    mixed = [j["out"].clone() for j in jobs]
    for j, m in zip(jobs, mixed):
        j["out"].fill_(float("nan"))
        ctx.check(ctx.run_jobs([as_tuple(j)]), "alone")
        assert torch_cuda.equal(j["out"].view(torch_cuda.int32) if j["out"].dtype == torch_cuda.float32
                                else torch_cuda.view_as_real(j["out"]).view(torch_cuda.int32),
                                m.view(torch_cuda.int32) if m.dtype == torch_cuda.float32
                                else torch_cuda.view_as_real(m).view(torch_cuda.int32)), (j["kind"], j["n"])


def test_run_up_to_2e17(torch_cuda, ctx_cache, oracle_mod):
    """Every kind and size up to complex 2^17 / real 2^18 in one run: oracle
    parity, and the same bits as each job run alone."""
    torch = torch_cuda
    rng = np.random.default_rng(7)
    jobs = []
    for kind in ("cfwd", "cinv"):
        for l2 in range(0, 18):
            jobs.append(make_job(torch, rng, kind, 1 << l2, 3 if l2 <= 14 else 2))
    for kind in ("rfwd", "rinv"):
        for l2 in range(0, 19):
            jobs.append(make_job(torch, rng, kind, 1 << l2, 3 if l2 <= 15 else 2))
    jobs = [jobs[i] for i in rng.permutation(len(jobs))]
    ctx = ctx_cache(1 << 18)
    ctx.check(ctx.run_jobs([as_tuple(j) for j in jobs]), "mixed run")
    o = oracle_mod.Oracle(1 << 18)
    mixed = [j["out"].clone() for j in jobs]
    for j, m in zip(jobs, mixed):
        got = m.cpu().numpy()
        for f in range(j["count"]):
            assert_close(got[f], oracle_out(o, j, f), j["n"], f"mixed {j['kind']} n={j['n']} frame {f}")
        j["out"].fill_(float("nan"))
        ctx.check(ctx.run_jobs([as_tuple(j)]), "alone")
        a = j["out"].view(torch.int32) if j["out"].dtype == torch.float32 else torch.view_as_real(j["out"]).view(torch.int32)
        b = m.view(torch.int32) if m.dtype == torch.float32 else torch.view_as_real(m).view(torch.int32)
        assert torch.equal(a, b), (j["kind"], j["n"])


def test_plan_replays_and_reads_current_inputs(torch_cuda, ctx_cache, oracle_mod):
    torch = torch_cuda
    rng = np.random.default_rng(2)
    jobs = [make_job(torch, rng, k, n, c) for k, n, c in
            [("cfwd", 1024, 5), ("rinv", 4096, 3), ("cinv", 1 << 16, 2), ("rfwd", 1 << 17, 1), ("rinv", 1 << 18, 1)]]
    ctx = ctx_cache(1 << 18)
    plan = ctx.plan([as_tuple(j) for j in jobs])
    assert plan.bytes > 0
    ctx.check(plan.exec(), "exec 1")
    first = [j["out"].clone() for j in jobs]
    ctx.check(plan.exec(), "exec 2")
    for j, f in zip(jobs, first):
        assert torch.equal(torch.view_as_real(j["out"]) if j["out"].is_complex() else j["out"],
                           torch.view_as_real(f) if f.is_complex() else f)
    # new data in the same buffers: the replay transforms the current contents
    for j in jobs:
        m, t = IN[j["kind"]](j["n"])
        x = (rng.uniform(-1, 1, (j["count"], m)) + (1j * rng.uniform(-1, 1, (j["count"], m)) if t == "c" else 0))
        j["x"] = x.astype(np.complex64 if t == "c" else np.float32)
        j["xd"].copy_(torch.from_numpy(j["x"]))
    s = torch.cuda.Stream()
    ctx.check(plan.exec(s), "exec on stream")
    s.synchronize()
    o = oracle_mod.Oracle(1 << 18)
    for j in jobs:
        got = j["out"].cpu().numpy()
        for f in range(j["count"]):
            assert_close(got[f], oracle_out(o, j, f), j["n"], f"replay {j['kind']} {j['n']}")
    plan.close()


def test_plan_groups_multi_pass_sizes(torch_cuda, ctx_cache, oracle_mod):
    """Transforms the job kernel would split into pass units run as grouped
    launches over pointer tables (single-CTA tables at complex 2^13 / real
    2^15, the cluster kernel at complex 2^15 and for the real forward and
    inverse at 2^16, split / merge fused), beside the persistent kernel that
    takes the small ones: one replay launches exactly those kernels."""
    from ckfft_gb300 import binding
    torch = torch_cuda
    rng = np.random.default_rng(5)
    spec = [("cfwd", 1 << 13, 3), ("rfwd", 1 << 15, 2), ("cinv", 1 << 15, 3), ("rinv", 1 << 16, 2),
            ("rfwd", 1 << 16, 3), ("cfwd", 256, 7), ("rinv", 64, 5)]
    jobs = [make_job(torch, rng, k, n, c) for k, n, c in spec]
    ctx = ctx_cache(1 << 16)
    plan = ctx.plan([as_tuple(j) for j in jobs])
    before = binding.launch_count()
    ctx.check(plan.exec(), "exec")
    # 2 single-CTA tables + 3 cluster launches (complex 2^15, real 2^16 both ways) + the job kernel
    assert binding.launch_count() - before == 6
    o = oracle_mod.Oracle(1 << 16)
    for j in jobs:
        got = j["out"].cpu().numpy()
        for f in range(j["count"]):
            assert_close(got[f], oracle_out(o, j, f), j["n"], f"grouped {j['kind']} {j['n']}")
    plan.close()


def test_workload4_every_job(torch_cuda, ctx_cache, oracle_mod):
    """The uneven batch: 10000 transforms, log2 n in 6..16, 70% complex, 50%
    inverse, one graph replay; every job's output against the oracle (jobs of
    one kind and size checked together through the oracle's threaded batch)."""
    from conftest import assert_close_rows, host_threads
    from ckfft_gb300 import workloads as wl
    torch = torch_cuda
    orc = oracle_mod
    spec = wl.uneven_jobs()
    rng = np.random.default_rng(wl.W4_SEED)
    ctx = ctx_cache(1 << 16)
    jobs = []
    for real, inv, l2 in spec:
        kind = ("rinv" if inv else "rfwd") if real else ("cinv" if inv else "cfwd")
        jobs.append(make_job(torch, rng, kind, 1 << l2, 1))
    plan = ctx.plan([as_tuple(j) for j in jobs])
    ctx.check(plan.exec(), "workload 4")
    torch.cuda.synchronize()
    o = orc.Oracle(1 << 16)
    code = {"cfwd": orc.KIND_CFWD, "cinv": orc.KIND_CINV, "rfwd": orc.KIND_RFWD, "rinv": orc.KIND_RINV}
    groups = {}
    for idx, j in enumerate(jobs):
        groups.setdefault((j["kind"], j["n"]), []).append(idx)
    checked = 0
    for (kind, n), idxs in sorted(groups.items()):
        xs = np.stack([jobs[i]["x"][0] for i in idxs])
        got = torch.stack([jobs[i]["out"][0] for i in idxs]).cpu().numpy()
        ref = o.batch(code[kind], n, len(idxs), xs, host_threads())
        assert_close_rows(got, ref, n, f"workload 4 {kind} n={n}")
        checked += len(idxs)
    assert checked == len(jobs) == wl.W4_JOBS
    plan.close()


def test_job_validation(torch_cuda, ctx_cache, lib):
    torch = torch_cuda
    ctx = ctx_cache(1 << 10)
    a = torch.zeros(4096, dtype=torch.complex64, device="cuda")
    b = torch.zeros(4096, dtype=torch.complex64, device="cuda")
    h = torch.zeros(4096, dtype=torch.complex64)
    assert ctx.run_jobs([(0, 1 << 11, 1, a, b)]) == 0          # n > nMax
    assert ctx.run_jobs([(5, 64, 1, a, b)]) == 0               # bad kind
    assert ctx.run_jobs([(0, 48, 1, a, b)]) == 0               # not a power of two
    assert ctx.run_jobs([(0, 64, 1, h, b)]) == 0               # host memory
    assert "device" in lib.CkFftCudaGetLastError().decode()
    assert ctx.run_jobs([(0, 64, 1, a, a)]) == 0               # in place
    assert ctx.run_jobs([(0, 64, -1, a, b)]) == 0
    assert ctx.run_jobs([(0, 64, 0, a, b)]) == 1               # nothing to do
    assert ctx.run_jobs([]) == 1
