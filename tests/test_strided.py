"""Advanced-layout batches (CkFftCuda*Strided) against the contiguous batch
path (bit-identical: the same frame bodies, only the addressing differs) and
against the oracle, for every layout family the header names: interleaved
channels, matrix columns, overlapping frames at even and odd hops, padded
rows, broadcast input, sizes that gather and scatter, and page-locked host
buffers; plus the layout validation."""
import numpy as np
import pytest

from ckfft_gb300 import binding
from conftest import assert_close

pytestmark = pytest.mark.gpu

ELEM = {"cfwd": (np.complex64, np.complex64), "cinv": (np.complex64, np.complex64),
        "rfwd": (np.float32, np.complex64), "rinv": (np.complex64, np.float32)}


def counts(kind, n):
    """Elements per transform on the input and output side."""
    if kind == "rfwd":
        return n, n // 2 + 1
    if kind == "rinv":
        return n // 2 + 1, n
    return n, n


def make_input(rng, kind, size):
    dt = ELEM[kind][0]
    if dt == np.float32:
        return rng.uniform(-1, 1, size).astype(np.float32)
    return (rng.uniform(-1, 1, size) + 1j * rng.uniform(-1, 1, size)).astype(np.complex64)


def gather(buf, count, length, stride, dist):
    f = np.arange(count)[:, None] * dist + np.arange(length)[None, :] * stride
    return buf[f]


def run_case(torch, ctx, kind, n, count, is_, id_, os_, od_, seed=0, where="device"):
    """Returns (strided result as rows, contiguous-batch result, input rows)."""
    ni, no = counts(kind, n)
    rng = np.random.default_rng(seed)
    in_len = (count - 1) * id_ + (ni - 1) * is_ + 1
    out_len = (count - 1) * od_ + (no - 1) * os_ + 1
    src = make_input(rng, kind, in_len)
    tdt = {np.float32: torch.float32, np.complex64: torch.complex64}
    if where == "device":
        xi = torch.from_numpy(src).cuda()
        yo = torch.zeros(out_len, dtype=tdt[ELEM[kind][1]], device="cuda")
    else:
        xi = torch.from_numpy(src).pin_memory()
        yo = torch.zeros(out_len, dtype=tdt[ELEM[kind][1]]).pin_memory()
    ctx.check(ctx.strided(kind, n, count, xi, is_, id_, yo, os_, od_), f"{kind} n={n} layout")
    got = gather(yo.cpu().numpy(), count, no, os_, od_)
    rows = np.ascontiguousarray(gather(src, count, ni, is_, id_))
    xr = torch.from_numpy(rows).cuda()
    ref = torch.zeros((count, no), dtype=tdt[ELEM[kind][1]], device="cuda")
    ctx.check(ctx.batch(kind, n, count, xr, ref))
    return got, ref.cpu().numpy(), rows


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


LAYOUTS = [
    # name, kind, n, count, in_stride, in_dist, out_stride, out_dist
    ("channels-8", "cfwd", 1024, 8, 8, 1, 8, 1),
    ("channels-6-real", "rfwd", 2048, 6, 6, 1, 1, 1025),
    ("channels-out-real-inv", "rinv", 512, 4, 1, 257, 4, 1),
    ("matrix-columns", "cinv", 256, 512, 512, 1, 1, 256),
    ("stft-hop-256", "rfwd", 1024, 40, 1, 256, 1, 513),
    ("stft-odd-hop", "rfwd", 1024, 33, 1, 255, 1, 513),
    ("padded-rows", "cfwd", 4096, 7, 1, 4100, 1, 4103),
    ("odd-out-dist-real-inv", "rinv", 4096, 5, 1, 2049, 1, 4097),
    ("stride-3-both", "cinv", 64, 50, 3, 3 * 64, 2, 2 * 64),
    ("broadcast", "cfwd", 2048, 4, 1, 0, 1, 2048),
    ("smallest-complex", "cfwd", 1, 9, 2, 3, 3, 1),
    ("real-8", "rinv", 8, 100, 2, 11, 1, 8),
    ("real-2^15-columns", "rfwd", 1 << 15, 3, 3, 1, 1, (1 << 14) + 1),
    ("complex-2^14-stride", "cfwd", 1 << 14, 3, 2, 1 << 15, 1, 1 << 14),
    # consecutive transforms adjacent (distance 1): CTAs move whole rows
    ("inter-2^13-both", "cfwd", 1 << 13, 5, 5, 1, 5, 1),
    ("inter-2^12-in", "cinv", 1 << 12, 7, 9, 1, 1, 1 << 12),
    ("inter-2^11-out", "cfwd", 1 << 11, 3, 1, 1 << 11, 3, 1),
    ("inter-64-both", "cinv", 64, 100, 100, 1, 101, 1),
    ("inter-real-2^14-in", "rfwd", 1 << 14, 3, 3, 1, 1, (1 << 13) + 1),
    ("inter-real-2^14-out", "rinv", 1 << 14, 5, 1, (1 << 13) + 1, 5, 1),
    ("inter-real-128-in", "rfwd", 128, 70, 70, 1, 2, 130),
    ("inter-real-128-out", "rinv", 128, 65, 1, 65, 65, 1),
    ("inter-real-4096-in-out-strided", "rfwd", 4096, 9, 9, 1, 9, 1),
    # distance 1 beyond the distance-1 kernels: transposed chunks through
    # contiguous rows (50 transforms of 2^16: chunks of 32 and 18)
    ("transposed-2^16-both-two-chunks", "cfwd", 1 << 16, 50, 50, 1, 51, 1),
    ("transposed-2^14-in", "cinv", 1 << 14, 40, 41, 1, 1, 1 << 14),
    ("transposed-real-2^16-out", "rinv", 1 << 16, 33, 1, (1 << 15) + 1, 33, 1),
    ("transposed-real-2^18-in", "rfwd", 1 << 18, 3, 3, 1, 1, (1 << 17) + 1),
]


@pytest.mark.parametrize("name,kind,n,count,is_,id_,os_,od_", LAYOUTS, ids=[l[0] for l in LAYOUTS])
def test_layouts_match_contiguous_and_oracle(torch_cuda, ctx_cache, oracle_mod, name, kind, n, count, is_, id_,
                                             os_, od_):
    ctx = ctx_cache(max(n, 8))
    got, ref, rows = run_case(torch_cuda, ctx, kind, n, count, is_, id_, os_, od_, seed=len(name))
    assert np.array_equal(bits(got), bits(ref)), name
    o = oracle_mod.Oracle(max(n, 8))
    for f in range(0, count, max(1, count // 4)):
        if kind == "rfwd":
            want = o.real_forward(n, rows[f])
        elif kind == "rinv":
            want = o.real_inverse(n, rows[f])
        else:
            want = o.complex(n, rows[f], kind == "cinv")
        if n <= 2:
            assert np.array_equal(bits(got[f]), bits(want))
        else:
            assert_close(got[f], want, n, f"{name} frame {f}")


@pytest.mark.parametrize("kind,n,is_,os_", [("cfwd", 1 << 16, 2, 1), ("cinv", 1 << 18, 1, 3),
                                            ("rfwd", 1 << 17, 2, 1), ("rinv", 1 << 16, 1, 2),
                                            ("rfwd", 4, 3, 1), ("rinv", 2, 1, 2)])
def test_gather_scatter_sizes(torch_cuda, ctx_cache, kind, n, is_, os_):
    """Multi-pass and closed-form sizes run gather -> contiguous -> scatter."""
    ctx = ctx_cache(max(n, 8))
    ni, no = counts(kind, n)
    count = 3
    got, ref, _ = run_case(torch_cuda, ctx, kind, n, count, is_, ni * is_ + 5, os_, no * os_ + 1, seed=n)
    assert np.array_equal(bits(got), bits(ref))


def test_page_locked_host_layout(torch_cuda, ctx_cache):
    ctx = ctx_cache(1024)
    got, ref, _ = run_case(torch_cuda, ctx, "cfwd", 1024, 8, 8, 1, 8, 1, seed=3, where="pinned")
    assert np.array_equal(bits(got), bits(ref))
    ctx = ctx_cache(1 << 17)
    got, ref, _ = run_case(torch_cuda, ctx, "rfwd", 1 << 17, 2, 2, 1, 1, (1 << 16) + 1, seed=4, where="pinned")
    assert np.array_equal(bits(got), bits(ref))


def test_async_on_user_stream(torch_cuda, ctx_cache):
    torch = torch_cuda
    n, ch = 2048, 8
    ctx = ctx_cache(n)
    rng = np.random.default_rng(5)
    x = torch.from_numpy(make_input(rng, "cfwd", n * ch)).cuda()
    y = torch.zeros(n * ch, dtype=torch.complex64, device="cuda")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    ctx.check(ctx.strided("cfwd", n, ch, x, ch, 1, y, ch, 1, s))
    s.synchronize()
    ref = torch.zeros((ch, n), dtype=torch.complex64, device="cuda")
    ctx.check(ctx.batch("cfwd", n, ch, x.view(n, ch).t().contiguous(), ref))
    assert np.array_equal(bits(y.view(n, ch).t().cpu().numpy()), bits(ref.cpu().numpy()))


def test_layout_validation(torch_cuda, ctx_cache):
    torch = torch_cuda
    ctx = ctx_cache(1024)
    x = torch.zeros(1 << 16, dtype=torch.complex64, device="cuda")
    y = torch.zeros(1 << 16, dtype=torch.complex64, device="cuda")
    assert ctx.strided("cfwd", 1024, 2, x, 0, 1024, y, 1, 1024) == 0        # stride 0
    assert ctx.strided("cfwd", 1024, 2, x, 1, -1, y, 1, 1024) == 0          # negative distance
    assert ctx.strided("cfwd", 1024, 2, x, 1, 1024, y, 1, 512) == 0         # output frames overlap
    assert "overlap" in binding.last_error()
    assert ctx.strided("cfwd", 1024, 2, x, 1, 1024, y, 1, 1) == 0           # interleaved, stride too small
    assert ctx.strided("cfwd", 1024, 2, x, 2, 1, y, 2, 1) == 1              # interleaved pair: fine
    assert ctx.strided("cfwd", 1024, 2, x, 1, 1024, x[1000:], 1, 1024) == 0  # input and output intersect
    assert ctx.strided("cfwd", 1000, 2, x, 1, 1024, y, 1, 1024) == 0        # not a power of two
    assert ctx.strided("cfwd", 1024, 0, x, 1, 1024, y, 1, 1024) == 1        # empty batch
    assert ctx.strided("cfwd", 1024, -1, x, 1, 1024, y, 1, 1024) == 0



def test_pageable_host_layout_is_staged(torch_cuda, ctx_cache):
    """Pageable buffers: the layout's spans are staged through device memory;
    the gaps of a strided output keep their contents."""
    ctx = ctx_cache(1024)
    rng = np.random.default_rng(8)
    x = (rng.uniform(-1, 1, 4 * 1024) + 1j * rng.uniform(-1, 1, 4 * 1024)).astype(np.complex64)
    out = np.full(8 * 1024, 7 + 7j, np.complex64)
    ctx.check(ctx.strided("cfwd", 1024, 4, x, 4, 1, out, 2, 2048))
    xd = torch_cuda.from_numpy(x).cuda()
    yd = torch_cuda.full((8 * 1024,), 7 + 7j, dtype=torch_cuda.complex64, device="cuda")
    ctx.check(ctx.strided("cfwd", 1024, 4, xd, 4, 1, yd, 2, 2048))
    assert np.array_equal(bits(out), bits(yd.cpu().numpy()))
    assert np.all(out[1::2] == 7 + 7j)
