"""ctypes binding of libckfft_cuda.so (include/ckfft_cuda.h).

This is plumbing for Python callers, tests and the benchmark: every call goes
through the C ABI into the CUDA kernels.  There is no Python or CPU fallback;
if the library is missing, `load()` raises.

Arrays may be numpy arrays (host memory) or torch tensors (host or CUDA);
anything exposing a data pointer works through the raw `call_*` helpers.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libckfft_cuda.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "ckfft_cuda.h")

FORWARD, INVERSE, BOTH = 1, 2, 3

_lib = None


class CkFftError(RuntimeError):
    """A CkFft call returned 0 / NULL; the message is CkFftCudaGetLastError()."""


def header_functions(header: str | None = None, prefix: str = "CkFft") -> list[str]:
    """Names of the functions declared in a public header (default
    include/ckfft_cuda.h) that start with `prefix`."""
    text = open(header or HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = "\n".join(l for l in text.splitlines() if not l.lstrip().startswith("#"))
    names = re.findall(r"\b(" + prefix + r"\w*)\s*\(", text)
    seen = []
    for n in names:
        if n not in seen:
            seen.append(n)
    return seen


def load(path: str | None = None):
    """Loads (once) and returns the CDLL with argument types declared."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError(f"{p} is missing: build it with `python -m ckfft_gb300.build`")
    lib = C.CDLL(p)
    vp, i, sz = C.c_void_p, C.c_int, C.c_size_t
    lib.CkFftInit.restype = vp
    lib.CkFftInit.argtypes = [i, i, vp, C.POINTER(sz)]
    lib.CkFftShutdown.restype = None
    lib.CkFftShutdown.argtypes = [vp]
    for f in ("CkFftComplexForward", "CkFftComplexInverse", "CkFftRealForward"):
        getattr(lib, f).restype = i
        getattr(lib, f).argtypes = [vp, i, vp, vp]
    lib.CkFftRealInverse.restype = i
    lib.CkFftRealInverse.argtypes = [vp, i, vp, vp, vp]
    lib.CkFftCudaGetLastError.restype = C.c_char_p
    lib.CkFftCudaGetLastError.argtypes = []
    for f in ("CkFftCudaComplexForwardBatch", "CkFftCudaComplexInverseBatch",
              "CkFftCudaRealForwardBatch", "CkFftCudaRealInverseBatch"):
        getattr(lib, f).restype = i
        getattr(lib, f).argtypes = [vp, i, i, vp, vp, vp]
    lib.CkFftCudaLaunchCount.restype = C.c_longlong
    lib.CkFftCudaLaunchCount.argtypes = []
    _declare_extras(lib)
    if path is None:
        _lib = lib
    return lib


def _declare_extras(lib):
    """Argument types of the later additions to the header, when present."""
    vp, i, ll = C.c_void_p, C.c_int, C.c_longlong
    if hasattr(lib, "CkFftCudaComplexBatchNoAlloc"):
        lib.CkFftCudaComplexBatchNoAlloc.restype = i
        lib.CkFftCudaComplexBatchNoAlloc.argtypes = [vp, i, i, i, vp, vp, vp]
    for f in ("CkFftCudaComplexForwardStrided", "CkFftCudaComplexInverseStrided",
              "CkFftCudaRealForwardStrided", "CkFftCudaRealInverseStrided"):
        if hasattr(lib, f):
            getattr(lib, f).restype = i
            getattr(lib, f).argtypes = [vp, i, ll, vp, ll, ll, vp, ll, ll, vp]
    if hasattr(lib, "CkFftCudaSelfTestWait"):
        lib.CkFftCudaSelfTestWait.restype = i
        lib.CkFftCudaSelfTestWait.argtypes = [vp, i]
    if hasattr(lib, "CkFftCudaStft"):
        lib.CkFftCudaStft.restype = i
        lib.CkFftCudaStft.argtypes = [vp, i, ll, vp, ll, ll, vp, C.c_float, vp, vp]
        lib.CkFftCudaFilterInverse.restype = i
        lib.CkFftCudaFilterInverse.argtypes = [vp, i, ll, vp, vp, C.c_float, vp, vp]
    if hasattr(lib, "kiss_fft_alloc"):
        for f in ("kiss_fft_alloc", "kiss_fftr_alloc"):
            getattr(lib, f).restype = vp
            getattr(lib, f).argtypes = [i, i, vp, C.POINTER(C.c_size_t)]
        for f in ("kiss_fft", "kiss_fftr", "kiss_fftri"):
            getattr(lib, f).restype = None
            getattr(lib, f).argtypes = [vp, vp, vp]
        lib.kiss_fft_stride.restype = None
        lib.kiss_fft_stride.argtypes = [vp, vp, vp, i]
        for f in ("kiss_fft_free", "kiss_fftr_free"):
            getattr(lib, f).restype = None
            getattr(lib, f).argtypes = [vp]
        lib.kiss_fft_next_fast_size.restype = i
        lib.kiss_fft_next_fast_size.argtypes = [i]
    if hasattr(lib, "CkFftCudaServerCreate"):
        lib.CkFftCudaServerCreate.restype = vp
        lib.CkFftCudaServerCreate.argtypes = [vp, C.c_size_t, i, ll]
        lib.CkFftCudaServerDestroy.restype = None
        lib.CkFftCudaServerDestroy.argtypes = [vp]
        lib.CkFftCudaServerSubmit.restype = ll
        lib.CkFftCudaServerSubmit.argtypes = [vp, vp]
        lib.CkFftCudaServerWait.restype = i
        lib.CkFftCudaServerWait.argtypes = [vp, ll, C.c_double, C.POINTER(C.c_double)]
        lib.CkFftCudaServerReplay.restype = i
        lib.CkFftCudaServerReplay.argtypes = [vp, vp, i, vp, vp]
        lib.CkFftCudaReplayPerRequest.restype = i
        lib.CkFftCudaReplayPerRequest.argtypes = [vp, vp, i, vp, vp]
    if hasattr(lib, "CkFftCudaRunJobs"):
        lib.CkFftCudaRunJobs.restype = i
        lib.CkFftCudaRunJobs.argtypes = [vp, vp, i, vp]
        lib.CkFftCudaPlanJobs.restype = vp
        lib.CkFftCudaPlanJobs.argtypes = [vp, vp, i]
        lib.CkFftCudaExecPlan.restype = i
        lib.CkFftCudaExecPlan.argtypes = [vp, vp]
        lib.CkFftCudaDestroyPlan.restype = None
        lib.CkFftCudaDestroyPlan.argtypes = [vp]
        lib.CkFftCudaPlanBytes.restype = ll
        lib.CkFftCudaPlanBytes.argtypes = [vp]


class Job(C.Structure):
    """CkFftCudaJob: `count` transforms of size n between device buffers."""
    _fields_ = [("kind", C.c_int), ("n", C.c_int), ("count", C.c_int),
                ("input", C.c_void_p), ("output", C.c_void_p)]


KIND = {"cfwd": 0, "cinv": 1, "rfwd": 2, "rinv": 3}


def job_array(jobs):
    """jobs: iterable of (kind, n, count, input, output) with kind a KIND key or int."""
    jobs = list(jobs)
    arr = (Job * max(1, len(jobs)))()
    for i, (kind, n, count, inp, out) in enumerate(jobs):
        arr[i] = Job(KIND.get(kind, kind), n, count, ptr(inp), ptr(out))
    return arr, len(jobs)


class Request(C.Structure):
    """CkFftCudaRequest: a job and its arrival time (seconds after the replay starts)."""
    _fields_ = [("arrival_s", C.c_double), ("job", Job)]


class ServeStats(C.Structure):
    _fields_ = [("requests", C.c_longlong), ("seconds", C.c_double), ("algo_bytes", C.c_double),
                ("p50_s", C.c_double), ("p99_s", C.c_double), ("p999_s", C.c_double), ("max_s", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def last_error() -> str:
    return load().CkFftCudaGetLastError().decode(errors="replace")


def ptr(a) -> int | None:
    """Raw data pointer of a numpy array or torch tensor (None passes NULL)."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    if hasattr(a, "ctypes"):
        return a.ctypes.data
    raise TypeError(f"cannot take the address of {type(a)}")


def launch_count() -> int:
    return load().CkFftCudaLaunchCount()


class Context:
    """Owns one CkFftContext (CkFftInit / CkFftShutdown)."""

    def __init__(self, nmax: int, direction: int = BOTH):
        self.lib = load()
        self.nmax = nmax
        self.direction = direction
        self.handle = self.lib.CkFftInit(nmax, direction, None, None)
        if not self.handle:
            raise CkFftError(f"CkFftInit({nmax}, {direction}) failed: {last_error()}")

    def close(self):
        if getattr(self, "handle", None):
            self.lib.CkFftShutdown(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- raw calls: pointers in, return code out (1 ok, 0 invalid/failed)
    def complex_forward(self, n, inp, out) -> int:
        return self.lib.CkFftComplexForward(self.handle, n, ptr(inp), ptr(out))

    def complex_inverse(self, n, inp, out) -> int:
        return self.lib.CkFftComplexInverse(self.handle, n, ptr(inp), ptr(out))

    def real_forward(self, n, inp, out) -> int:
        return self.lib.CkFftRealForward(self.handle, n, ptr(inp), ptr(out))

    def real_inverse(self, n, inp, out, tmp) -> int:
        return self.lib.CkFftRealInverse(self.handle, n, ptr(inp), ptr(out), ptr(tmp))

    def batch(self, kind: str, n: int, count: int, inp, out, stream=None) -> int:
        """kind: 'cfwd', 'cinv', 'rfwd', 'rinv'; stream: cudaStream_t as int or a torch stream."""
        fn = {
            "cfwd": self.lib.CkFftCudaComplexForwardBatch,
            "cinv": self.lib.CkFftCudaComplexInverseBatch,
            "rfwd": self.lib.CkFftCudaRealForwardBatch,
            "rinv": self.lib.CkFftCudaRealInverseBatch,
        }[kind]
        s = getattr(stream, "cuda_stream", stream)
        return fn(self.handle, n, count, ptr(inp), ptr(out), s)

    def strided(self, kind: str, n: int, count: int, inp, in_stride: int, in_dist: int,
                out, out_stride: int, out_dist: int, stream=None) -> int:
        """Advanced-layout batch: element p of transform f at inp[f*in_dist + p*in_stride]
        -> out[f*out_dist + p*out_stride] (elements of each side's type)."""
        fn = {
            "cfwd": self.lib.CkFftCudaComplexForwardStrided,
            "cinv": self.lib.CkFftCudaComplexInverseStrided,
            "rfwd": self.lib.CkFftCudaRealForwardStrided,
            "rinv": self.lib.CkFftCudaRealInverseStrided,
        }[kind]
        s = getattr(stream, "cuda_stream", stream)
        return fn(self.handle, n, count, ptr(inp), in_stride, in_dist, ptr(out), out_stride, out_dist, s)

    def stft(self, n: int, frames: int, signal, hop: int, frame_len: int, window, scale: float, out,
             stream=None) -> int:
        """CkFftCudaStft: windowed frames at `hop` -> real forward x scale."""
        s = getattr(stream, "cuda_stream", stream)
        return self.lib.CkFftCudaStft(self.handle, n, frames, ptr(signal), hop, frame_len, ptr(window), scale,
                                      ptr(out), s)

    def filter_inverse(self, n: int, frames: int, spectra, filt, scale: float, out, stream=None) -> int:
        """CkFftCudaFilterInverse: bins x filter x scale -> real inverse."""
        s = getattr(stream, "cuda_stream", stream)
        return self.lib.CkFftCudaFilterInverse(self.handle, n, frames, ptr(spectra), ptr(filt), scale, ptr(out), s)

    def run_jobs(self, jobs, stream=None) -> int:
        arr, n = job_array(jobs)
        s = getattr(stream, "cuda_stream", stream)
        return self.lib.CkFftCudaRunJobs(self.handle, C.cast(arr, C.c_void_p), n, s)

    def plan(self, jobs) -> "Plan":
        return Plan(self, jobs)

    def check(self, rc: int, what: str = "call"):
        if rc != 1:
            raise CkFftError(f"{what} failed: {last_error()}")


class Plan:
    """CkFftCudaPlan: a mixed run captured once, replayed with one graph launch."""

    def __init__(self, ctx: Context, jobs):
        self.lib = ctx.lib
        arr, n = job_array(jobs)
        self.handle = self.lib.CkFftCudaPlanJobs(ctx.handle, C.cast(arr, C.c_void_p), n)
        if not self.handle:
            raise CkFftError(f"CkFftCudaPlanJobs failed: {last_error()}")
        self.bytes = self.lib.CkFftCudaPlanBytes(self.handle)

    def exec(self, stream=None) -> int:
        s = getattr(stream, "cuda_stream", stream)
        return self.lib.CkFftCudaExecPlan(self.handle, s)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.CkFftCudaDestroyPlan(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """CkFftCudaServer: continuous-batching request server on one context."""

    def __init__(self, ctx: Context, scratch_budget_bytes: int = 2 << 30, max_inflight: int = 3,
                 direct_threshold_bytes: int = 8 << 20):
        self.lib = ctx.lib
        self.ctx = ctx
        self.handle = self.lib.CkFftCudaServerCreate(ctx.handle, scratch_budget_bytes, max_inflight,
                                                     direct_threshold_bytes)
        if not self.handle:
            raise CkFftError(f"CkFftCudaServerCreate failed: {last_error()}")

    def submit(self, kind, n, count, inp, out) -> int:
        job = Job(KIND.get(kind, kind), n, count, ptr(inp), ptr(out))
        return self.lib.CkFftCudaServerSubmit(self.handle, C.byref(job))

    def wait(self, ticket: int, timeout_s: float = -1.0):
        lat = C.c_double(0.0)
        ok = self.lib.CkFftCudaServerWait(self.handle, ticket, timeout_s, C.byref(lat))
        return ok, lat.value

    def replay(self, requests):
        """requests: list of (arrival_s, kind, n, count, input, output)."""
        arr, lat, st = _requests(requests)
        ok = self.lib.CkFftCudaServerReplay(self.handle, C.cast(arr, C.c_void_p), len(requests), lat, C.byref(st))
        return ok, list(lat), st.as_dict()

    def close(self):
        if getattr(self, "handle", None):
            self.lib.CkFftCudaServerDestroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _requests(requests):
    arr = (Request * max(1, len(requests)))()
    for i, (t, kind, n, count, inp, out) in enumerate(requests):
        arr[i] = Request(t, Job(KIND.get(kind, kind), n, count, ptr(inp), ptr(out)))
    lat = (C.c_double * max(1, len(requests)))()
    return arr, lat, ServeStats()


def replay_per_request(ctx: Context, requests):
    """The same trace through one blocking batch call per request."""
    arr, lat, st = _requests(requests)
    ok = ctx.lib.CkFftCudaReplayPerRequest(ctx.handle, C.cast(arr, C.c_void_p), len(requests), lat, C.byref(st))
    return ok, list(lat), st.as_dict()
