// ckfft_api.cpp -- the C ABI (include/ckfft_cuda.h) over the CUDA kernels.
//
// Mirrors the reference's API layer (src/ckfft/ckfft.cpp:14-119): the same
// argument checks in the same order with the same 0 / NULL results, and the
// context rules of src/ckfft/context.cpp:45-143 (size query through bufSize,
// caller-provided memory, Shutdown freeing only what Init allocated).
// Instead of FP32 tables in host memory the context owns FP64-derived
// twiddle tables in device memory, and every transform runs as CUDA kernels.
//
// Pointer handling: device and managed pointers on the context's device are
// used in place.  Page-locked host buffers of single-CTA sizes are read and
// written by the kernels themselves over the CPU-GPU link (one crossing per
// byte, no staging copy; CKFFT_CUDA_ZERO_COPY=0 turns this off).  Other host
// pointers (pageable, or multi-pass sizes) are moved through device-resident
// staging buffers, split into chunks that run on three streams so that
// host->device copies, kernels and device->host copies of consecutive chunks
// overlap.
#include "ckfft_cuda.h"

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "kernels.h"

namespace ckg {
void build_twiddles(int log2n, std::vector<float2>& tab);
}

namespace {

thread_local std::string t_error;

void set_error(const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_error = buf;
}

int fail(const char* what)
{
    set_error("%s", what);
    return 0;
}

int cuda_fail(const char* where, cudaError_t e)
{
    set_error("%s: %s", where, cudaGetErrorString(e));
    return 0;
}

// isPowerOfTwo of src/ckfft/math_util.h:12-15, applied to the int the caller
// passed.  Values <= 0 are rejected too (the reference lets INT_MIN through
// this test and then misbehaves).
bool valid_size(int n, int nmax)
{
    if (n <= 0) return false;
    const unsigned u = (unsigned)n;
    return (u & (u - 1)) == 0 && n <= nmax;
}

int log2i(long long n)
{
    int l = 0;
    while ((1ll << l) < n) ++l;
    return l;
}

constexpr int kSlots = 3;
constexpr size_t kChunkBytes = 64ull << 20;   // per staging buffer

struct Slot {
    cudaStream_t stream = nullptr;
    void* din = nullptr;
    size_t din_cap = 0;
    void* dout = nullptr;
    size_t dout_cap = 0;
};

struct Lane {
    Slot slot[kSlots];
    void* scratch = nullptr;
    size_t scratch_cap = 0;
    void* bounce = nullptr;     // page-locked, mapped: small calls on pageable host memory
    size_t bounce_cap = 0;
    bool busy = false;
};

struct LanePool {
    std::mutex mu;
    std::vector<Lane*> lanes;
};

constexpr uint32_t kMagic = 0x43554646u;   // "CUFF"

}  // namespace

struct _CkFftContext {
    uint32_t magic;
    int nmax;
    int log2max;
    int direction;
    int device;
    int own_buf;
    float2* dtw;            // twiddle levels, 2 * nmax entries
    LanePool* pool;
};

namespace {

// Keeps the context's device current for the duration of a call.
struct DeviceScope {
    int prev = -1;
    bool ok = true;
    explicit DeviceScope(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) { ok = false; return; }
        if (prev != dev && cudaSetDevice(dev) != cudaSuccess) ok = false;
    }
    ~DeviceScope()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

Lane* acquire_lane(CkFftContext* c)
{
    std::lock_guard<std::mutex> lock(c->pool->mu);
    for (Lane* l : c->pool->lanes) {
        if (!l->busy) { l->busy = true; return l; }
    }
    Lane* l = new (std::nothrow) Lane();
    if (!l) return nullptr;
    for (int i = 0; i < kSlots; ++i) {
        // blocking streams: a call made after work on the legacy default
        // stream (a fill, a copy) sees that work done, as a synchronous
        // library call should
        if (cudaStreamCreateWithFlags(&l->slot[i].stream, cudaStreamDefault) != cudaSuccess) {
            for (int j = 0; j < i; ++j) cudaStreamDestroy(l->slot[j].stream);
            delete l;
            return nullptr;
        }
    }
    l->busy = true;
    c->pool->lanes.push_back(l);
    return l;
}

void release_lane(CkFftContext* c, Lane* l)
{
    std::lock_guard<std::mutex> lock(c->pool->mu);
    l->busy = false;
}

void free_lane(Lane* l)
{
    for (int i = 0; i < kSlots; ++i) {
        if (l->slot[i].stream) cudaStreamSynchronize(l->slot[i].stream);
        cudaFree(l->slot[i].din);
        cudaFree(l->slot[i].dout);
        if (l->slot[i].stream) cudaStreamDestroy(l->slot[i].stream);
    }
    cudaFree(l->scratch);
    if (l->bounce) cudaFreeHost(l->bounce);
    delete l;
}

cudaError_t grow(void** p, size_t* cap, size_t need)
{
    if (*cap >= need) return cudaSuccess;
    cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = ckg::dev_malloc(p, need);
    if (e == cudaSuccess) *cap = need;
    return e;
}

enum class Mem { Host, Device };

// Classifies a pointer; returns false (with an error set) for device memory
// that belongs to another device.
bool classify(const void* p, int dev, Mem* where)
{
    cudaPointerAttributes a;
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *where = Mem::Host;
        return true;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) {
        if (a.type == cudaMemoryTypeDevice && a.device != dev) {
            set_error("pointer %p is device memory of device %d, context is on device %d", p, a.device, dev);
            return false;
        }
        *where = Mem::Device;
        return true;
    }
    *where = Mem::Host;
    return true;
}

bool zero_copy_enabled()
{
    static const bool on = [] {
        const char* v = std::getenv("CKFFT_CUDA_ZERO_COPY");
        return !(v && v[0] == '0');
    }();
    return on;
}

// cuPointerGetAttribute, taken from the driver through the runtime (the
// library links the runtime only).
using PtrAttrFn = CUresult (*)(void*, CUpointer_attribute, CUdeviceptr);

PtrAttrFn ptr_attr_fn()
{
    static const PtrAttrFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return (PtrAttrFn) nullptr;
        }
        return (PtrAttrFn)f;
    }();
    return fn;
}

// True when [p, p + bytes) lies inside ONE page-locked host allocation that
// the current device addresses at the same pointer, so that kernels may read
// or write the whole range in place.  Anything else (pageable memory, a range
// that runs past its allocation) answers false and is staged.
bool mapped_range(const void* p, size_t bytes)
{
    if (bytes == 0) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type != cudaMemoryTypeHost || a.devicePointer != p) return false;
    const PtrAttrFn fn = ptr_attr_fn();
    if (!fn) return false;
    unsigned long long first = 0, last = 0;
    if (fn(&first, CU_POINTER_ATTRIBUTE_BUFFER_ID, (CUdeviceptr)(uintptr_t)p) != CUDA_SUCCESS) return false;
    if (fn(&last, CU_POINTER_ATTRIBUTE_BUFFER_ID, (CUdeviceptr)((uintptr_t)p + bytes - 1)) != CUDA_SUCCESS)
        return false;
    return first != 0 && first == last;
}

bool mapped_host(const void* p, size_t bytes) { return zero_copy_enabled() && mapped_range(p, bytes); }

// One transform family request.
struct Work {
    ckg::Kind kind;
    int n;
    int log2n;
    long long count;
    size_t in_bytes;        // per transform
    size_t out_bytes;
    long long in_dist;      // elements of the input type between transforms
    long long out_dist;
};

Work make_work(ckg::Kind kind, int n, long long count)
{
    Work w;
    w.kind = kind;
    w.n = n;
    w.log2n = log2i(n);
    w.count = count;
    const size_t cplx = sizeof(CkFftComplex);
    switch (kind) {
    case ckg::C2C_FWD:
    case ckg::C2C_INV:
        w.in_bytes = w.out_bytes = cplx * (size_t)n;
        w.in_dist = w.out_dist = n;
        break;
    case ckg::R2C:
        w.in_bytes = sizeof(float) * (size_t)n;
        w.out_bytes = cplx * (size_t)(n / 2 + 1);
        w.in_dist = n;
        w.out_dist = n / 2 + 1;
        break;
    case ckg::C2R:
        w.in_bytes = cplx * (size_t)(n / 2 + 1);
        w.out_bytes = sizeof(float) * (size_t)n;
        w.in_dist = n / 2 + 1;
        w.out_dist = n;
        break;
    }
    return w;
}

bool is_real(ckg::Kind k) { return k == ckg::R2C || k == ckg::C2R; }

bool needs_large(const Work& w)
{
    return is_real(w.kind) ? w.log2n > ckg::kSmallMaxLog2Real : w.log2n > ckg::kSmallMaxLog2Complex;
}

// Enqueues the kernels for `cnt` transforms between device buffers.
// `scratch` must hold large_scratch_bytes() * cnt bytes when the size needs
// the multi-pass path (a smaller scratch runs the batch in groups).
cudaError_t enqueue(const CkFftContext* c, const Work& w, long long cnt, const void* din, void* dout,
                    void* scratch, size_t scratch_bytes, cudaStream_t s)
{
    if (cnt <= 0) return cudaSuccess;
    if (is_real(w.kind) && w.n <= 4)
        return ckg::launch_real_tiny(w.kind, w.n, din, dout, cnt, w.in_dist, w.out_dist, s);
    if (!is_real(w.kind) && ckg::cluster_supported(w.log2n) && ckg::cluster_enabled())
        return ckg::launch_cluster_c2c(w.kind == ckg::C2C_INV, w.log2n, din, dout, cnt, w.in_dist, w.out_dist,
                                       c->dtw, s);
    if (!needs_large(w))
        return ckg::launch_small(w.kind, w.log2n, din, dout, cnt, w.in_dist, w.out_dist, c->dtw, s);
    switch (w.kind) {
    case ckg::C2C_FWD:
    case ckg::C2C_INV:
        return ckg::launch_large_c2c(w.kind == ckg::C2C_INV, w.log2n, din, dout, cnt, w.in_dist, w.out_dist,
                                     c->dtw, scratch, scratch_bytes, s);
    case ckg::R2C:
        return ckg::launch_large_r2c(w.log2n, din, dout, cnt, w.in_dist, w.out_dist, c->dtw, scratch,
                                     scratch_bytes, s);
    case ckg::C2R:
        return ckg::launch_large_c2r(w.log2n, din, dout, cnt, w.in_dist, w.out_dist, c->dtw, scratch,
                                     scratch_bytes, s);
    }
    return cudaErrorInvalidValue;
}

// Scratch for the multi-pass path: enough for a group of transforms whose
// intermediate stays within a bounded size (at least one transform).
size_t scratch_need(const Work& w, long long cnt)
{
    if (!needs_large(w)) return 0;
    if (!is_real(w.kind) && ckg::cluster_supported(w.log2n) && ckg::cluster_enabled()) return 0;
    if (!is_real(w.kind) && ckg::mid_supported(w.log2n) && ckg::mid_enabled(w.log2n))
        return ckg::mid_scratch_bytes(w.log2n, cnt);
    const size_t one = ckg::large_scratch_bytes(w.kind, w.log2n);
    const size_t cap = 256ull << 20;
    long long g = (long long)(cap / one);
    if (g < 1) g = 1;
    if (g > cnt) g = cnt;
    return one * (size_t)g;
}

// Whether kernels reading and writing page-locked host memory in place beat
// the staged copy pipeline.  Measured on GB300 (real n = 4096, page-locked
// input and output): in place wins at every batch size when each output row
// is whole 128-byte lines (real inverse: 307 vs 247 GB/s at 65536 frames) and
// for every small call (one frame: 13.6 vs 21.4 us); with ragged output rows
// (real forward, n/2+1 complex) the kernels' partial-line writes to host
// memory cost more than the staged copies beyond about 128 MiB of output
// (258 vs 277 GB/s at 16384 frames, 266 vs 316 at 65536).
bool zero_copy_pays(const Work& w, bool host_out)
{
    if (!host_out || w.out_bytes % 128 == 0) return true;
    return (size_t)w.count * w.out_bytes <= (128ull << 20);
}

// Blocking run whose host-side buffers are mapped page-locked memory: one
// launch over the whole batch on a lane stream, kernels reading and writing
// the host memory in place (plain loads for a host input).
int run_direct(CkFftContext* c, const Work& w, const void* in, void* out, bool host_in, cudaStream_t user_stream)
{
    Lane* lane = acquire_lane(c);
    if (!lane) return fail("cannot create a staging lane (CUDA streams)");
    Slot& sl = lane->slot[0];
    cudaError_t e = cudaSuccess;
    const char* where = "kernel launch";
    cudaEvent_t dep = nullptr;
    if (user_stream) {
        if ((e = cudaEventCreateWithFlags(&dep, cudaEventDisableTiming)) != cudaSuccess) where = "cudaEventCreate";
        else if ((e = cudaEventRecord(dep, user_stream)) != cudaSuccess) where = "cudaEventRecord";
        else if ((e = cudaStreamWaitEvent(sl.stream, dep, 0)) != cudaSuccess) where = "cudaStreamWaitEvent";
    }
    if (e == cudaSuccess) {
        if (host_in) {
            ckg::PlainLoadsScope plain;
            e = enqueue(c, w, w.count, in, out, nullptr, 0, sl.stream);
        } else {
            e = enqueue(c, w, w.count, in, out, nullptr, 0, sl.stream);
        }
    }
    const cudaError_t se = cudaStreamSynchronize(sl.stream);
    if (e == cudaSuccess && se != cudaSuccess) { e = se; where = "cudaStreamSynchronize"; }
    if (dep) cudaEventDestroy(dep);
    release_lane(c, lane);
    if (e != cudaSuccess) return cuda_fail(where, e);
    if (ckg::take_device_error()) return fail("a kernel's bounded wait for its input copy timed out");
    return 1;
}

// Calls on pageable host memory up to this many bytes per side bounce
// through the lane's page-locked buffer: the CPU copies the input in, the
// kernel reads and writes the page-locked memory in place over the CPU-GPU
// link, the CPU copies the output out.  Two cudaMemcpy of pageable memory
// cost about 14 us on GB300 for 8 KiB each way (they are synchronous and
// staged by the driver); the two host copies take well under 1 us.
constexpr size_t kBounceMaxBytes = 1u << 20;

bool bounce_pays(const Work& w, Mem min, Mem mout)
{
    if (needs_large(w) || (min != Mem::Host && mout != Mem::Host)) return false;
    return (size_t)w.count * w.in_bytes <= kBounceMaxBytes && (size_t)w.count * w.out_bytes <= kBounceMaxBytes;
}

int run_bounce(CkFftContext* c, const Work& w, const void* in, void* out, Mem min, Mem mout)
{
    Lane* lane = acquire_lane(c);
    if (!lane) return fail("cannot create a staging lane (CUDA streams)");
    const size_t ib = (size_t)w.count * w.in_bytes, ob = (size_t)w.count * w.out_bytes;
    const size_t ibr = (ib + 255) / 256 * 256;
    const size_t need = (min == Mem::Host ? ibr : 0) + (mout == Mem::Host ? ob : 0);
    cudaError_t e = cudaSuccess;
    const char* where = "kernel launch";
    if (lane->bounce_cap < need) {
        if (lane->bounce) cudaFreeHost(lane->bounce);
        lane->bounce = nullptr;
        lane->bounce_cap = 0;
        const size_t cap = need < (64u << 10) ? (64u << 10) : need;
        e = cudaHostAlloc(&lane->bounce, cap, cudaHostAllocMapped | cudaHostAllocPortable);
        if (e == cudaSuccess) lane->bounce_cap = cap;
        else where = "cudaHostAlloc(bounce)";
    }
    if (e == cudaSuccess) {
        char* p = (char*)lane->bounce;
        const void* din = in;
        void* dout = out;
        if (min == Mem::Host) {
            std::memcpy(p, in, ib);
            din = p;
            p += ibr;
        }
        if (mout == Mem::Host) dout = p;
        Slot& sl = lane->slot[0];
        {
            ckg::PlainLoadsScope plain;    // page-locked host memory: plain loads, no bulk copies
            e = enqueue(c, w, w.count, din, dout, nullptr, 0, sl.stream);
        }
        const cudaError_t se = cudaStreamSynchronize(sl.stream);
        if (e == cudaSuccess && se != cudaSuccess) { e = se; where = "cudaStreamSynchronize"; }
        if (e == cudaSuccess && mout == Mem::Host) std::memcpy(out, dout, ob);
    }
    release_lane(c, lane);
    if (e != cudaSuccess) return cuda_fail(where, e);
    if (ckg::take_device_error()) return fail("a kernel's bounded wait for its input copy timed out");
    return 1;
}

// Runs a request.  stream != NULL with device pointers: asynchronous on that
// stream.  Mapped page-locked host buffers of single-CTA sizes: one blocking
// launch in place.  Otherwise blocking, staged through a lane of the
// context's pool.
int run(CkFftContext* c, const Work& w, const void* in, void* out, cudaStream_t user_stream,
        void* user_scratch = nullptr, size_t user_scratch_bytes = 0)
{
    DeviceScope scope(c->device);
    if (!scope.ok) return fail("cannot select the context's CUDA device");
    if (w.count == 0) return 1;
    Mem min, mout;
    if (!classify(in, c->device, &min) || !classify(out, c->device, &mout)) return 0;

    if (user_stream && min == Mem::Device && mout == Mem::Device) {
        // asynchronous path: scratch from the library's stream-ordered pool
        const size_t need = scratch_need(w, w.count);
        void* scratch = nullptr;
        if (need) {
            cudaError_t e = ckg::pool_alloc_async(&scratch, need, user_stream);
            if (e != cudaSuccess) return cuda_fail("stream-ordered scratch allocation", e);
        }
        cudaError_t e = enqueue(c, w, w.count, in, out, scratch, need, user_stream);
        if (scratch) cudaFreeAsync(scratch, user_stream);
        if (e != cudaSuccess) return cuda_fail("kernel launch", e);
        return 1;
    }
    if (!needs_large(w) && (min == Mem::Host || mout == Mem::Host) && zero_copy_pays(w, mout == Mem::Host) &&
        (min == Mem::Device || mapped_host(in, (size_t)w.count * w.in_bytes)) &&
        (mout == Mem::Device || mapped_host(out, (size_t)w.count * w.out_bytes)))
        return run_direct(c, w, in, out, min == Mem::Host, user_stream);
    if (!user_stream && bounce_pays(w, min, mout)) return run_bounce(c, w, in, out, min, mout);

    Lane* lane = acquire_lane(c);
    if (!lane) return fail("cannot create a staging lane (CUDA streams)");
    int ok = 1;
    cudaError_t e = cudaSuccess;
    const char* where = "";
    unsigned used = 0;                    // slot streams this call enqueued work on
    // a user stream orders the blocking call after the stream's earlier work
    cudaEvent_t dep = nullptr;
    if (user_stream) {
        if ((e = cudaEventCreateWithFlags(&dep, cudaEventDisableTiming)) != cudaSuccess) { where = "cudaEventCreate"; goto done; }
        if ((e = cudaEventRecord(dep, user_stream)) != cudaSuccess) { where = "cudaEventRecord"; goto done; }
        for (int i = 0; i < kSlots; ++i) cudaStreamWaitEvent(lane->slot[i].stream, dep, 0);
    }
    {
        const size_t per = w.in_bytes > w.out_bytes ? w.in_bytes : w.out_bytes;
        long long chunk = w.count;
        const bool staged = (min == Mem::Host || mout == Mem::Host);
        if (staged) {
            chunk = (long long)(kChunkBytes / per);
            if (chunk < 1) chunk = 1;
            if (chunk > w.count) chunk = w.count;
        }
        // scratch is shared by the slots; with several chunks in flight the
        // multi-pass path uses one slot at a time (chunks run in order below)
        void* scratch = user_scratch;
        size_t scratch_bytes = user_scratch_bytes;
        const size_t need = scratch_need(w, chunk);
        if (need && scratch_bytes < ckg::large_scratch_bytes(w.kind, w.log2n)) {
            if ((e = grow(&lane->scratch, &lane->scratch_cap, need)) != cudaSuccess) { where = "cudaMalloc(scratch)"; goto done; }
            scratch = lane->scratch;
            scratch_bytes = lane->scratch_cap;
        }
        const bool serial = need != 0;      // shared scratch: keep chunks on one stream
        for (long long off = 0, i = 0; off < w.count; off += chunk, ++i) {
            const long long cnt = (w.count - off < chunk) ? w.count - off : chunk;
            const int si = serial ? 0 : (int)(i % kSlots);
            used |= 1 << si;
            Slot& sl = lane->slot[si];
            const void* din = (const char*)in + (size_t)off * w.in_bytes;
            void* dout = (char*)out + (size_t)off * w.out_bytes;
            if (min == Mem::Host) {
                if (sl.din_cap < (size_t)cnt * w.in_bytes) {
                    cudaStreamSynchronize(sl.stream);
                    if ((e = grow(&sl.din, &sl.din_cap, (size_t)chunk * w.in_bytes)) != cudaSuccess) { where = "cudaMalloc(staging)"; goto done; }
                }
                if ((e = cudaMemcpyAsync(sl.din, din, (size_t)cnt * w.in_bytes, cudaMemcpyHostToDevice, sl.stream)) != cudaSuccess) { where = "cudaMemcpyAsync(H2D)"; goto done; }
                din = sl.din;
            }
            void* host_out = nullptr;
            if (mout == Mem::Host) {
                if (sl.dout_cap < (size_t)cnt * w.out_bytes) {
                    cudaStreamSynchronize(sl.stream);
                    if ((e = grow(&sl.dout, &sl.dout_cap, (size_t)chunk * w.out_bytes)) != cudaSuccess) { where = "cudaMalloc(staging)"; goto done; }
                }
                host_out = dout;
                dout = sl.dout;
            }
            if ((e = enqueue(c, w, cnt, din, dout, scratch, scratch_bytes, sl.stream)) != cudaSuccess) { where = "kernel launch"; goto done; }
            if (host_out) {
                if ((e = cudaMemcpyAsync(host_out, dout, (size_t)cnt * w.out_bytes, cudaMemcpyDeviceToHost, sl.stream)) != cudaSuccess) { where = "cudaMemcpyAsync(D2H)"; goto done; }
            }
        }
    }
done:
    for (int i = 0; i < kSlots; ++i) {
        if (!(used >> i & 1)) continue;              // streams this call left idle
        cudaError_t se = cudaStreamSynchronize(lane->slot[i].stream);
        if (e == cudaSuccess && se != cudaSuccess) { e = se; where = "cudaStreamSynchronize"; }
    }
    if (dep) cudaEventDestroy(dep);
    release_lane(c, lane);
    if (e != cudaSuccess) ok = cuda_fail(where, e);
    else if (ckg::take_device_error()) ok = fail("a kernel's bounded wait for its input copy timed out");
    return ok;
}

bool ctx_ok(const CkFftContext* c) { return c && c->magic == kMagic; }
bool has_fwd(const CkFftContext* c) { return (c->direction & kCkFftDirection_Forward) != 0; }
bool has_inv(const CkFftContext* c) { return (c->direction & kCkFftDirection_Inverse) != 0; }

// Checks of src/ckfft/ckfft.cpp:38-49 / 80-91 / 99-110 (tmpBuf first for
// the real inverse, :57-60), then the batch count.
int check_call(const CkFftContext* c, bool inverse, int n, const void* in, const void* out, long long count)
{
    if (!ctx_ok(c) || !(inverse ? has_inv(c) : has_fwd(c)))
        return fail(ctx_ok(c) ? "context was created without this direction" : "NULL or invalid context");
    if (!valid_size(n, c->nmax)) return fail("n must be a power of two no larger than the context's nMax");
    if (!in || !out || in == out) return fail("input and output must be distinct non-NULL buffers");
    if (count < 0) return fail("count must be >= 0");
    return 1;
}

// ------------------------------------------------------------ strided batches

// Distance-1 layouts (interleaved channels, matrix columns) of the sizes the
// distance-1 kernels of fft_inter.cu do not cover, and complex transforms
// from 2^12 whose input side alone is distance-1, run as chunks of F
// transforms: each distance-1 side is transposed between the layout and
// contiguous rows of a scratch block sized to stay in L2 (96 MiB), and the
// contiguous batched kernels transform the rows.  The transposes move runs
// of 32 transforms (128 / 256 contiguous bytes of every layout row), and the
// transforms are the contiguous path's own, bit for bit.  A side that is not
// distance-1 must be contiguous rows (stride 1) the batched kernels read
// directly.  Measured on GB300 (GB/s): complex n = 2^16 x 1024 on both
// sides 1555 against 542 through the element-wise gather / scatter; n = 4096
// x 16384 with the input side alone distance-1 3092 against 2693 for the
// distance-1 kernel; where that kernel covers both sides or a real side it
// stays ahead (n = 4096 both sides 2253 against 2071, reals in 2723 against
// 2566, reals out 3128 against 2280, matrix columns 1024 x 65536 3222
// against 2218).

constexpr size_t kTransposeChunkBytes = 96ull << 20;

cudaError_t enqueue_transposed(CkFftContext* c, const Work& w, const void* in, long long is, void* out,
                               long long os, bool cin, bool cout, cudaStream_t s)
{
    const int ein = w.kind == ckg::R2C ? 4 : 8, eout = w.kind == ckg::C2R ? 4 : 8;
    const long long ni = (long long)(w.in_bytes / ein), no = (long long)(w.out_bytes / eout);
    const size_t per = (cin ? w.in_bytes : 0) + (cout ? w.out_bytes : 0);
    long long F = (long long)((kTransposeChunkBytes) / per);
    if (F >= 32) F = F / 32 * 32;                     // whole transpose tiles
    if (F < 1) F = 1;
    if (F > w.count) F = w.count;
    Work wc = make_work(w.kind, w.n, F);
    wc.in_dist = cin ? ni : w.in_dist;
    wc.out_dist = cout ? no : w.out_dist;
    const size_t bin = cin ? (w.in_bytes * (size_t)F + 255) & ~(size_t)255 : 0;
    const size_t bout = cout ? (w.out_bytes * (size_t)F + 255) & ~(size_t)255 : 0;
    const size_t large = scratch_need(wc, F);
    void* block = nullptr;
    cudaError_t e = ckg::pool_alloc_async(&block, bin + bout + large, s);
    if (e != cudaSuccess) return e;
    char* tin = (char*)block;
    char* tout = tin + bin;
    void* tl = large ? (void*)(tout + bout) : nullptr;
    for (long long off = 0; off < w.count && e == cudaSuccess; off += F) {
        const long long cnt = w.count - off < F ? w.count - off : F;
        const char* src = (const char*)in + (size_t)(off * w.in_dist) * ein;
        char* dst = (char*)out + (size_t)(off * w.out_dist) * eout;
        if (cin) e = ckg::launch_transpose(src, is, tin, ni, ni, cnt, ein, true, false, s);
        if (e == cudaSuccess) e = enqueue(c, wc, cnt, cin ? tin : src, cout ? tout : dst, tl, large, s);
        if (e == cudaSuccess && cout) e = ckg::launch_transpose(tout, no, dst, os, cnt, no, eout, false, true, s);
    }
    cudaFreeAsync(block, s);
    return e;
}

// Enqueues an advanced-layout batch on `s` (buffers the device can address).
cudaError_t enqueue_strided(CkFftContext* c, const Work& w, const void* in, long long is, void* out, long long os,
                            cudaStream_t s)
{
    const bool rin = w.kind == ckg::R2C, rout = w.kind == ckg::C2R;
    // contiguous rows at any distance: the batched kernels read them directly
    // (real rows as packed pairs: 8-byte aligned, even distance)
    const bool in_rows = is == 1 && (!rin || (w.in_dist % 2 == 0 && ((uintptr_t)in & 7) == 0));
    const bool out_rows = os == 1 && (!rout || (w.out_dist % 2 == 0 && ((uintptr_t)out & 7) == 0));
    const bool rows = in_rows && out_rows;
    cudaError_t e;
    if (rows) {
        const size_t need = scratch_need(w, w.count);
        void* scratch = nullptr;
        if (need && (e = ckg::pool_alloc_async(&scratch, need, s)) != cudaSuccess) return e;
        e = enqueue(c, w, w.count, in, out, scratch, need, s);
        if (scratch) cudaFreeAsync(scratch, s);
        return e;
    }
    // consecutive transforms adjacent (interleaved channels, matrix columns)
    const bool cin = w.in_dist == 1 && is > 1, cout = w.out_dist == 1 && os > 1;
    const bool complex_in_only = !is_real(w.kind) && cin && !cout && w.log2n >= 12;
    if (!complex_in_only && ckg::inter_applies(w.kind, w.log2n, cin, cout))
        return ckg::launch_inter(w.kind, w.log2n, in, out, w.count, ckg::Layout{is, w.in_dist, os, w.out_dist}, cin,
                                 cout, c->dtw, s);
    if ((cin || cout) && (cin || in_rows) && (cout || out_rows))
        return enqueue_transposed(c, w, in, is, out, os, cin, cout, s);
    if (ckg::strided_supported(w.kind, w.log2n))
        return ckg::launch_strided(w.kind, w.log2n, in, out, w.count, ckg::Layout{is, w.in_dist, os, w.out_dist},
                                   c->dtw, s);
    // gather -> contiguous transform -> scatter, in groups of bounded scratch
    const int ein = rin ? 4 : 8, eout = rout ? 4 : 8;
    const long long ni = (long long)(w.in_bytes / ein), no = (long long)(w.out_bytes / eout);
    const size_t per = w.in_bytes + w.out_bytes;
    long long g = (long long)((256ull << 20) / per);
    if (g < 1) g = 1;
    if (g > w.count) g = w.count;
    const size_t rows_in = (w.in_bytes * (size_t)g + 255) & ~(size_t)255;
    const size_t rows_out = (w.out_bytes * (size_t)g + 255) & ~(size_t)255;
    const size_t large = scratch_need(w, g);
    void* block = nullptr;
    if ((e = ckg::pool_alloc_async(&block, rows_in + rows_out + large, s)) != cudaSuccess) return e;
    char* tin = (char*)block;
    char* tout = tin + rows_in;
    void* tl = large ? (void*)(tout + rows_out) : nullptr;
    for (long long off = 0; off < w.count && e == cudaSuccess; off += g) {
        const long long cnt = w.count - off < g ? w.count - off : g;
        const Work wc = make_work(w.kind, w.n, cnt);
        e = ckg::launch_gather((const char*)in + (size_t)(off * w.in_dist) * ein, is, w.in_dist, tin, cnt, ni, ein, s);
        if (e == cudaSuccess) e = enqueue(c, wc, cnt, tin, tout, tl, large, s);
        if (e == cudaSuccess)
            e = ckg::launch_scatter(tout, (char*)out + (size_t)(off * w.out_dist) * eout, os, w.out_dist, cnt, no,
                                    eout, s);
    }
    cudaFreeAsync(block, s);
    return e;
}

// Validation of an advanced layout (after check_call): element counts,
// non-overlapping output transforms, disjoint input and output ranges.
// On success sets the byte spans of both sides.
int check_layout(const Work& w, const void* in, long long is, long long id, const void* out, long long os,
                 long long od, size_t* in_span, size_t* out_span)
{
    if (is < 1 || os < 1) return fail("strides must be >= 1");
    if (id < 0 || od < 0) return fail("distances must be >= 0");
    const int ein = w.kind == ckg::R2C ? 4 : 8, eout = w.kind == ckg::C2R ? 4 : 8;
    const __int128 ni = (__int128)(w.in_bytes / ein), no = (__int128)(w.out_bytes / eout);
    const __int128 cnt = w.count;
    if (cnt > 1) {
        const bool side = (__int128)od >= (no - 1) * os + 1;
        const bool inter = od >= 1 && (__int128)os >= (cnt - 1) * od + 1;
        if (!side && !inter) return fail("output transforms overlap (stride / distance)");
    }
    const __int128 si = ((cnt - 1) * id + (ni - 1) * is + 1) * ein;
    const __int128 so = ((cnt - 1) * od + (no - 1) * os + 1) * eout;
    const __int128 lim = (__int128)1 << 62;
    if (si > lim || so > lim) return fail("layout spans more than 2^62 bytes");
    const uintptr_t a0 = (uintptr_t)in, a1 = a0 + (uintptr_t)si, b0 = (uintptr_t)out, b1 = b0 + (uintptr_t)so;
    if (a1 < a0 || b1 < b0) return fail("layout wraps the address space");
    if (a0 < b1 && b0 < a1) return fail("input and output ranges overlap");
    *in_span = (size_t)si;
    *out_span = (size_t)so;
    return 1;
}

// One buffer of a layout call: `span` bytes at `ptr`, read by the kernels
// or (output) written by them.  `dev` is the address the kernels use.
struct Span {
    const void* ptr;
    size_t span;
    bool output;
    void* dev;
    bool staged;
};

constexpr size_t kStageLimit = 4ull << 30;

// Runs body(stream) with every span addressable by the device.  Device and
// managed memory and page-locked host ranges are used in place; pageable
// host spans are staged through stream-ordered device memory (copied in
// before the kernels -- outputs too, so that the gaps of a strided output
// keep their contents -- and outputs copied back after; at most 4 GiB per
// call).  stream != NULL with device spans only: asynchronous on that
// stream.  Otherwise blocking on a lane stream ordered after the stream's
// earlier work.
template <class Body>
int run_spans(CkFftContext* c, Span* sp, int nsp, void* stream, Body body)
{
    DeviceScope scope(c->device);
    if (!scope.ok) return fail("cannot select the context's CUDA device");
    bool all_dev = true, host_in = false;
    size_t staged = 0;
    for (int i = 0; i < nsp; ++i) {
        sp[i].dev = (void*)sp[i].ptr;
        sp[i].staged = false;
        if (!sp[i].ptr || sp[i].span == 0) continue;
        Mem m;
        if (!classify(sp[i].ptr, c->device, &m)) return 0;
        if (m == Mem::Device) continue;
        all_dev = false;
        if (mapped_range(sp[i].ptr, sp[i].span)) {
            if (!sp[i].output) host_in = true;
            continue;
        }
        sp[i].staged = true;
        staged += (sp[i].span + 255) & ~(size_t)255;
    }
    if (staged > kStageLimit)
        return fail("more than 4 GiB of pageable host memory in one call: use device or page-locked buffers");
    const cudaStream_t us = (cudaStream_t)stream;
    if (us && all_dev) {
        const cudaError_t e = body(us);
        return e == cudaSuccess ? 1 : cuda_fail("kernel launch", e);
    }
    Lane* lane = acquire_lane(c);
    if (!lane) return fail("cannot create a staging lane (CUDA streams)");
    const cudaStream_t s = lane->slot[0].stream;
    cudaError_t e = cudaSuccess;
    const char* where = "kernel launch";
    if (!us && staged && staged <= kBounceMaxBytes) {
        // small pageable spans: through the lane's page-locked buffer (run_bounce)
        if (lane->bounce_cap < staged) {
            if (lane->bounce) cudaFreeHost(lane->bounce);
            lane->bounce = nullptr;
            lane->bounce_cap = 0;
            const size_t cap = staged < (64u << 10) ? (64u << 10) : staged;
            if ((e = cudaHostAlloc(&lane->bounce, cap, cudaHostAllocMapped | cudaHostAllocPortable)) == cudaSuccess)
                lane->bounce_cap = cap;
            else
                where = "cudaHostAlloc(bounce)";
        }
        if (e == cudaSuccess) {
            char* at = (char*)lane->bounce;
            for (int i = 0; i < nsp; ++i) {
                if (!sp[i].staged) continue;
                sp[i].dev = at;
                at += (sp[i].span + 255) & ~(size_t)255;
                // outputs too: the gaps of a strided output keep their contents
                std::memcpy(sp[i].dev, sp[i].ptr, sp[i].span);
            }
            {
                ckg::PlainLoadsScope plain;
                e = body(s);
            }
            const cudaError_t se = cudaStreamSynchronize(s);
            if (e == cudaSuccess && se != cudaSuccess) { e = se; where = "cudaStreamSynchronize"; }
            for (int i = 0; i < nsp && e == cudaSuccess; ++i)
                if (sp[i].staged && sp[i].output) std::memcpy((void*)sp[i].ptr, sp[i].dev, sp[i].span);
        }
        release_lane(c, lane);
        if (e != cudaSuccess) return cuda_fail(where, e);
        if (ckg::take_device_error()) return fail("a kernel's bounded wait for its input copy timed out");
        return 1;
    }
    cudaEvent_t dep = nullptr;
    void* block = nullptr;
    if (us) {
        if ((e = cudaEventCreateWithFlags(&dep, cudaEventDisableTiming)) != cudaSuccess) where = "cudaEventCreate";
        else if ((e = cudaEventRecord(dep, us)) != cudaSuccess) where = "cudaEventRecord";
        else if ((e = cudaStreamWaitEvent(s, dep, 0)) != cudaSuccess) where = "cudaStreamWaitEvent";
    }
    if (e == cudaSuccess && staged) {
        if ((e = ckg::pool_alloc_async(&block, staged, s)) != cudaSuccess) where = "stream-ordered staging allocation";
        char* at = (char*)block;
        for (int i = 0; i < nsp && e == cudaSuccess; ++i) {
            if (!sp[i].staged) continue;
            sp[i].dev = at;
            at += (sp[i].span + 255) & ~(size_t)255;
            if ((e = cudaMemcpyAsync(sp[i].dev, sp[i].ptr, sp[i].span, cudaMemcpyHostToDevice, s)) != cudaSuccess)
                where = "cudaMemcpyAsync(H2D)";
        }
    }
    if (e == cudaSuccess) {
        if (host_in) {
            ckg::PlainLoadsScope plain;
            e = body(s);
        } else {
            e = body(s);
        }
    }
    for (int i = 0; i < nsp && e == cudaSuccess; ++i) {
        if (!sp[i].staged || !sp[i].output) continue;
        if ((e = cudaMemcpyAsync((void*)sp[i].ptr, sp[i].dev, sp[i].span, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            where = "cudaMemcpyAsync(D2H)";
    }
    if (block) cudaFreeAsync(block, s);
    const cudaError_t se = cudaStreamSynchronize(s);
    if (e == cudaSuccess && se != cudaSuccess) { e = se; where = "cudaStreamSynchronize"; }
    if (dep) cudaEventDestroy(dep);
    release_lane(c, lane);
    if (e != cudaSuccess) return cuda_fail(where, e);
    if (ckg::take_device_error()) return fail("a kernel's bounded wait for its input copy timed out");
    return 1;
}

// Byte ranges [a, a + na) and [b, b + nb) intersect (empty ranges never do).
bool ranges_meet(const void* a, size_t na, const void* b, size_t nb)
{
    if (!a || !b || na == 0 || nb == 0) return false;
    const uintptr_t a0 = (uintptr_t)a, b0 = (uintptr_t)b;
    return a0 < b0 + nb && b0 < a0 + na;
}

int strided_call(CkFftContext* c, ckg::Kind kind, int n, long long count, const void* in, long long is,
                 long long id, void* out, long long os, long long od, void* stream)
{
    const bool inverse = kind == ckg::C2C_INV || kind == ckg::C2R;
    if (!check_call(c, inverse, n, in, out, count)) return 0;
    if (count > 0x7fffffffLL) return fail("count must be below 2^31");
    Work w = make_work(kind, n, count);
    if (count == 0) return 1;
    size_t in_span = 0, out_span = 0;
    if (!check_layout(w, in, is, id, out, os, od, &in_span, &out_span)) return 0;
    w.in_dist = id;
    w.out_dist = od;
    Span sp[2] = {{in, in_span, false, nullptr, false}, {out, out_span, true, nullptr, false}};
    return run_spans(c, sp, 2, stream, [&](cudaStream_t s) {
        return enqueue_strided(c, w, sp[0].dev, is, sp[1].dev, os, s);
    });
}

// ------------------------------------------------------------ fused steps

cudaError_t enqueue_stft(CkFftContext* c, int n, long long frames, const float* signal, long long hop,
                         const float* window, long long frame_len, float scale, CkFftComplex* out, cudaStream_t s)
{
    const int log2n = log2i(n);
    if (ckg::fused_supported(log2n))
        return ckg::launch_stft(log2n, signal, hop, window, frame_len, scale, out, frames, c->dtw, s);
    // windowed rows, contiguous real forward, then the scale
    const long long bins = n / 2 + 1;
    const Work all = make_work(ckg::R2C, n, frames);
    long long g = (long long)((256ull << 20) / ((size_t)n * 4));
    if (g < 1) g = 1;
    if (g > frames) g = frames;
    const size_t rows = ((size_t)g * n * 4 + 255) & ~(size_t)255;
    const size_t large = scratch_need(all, g);
    void* block = nullptr;
    cudaError_t e = ckg::pool_alloc_async(&block, rows + large, s);
    if (e != cudaSuccess) return e;
    float* r = (float*)block;
    void* tl = large ? (void*)((char*)block + rows) : nullptr;
    for (long long off = 0; off < frames && e == cudaSuccess; off += g) {
        const long long cnt = frames - off < g ? frames - off : g;
        e = ckg::launch_window_rows(signal + off * hop, hop, window, frame_len, r, cnt, n, s);
        if (e == cudaSuccess) e = enqueue(c, make_work(ckg::R2C, n, cnt), cnt, r, out + off * bins, tl, large, s);
        if (e == cudaSuccess && scale != 1.0f) e = ckg::launch_scale_rows(out + off * bins, cnt * bins, scale, s);
    }
    cudaFreeAsync(block, s);
    return e;
}

cudaError_t enqueue_filter(CkFftContext* c, int n, long long frames, const CkFftComplex* spectra,
                           const CkFftComplex* filter, float scale, float* out, cudaStream_t s)
{
    const int log2n = log2i(n);
    if (ckg::fused_supported(log2n))
        return ckg::launch_filter_inverse(log2n, spectra, filter, scale, out, frames, c->dtw, s);
    // filtered rows, then the contiguous real inverse
    const long long bins = n / 2 + 1;
    const Work all = make_work(ckg::C2R, n, frames);
    long long g = (long long)((256ull << 20) / ((size_t)bins * 8));
    if (g < 1) g = 1;
    if (g > frames) g = frames;
    const size_t rows = ((size_t)g * bins * 8 + 255) & ~(size_t)255;
    const size_t large = scratch_need(all, g);
    void* block = nullptr;
    cudaError_t e = ckg::pool_alloc_async(&block, rows + large, s);
    if (e != cudaSuccess) return e;
    void* tl = large ? (void*)((char*)block + rows) : nullptr;
    for (long long off = 0; off < frames && e == cudaSuccess; off += g) {
        const long long cnt = frames - off < g ? frames - off : g;
        e = ckg::launch_filter_rows(spectra + off * bins, filter, scale, block, cnt, bins, s);
        if (e == cudaSuccess) e = enqueue(c, make_work(ckg::C2R, n, cnt), cnt, block, out + off * n, tl, large, s);
    }
    cudaFreeAsync(block, s);
    return e;
}

int complex_call(CkFftContext* c, bool inverse, int n, long long count, const CkFftComplex* in,
                 CkFftComplex* out, void* stream)
{
    if (!check_call(c, inverse, n, in, out, count)) return 0;
    return run(c, make_work(inverse ? ckg::C2C_INV : ckg::C2C_FWD, n, count), in, out, (cudaStream_t)stream);
}

}  // namespace

namespace ckg {


bool context_view(const CkFftContext* c, ContextView* out)
{
    if (!ctx_ok(c)) return false;
    out->nmax = c->nmax;
    out->direction = c->direction;
    out->device = c->device;
    out->tw = c->dtw;
    return true;
}

void set_last_error(const char* msg) { set_error("%s", msg); }

}  // namespace ckg

extern "C" {

CkFftContext* CkFftInit(int nMax, CkFftDirection direction, void* buf, size_t* bufSize)
{
    // src/ckfft/ckfft.cpp:16-31
    if (nMax <= 0) { set_error("nMax must be > 0"); return nullptr; }
    if (((unsigned)nMax & ((unsigned)nMax - 1)) != 0) { set_error("nMax must be a power of two"); return nullptr; }
    if (direction != kCkFftDirection_Forward && direction != kCkFftDirection_Inverse &&
        direction != kCkFftDirection_Both) {
        set_error("invalid direction");
        return nullptr;
    }
    if (buf && !bufSize) { set_error("buf given without bufSize"); return nullptr; }

    // src/ckfft/context.cpp:47-72: required size, size query
    size_t req = sizeof(_CkFftContext);
    if (req % sizeof(CkFftComplex)) req += sizeof(CkFftComplex) - req % sizeof(CkFftComplex);
    if (bufSize && (!buf || *bufSize < req)) {
        *bufSize = req;
        set_error("buffer size query: %zu bytes required", req);
        return nullptr;
    }
    void* mem = buf ? buf : std::malloc(req);
    if (!mem) { set_error("out of host memory"); return nullptr; }
    CkFftContext* c = new (mem) _CkFftContext();
    c->magic = 0;
    c->nmax = nMax;
    c->log2max = log2i(nMax);
    c->direction = direction;
    c->own_buf = buf == nullptr;
    c->dtw = nullptr;
    c->pool = nullptr;

    cudaError_t e = cudaGetDevice(&c->device);
    std::vector<float2> tab;
    if (e != cudaSuccess) { cuda_fail("no CUDA device", e); goto fail_out; }
    if ((e = ckg::prepare_device()) != cudaSuccess) { cuda_fail("kernel set-up", e); goto fail_out; }
    ckg::build_twiddles(c->log2max, tab);
    if ((e = ckg::dev_malloc((void**)&c->dtw, sizeof(float2) * tab.size())) != cudaSuccess) { cuda_fail("cudaMalloc(twiddles)", e); goto fail_out; }
    if ((e = cudaMemcpy(c->dtw, tab.data(), sizeof(float2) * tab.size(), cudaMemcpyHostToDevice)) != cudaSuccess) { cuda_fail("cudaMemcpy(twiddles)", e); goto fail_out; }
    c->pool = new (std::nothrow) LanePool();
    if (!c->pool) { set_error("out of host memory"); goto fail_out; }
    c->magic = kMagic;
    return c;

fail_out:
    if (c->dtw) cudaFree(c->dtw);
    if (c->own_buf) std::free(mem);
    return nullptr;
}

void CkFftShutdown(CkFftContext* c)
{
    if (!ctx_ok(c)) return;
    {
        DeviceScope scope(c->device);
        for (Lane* l : c->pool->lanes) free_lane(l);
        delete c->pool;
        cudaFree(c->dtw);
    }
    c->magic = 0;
    if (c->own_buf) std::free(c);
}

int CkFftComplexForward(CkFftContext* c, int n, const CkFftComplex* in, CkFftComplex* out)
{
    return complex_call(c, false, n, 1, in, out, nullptr);
}

int CkFftComplexInverse(CkFftContext* c, int n, const CkFftComplex* in, CkFftComplex* out)
{
    return complex_call(c, true, n, 1, in, out, nullptr);
}

int CkFftRealForward(CkFftContext* c, int n, const float* in, CkFftComplex* out)
{
    if (!check_call(c, false, n, in, out, 1)) return 0;
    return run(c, make_work(ckg::R2C, n, 1), in, out, nullptr);
}

int CkFftRealInverse(CkFftContext* c, int n, const CkFftComplex* in, float* out, CkFftComplex* tmpBuf)
{
    if (!tmpBuf) return fail("tmpBuf must not be NULL");
    if (!check_call(c, true, n, in, out, 1)) return 0;
    // tmpBuf (n/2+1 complex) is exactly the multi-pass path's intermediate;
    // use it when it is device memory on the context's device
    Work w = make_work(ckg::C2R, n, 1);
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    if (needs_large(w)) {
        DeviceScope scope(c->device);
        Mem where;
        // (256-byte alignment: the row pass drops the dead intermediate's
        // 128-byte L2 lines after reading them)
        if (scope.ok && ((uintptr_t)tmpBuf & 255) == 0 && classify(tmpBuf, c->device, &where) &&
            where == Mem::Device) {
            scratch = tmpBuf;
            scratch_bytes = sizeof(CkFftComplex) * (size_t)(n / 2 + 1);
        }
        t_error.clear();
    }
    return run(c, w, in, out, nullptr, scratch, scratch_bytes);
}

const char* CkFftCudaGetLastError(void) { return t_error.c_str(); }

int CkFftCudaComplexForwardBatch(CkFftContext* c, int n, int count, const CkFftComplex* in,
                                 CkFftComplex* out, void* stream)
{
    return complex_call(c, false, n, count, in, out, stream);
}

int CkFftCudaComplexInverseBatch(CkFftContext* c, int n, int count, const CkFftComplex* in,
                                 CkFftComplex* out, void* stream)
{
    return complex_call(c, true, n, count, in, out, stream);
}

int CkFftCudaRealForwardBatch(CkFftContext* c, int n, int count, const float* in, CkFftComplex* out,
                              void* stream)
{
    if (!check_call(c, false, n, in, out, count)) return 0;
    return run(c, make_work(ckg::R2C, n, count), in, out, (cudaStream_t)stream);
}

int CkFftCudaRealInverseBatch(CkFftContext* c, int n, int count, const CkFftComplex* in, float* out,
                              void* stream)
{
    if (!check_call(c, true, n, in, out, count)) return 0;
    return run(c, make_work(ckg::C2R, n, count), in, out, (cudaStream_t)stream);
}

int CkFftCudaComplexForwardStrided(CkFftContext* c, int n, long long count, const CkFftComplex* in,
                                   long long in_stride, long long in_dist, CkFftComplex* out, long long out_stride,
                                   long long out_dist, void* stream)
{
    return strided_call(c, ckg::C2C_FWD, n, count, in, in_stride, in_dist, out, out_stride, out_dist, stream);
}

int CkFftCudaComplexInverseStrided(CkFftContext* c, int n, long long count, const CkFftComplex* in,
                                   long long in_stride, long long in_dist, CkFftComplex* out, long long out_stride,
                                   long long out_dist, void* stream)
{
    return strided_call(c, ckg::C2C_INV, n, count, in, in_stride, in_dist, out, out_stride, out_dist, stream);
}

int CkFftCudaRealForwardStrided(CkFftContext* c, int n, long long count, const float* in, long long in_stride,
                                long long in_dist, CkFftComplex* out, long long out_stride, long long out_dist,
                                void* stream)
{
    return strided_call(c, ckg::R2C, n, count, in, in_stride, in_dist, out, out_stride, out_dist, stream);
}

int CkFftCudaRealInverseStrided(CkFftContext* c, int n, long long count, const CkFftComplex* in,
                                long long in_stride, long long in_dist, float* out, long long out_stride,
                                long long out_dist, void* stream)
{
    return strided_call(c, ckg::C2R, n, count, in, in_stride, in_dist, out, out_stride, out_dist, stream);
}

int CkFftCudaStft(CkFftContext* c, int n, long long frames, const float* signal, long long hop,
                  long long frame_len, const float* window, float scale, CkFftComplex* out, void* stream)
{
    if (!ctx_ok(c) || !has_fwd(c))
        return fail(ctx_ok(c) ? "context was created without the forward direction" : "NULL or invalid context");
    if (!valid_size(n, c->nmax)) return fail("n must be a power of two no larger than the context's nMax");
    if (!signal || !out) return fail("signal and output must be non-NULL");
    if (frames < 0 || frames > 0x7fffffffLL) return fail("frames must be in [0, 2^31)");
    if (hop < 0) return fail("hop must be >= 0");
    if (frame_len < 0 || frame_len > n) return fail("frame_len must be in [0, n]");
    if ((uintptr_t)out & 7) return fail("output must be 8-byte aligned");
    if (frames == 0) return 1;
    const __int128 sig = frame_len ? ((__int128)(frames - 1) * hop + frame_len) * 4 : 0;
    if (sig > ((__int128)1 << 62)) return fail("signal span too large");
    const size_t s_sig = (size_t)sig, s_out = (size_t)frames * (size_t)(n / 2 + 1) * 8,
                 s_win = window ? (size_t)n * 4 : 0;
    if (ranges_meet(signal, s_sig, out, s_out) || ranges_meet(window, s_win, out, s_out))
        return fail("input and output ranges overlap");
    Span sp[3] = {{signal, s_sig, false, nullptr, false},
                  {window, s_win, false, nullptr, false},
                  {out, s_out, true, nullptr, false}};
    return run_spans(c, sp, 3, stream, [&](cudaStream_t s) {
        return enqueue_stft(c, n, frames, (const float*)sp[0].dev, hop, (const float*)sp[1].dev, frame_len, scale,
                            (CkFftComplex*)sp[2].dev, s);
    });
}

int CkFftCudaFilterInverse(CkFftContext* c, int n, long long frames, const CkFftComplex* spectra,
                           const CkFftComplex* filter, float scale, float* out, void* stream)
{
    if (!ctx_ok(c) || !has_inv(c))
        return fail(ctx_ok(c) ? "context was created without the inverse direction" : "NULL or invalid context");
    if (!valid_size(n, c->nmax)) return fail("n must be a power of two no larger than the context's nMax");
    if (!spectra || !out) return fail("spectra and output must be non-NULL");
    if (frames < 0 || frames > 0x7fffffffLL) return fail("frames must be in [0, 2^31)");
    if ((uintptr_t)out & 7) return fail("output must be 8-byte aligned");
    if (frames == 0) return 1;
    const size_t bins = (size_t)(n / 2 + 1);
    const size_t s_in = (size_t)frames * bins * 8, s_out = (size_t)frames * (size_t)n * 4,
                 s_f = filter ? bins * 8 : 0;
    if (ranges_meet(spectra, s_in, out, s_out) || ranges_meet(filter, s_f, out, s_out))
        return fail("input and output ranges overlap");
    Span sp[3] = {{spectra, s_in, false, nullptr, false},
                  {filter, s_f, false, nullptr, false},
                  {out, s_out, true, nullptr, false}};
    return run_spans(c, sp, 3, stream, [&](cudaStream_t s) {
        return enqueue_filter(c, n, frames, (const CkFftComplex*)sp[0].dev, (const CkFftComplex*)sp[1].dev, scale,
                              (float*)sp[2].dev, s);
    });
}

long long CkFftCudaLaunchCount(void) { return ckg::launch_count(); }

}  // extern "C"
