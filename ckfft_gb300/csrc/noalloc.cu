// noalloc.cu -- CkFftCudaComplexBatchNoAlloc: complex batches that allocate nothing.
//
// Some callers cannot let a library allocate device memory while they run:
// a real-time audio callback cannot wait for cudaMalloc / cudaFree (both may
// synchronise the whole device and take unbounded time), a host embedding the
// library under a fixed memory budget must not see allocations fail or grow
// mid-stream, and code that owns the device's memory pool (another framework,
// a custom allocator) does not want a second allocator underneath it.  The
// regular batch entry points may allocate: staging buffers for host pointers,
// and the intermediate array of the multi-pass path for n > 2^14.
//
// This entry point takes device pointers only and keeps the multi-pass
// intermediate in one file-scope __device__ array of kNoAllocScratchBytes
// (8 MiB, 2^20 complex values).  Every GPU that loads the library holds that
// array until the process exits.  Consequences:
//   * n is limited to 2^20 (larger sizes are rejected with an error);
//   * every call on a device shares the one array, so calls whose work
//     overlaps on that GPU (different streams, or host threads racing) race
//     on it; callers must order such calls themselves;
//   * the array keeps the last call's contents; nothing in it has to start
//     at zero (pass 1 overwrites every element pass 2 reads).
// The array's device address is looked up with cudaGetSymbolAddress (the
// host-side name is only a stand-in, never a device address) once per device,
// with that device current, when the first context is created on it
// (prepare_noalloc, called from the per-device set-up of CkFftInit).  That
// look-up loads this file's module, so the 8 MiB is committed at context
// creation and the entry point itself only reads the cached pointer.  A
// cudaDeviceReset destroys the array with everything else on the device:
// after one, unload the library (or restart the process) before using it
// again, since the cached addresses would be stale.
#include <mutex>

#include "ckfft_cuda.h"
#include "kernels.h"

namespace ckg {


constexpr int kNoAllocMaxLog2 = 20;
constexpr size_t kNoAllocScratchBytes = sizeof(float2) << kNoAllocMaxLog2;   // 8 MiB

}  // namespace ckg

// The scratch array.  Host code may not use this name as an address (on the
// host it denotes a shadow variable); it must go through cudaGetSymbolAddress.
static __device__ __align__(256) float2 g_noalloc_scratch[1 << ckg::kNoAllocMaxLog2];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on `dev`, resolved by prepare_noalloc.
cudaError_t scratch_address(int dev, void** ptr)
{
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_addr[dev]) return cudaErrorNotReady;      // no context was created on dev
    *ptr = g_scratch_addr[dev];
    return cudaSuccess;
}

int fail(const char* msg)
{
    ckg::set_last_error(msg);
    return 0;
}

bool on_device(const void* p, int dev)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace

namespace ckg {

// Resolves the array's device address on the current device (idempotent).
cudaError_t prepare_noalloc()
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (g_scratch_addr[dev]) return cudaSuccess;
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = p;
    return cudaSuccess;
}

}  // namespace ckg

extern "C" int CkFftCudaComplexBatchNoAlloc(CkFftContext* context, int n, int count, int inverse,
                                            const CkFftComplex* input, CkFftComplex* output, void* stream)
{
    ckg::ContextView cv;
    if (!ckg::context_view(context, &cv)) return fail("NULL or invalid context");
    const int need_dir = inverse ? kCkFftDirection_Inverse : kCkFftDirection_Forward;
    if (!(cv.direction & need_dir)) return fail("context was created without this direction");
    if (n <= 0 || (n & (n - 1)) != 0 || n > cv.nmax)
        return fail("n must be a power of two no larger than the context's nMax");
    if (n > (1 << ckg::kNoAllocMaxLog2))
        return fail("CkFftCudaComplexBatchNoAlloc: n exceeds 2^20, the size its fixed 8 MiB scratch array holds");
    if (!input || !output || (const void*)input == (const void*)output)
        return fail("input and output must be distinct non-NULL buffers");
    if (count < 0) return fail("count must be >= 0");

    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) return fail("no CUDA device");
    if (prev != cv.device && cudaSetDevice(cv.device) != cudaSuccess) return fail("cannot select the context's device");
    int ok = 1;
    if (!on_device(input, cv.device) || !on_device(output, cv.device)) {
        ok = fail("CkFftCudaComplexBatchNoAlloc takes device (or managed) memory only; host buffers would need staging allocations");
    } else if (count > 0) {
        int log2n = 0;
        while ((1 << log2n) < n) ++log2n;
        cudaStream_t s = (cudaStream_t)stream;
        cudaError_t e;
        if (log2n <= ckg::kSmallMaxLog2Complex) {
            e = ckg::launch_small(inverse ? ckg::C2C_INV : ckg::C2C_FWD, log2n, input, output, count, n, n, cv.tw, s);
        } else {
            void* scratch = nullptr;
            e = scratch_address(cv.device, &scratch);
            if (e == cudaSuccess)
                e = ckg::launch_large_c2c(inverse != 0, log2n, input, output, count, n, n, cv.tw, scratch,
                                          ckg::kNoAllocScratchBytes, s);
        }
        if (e == cudaSuccess && !stream) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            ckg::set_last_error(cudaGetErrorString(e));
            ok = 0;
        }
    }
    if (prev >= 0 && prev != cv.device) cudaSetDevice(prev);
    return ok;
}
