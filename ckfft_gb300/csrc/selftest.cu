// selftest.cu -- CkFftCudaSelfTestWait: makes one of the library's bounded
// device-side waits run out on purpose and checks that it ends the way every
// such wait must: the kernel records an error code in the per-device error
// word, returns, the host call reports it, and the context keeps working.
//
// Nothing here faults, traps or hangs: the waits are for a condition that
// nothing ever sets (a job counter no unit increments, an mbarrier expecting
// bytes no copy delivers), with a short bound, and no copy is ever in flight.
#include <cstdio>
#include <cstring>
#include <vector>

#include "ckfft_cuda.h"
#include "jobs.h"
#include "kernels.h"
#include "tma.cuh"

namespace ckg {

constexpr unsigned kSelfErrCounter = 2u;    // the job kernel's counter timeout code
constexpr int kSelfTries = 1 << 12;

// One thread waits on an mbarrier that expects 16 bytes no copy will bring.
__global__ void k_selftest_mbar(unsigned* err, int tries)
{
    __shared__ __align__(8) unsigned long long bar;
    if (threadIdx.x != 0) return;
    mbar_init(smem_addr(&bar), 1);
    fence_mbar_init();
    mbar_arrive_expect_tx(smem_addr(&bar), 16);
    mbar_wait(smem_addr(&bar), 0, err, tries);
}

}  // namespace ckg

using namespace ckg;

namespace {

int st_fail(const char* what)
{
    set_last_error(what);
    return 0;
}

// The context still transforms: forward FFT of a unit impulse is all ones.
int context_still_works(CkFftContext* ctx, cudaStream_t s)
{
    const int n = 64;
    std::vector<CkFftComplex> x(n, CkFftComplex{0.f, 0.f}), y(n);
    x[0].real = 1.f;
    void *dx = nullptr, *dy = nullptr;
    if (cudaMalloc(&dx, sizeof(CkFftComplex) * n) != cudaSuccess ||
        cudaMalloc(&dy, sizeof(CkFftComplex) * n) != cudaSuccess) {
        cudaFree(dx);
        return st_fail("self-test: cannot allocate the check buffers");
    }
    int ok = cudaMemcpyAsync(dx, x.data(), sizeof(CkFftComplex) * n, cudaMemcpyHostToDevice, s) == cudaSuccess &&
             cudaStreamSynchronize(s) == cudaSuccess &&
             CkFftCudaComplexForwardBatch(ctx, n, 1, (const CkFftComplex*)dx, (CkFftComplex*)dy, nullptr) &&
             cudaMemcpy(y.data(), dy, sizeof(CkFftComplex) * n, cudaMemcpyDeviceToHost) == cudaSuccess;
    for (int k = 0; ok && k < n; ++k) ok = y[k].real == 1.f && y[k].imag == 0.f;
    cudaFree(dx);
    cudaFree(dy);
    return ok ? 1 : st_fail("self-test: the context no longer transforms correctly after the timed-out wait");
}

}  // namespace

extern "C" int CkFftCudaSelfTestWait(CkFftContext* context, int which)
{
    ContextView cv;
    if (!context_view(context, &cv)) return st_fail("NULL or invalid context");
    if (which != 0 && which != 1) return st_fail("which must be 0 (job counter) or 1 (bulk-copy barrier)");
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != cv.device && cudaSetDevice(cv.device) != cudaSuccess) return st_fail("cannot select the device");
    take_device_error();                          // start from a clear error word
    cudaStream_t s = nullptr;
    int rc = 0;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
        rc = st_fail("cannot create a stream");
    } else {
        cudaError_t e = cudaSuccess;
        unsigned want = 0;
        void* dmem = nullptr;
        if (which == 0) {
            // one phase unit that needs one finished unit of transform 0,
            // which no unit will ever report: its wait runs out, it is skipped
            want = kSelfErrCounter;
            UnitRec r{};
            r.u = Unit{U_COLS_FWD, 6, 6, 0, 1, 0, 1, B_IN | (B_SCRATCH << 4)};
            const size_t total = sizeof(UnitRec) + 2 * sizeof(int);
            std::vector<char> host(total, 0);
            memcpy(host.data(), &r, sizeof(UnitRec));
            e = cudaMalloc(&dmem, total);
            if (e == cudaSuccess) e = cudaMemcpyAsync(dmem, host.data(), total, cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) {
                JobsArgs a{};
                a.recs = (const UnitRec*)dmem;
                a.nunits = 1;
                a.done = (int*)((char*)dmem + sizeof(UnitRec));
                a.head = a.done + 1;
                a.tw = cv.tw;
                a.err = device_error_word();
                a.wait_tries = kSelfTries;
                e = launch_jobs_one(a, s);
            }
        } else {
            want = kErrWaitTimeout;
            k_selftest_mbar<<<1, 32, 0, s>>>(device_error_word(), kSelfTries);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        cudaFree(dmem);
        if (e != cudaSuccess) {
            char m[200];
            snprintf(m, sizeof m, "self-test: CUDA error %s", cudaGetErrorString(e));
            rc = st_fail(m);
        } else {
            const unsigned got = take_device_error();
            if (got != want) {
                char m[200];
                snprintf(m, sizeof m, "self-test: error word %u after the wait, expected %u", got, want);
                rc = st_fail(m);
            } else {
                rc = context_still_works(context, s);
            }
        }
        cudaStreamDestroy(s);
    }
    if (prev >= 0 && prev != cv.device) cudaSetDevice(prev);
    return rc;
}
