// fft_jobs.cu -- the persistent job kernel: a mixed run of transforms (sizes,
// kinds and directions all different) in one launch fed by a device queue.
//
// Every CTA stays resident and repeatedly takes the next unit (jobs.h) with
// one atomic add on the queue head, then runs the device function for that
// unit's operation and size:
//   * single-CTA units run the same frame bodies as the batched kernels
//     (fft_small.cuh), each group of T threads on its own frame pointer;
//   * column / row units (real: merge / split fused) run the multi-pass bodies
//     (fft_passes.cuh) with L2-only loads, because their inputs were written
//     by other CTAs earlier in this launch (L1 is not coherent across SMs).
// A phase unit first waits (bounded, thread 0, acquire load) for its
// transform's counter to reach `need`; when a unit of a transform finishes,
// thread 0 fences and adds one to the counter (release).  A wait that runs
// out records an error in the error word and the unit is skipped.
#include "fft_passes.cuh"
#include "fft_small.cuh"
#include "jobs.h"
#include "kernels.h"
#include "tma.cuh"

namespace ckg {

constexpr unsigned kErrCounterTimeout = 2u;

__device__ __forceinline__ bool wait_counter(const int* p, int need, unsigned* err, int tries)
{
    if (tries <= 0) tries = 1 << 26;
#pragma unroll 1
    for (int it = 0; it < tries; ++it) {
        int v;
        asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
        if (v >= need) return true;
        __nanosleep(64);
    }
    if (err) *(volatile unsigned*)err = kErrCounterTimeout;
    return false;
}

// ----------------------------------------------------------- unit bodies

template <int OP, int L>
__device__ __noinline__ void run_single(const UnitRec& r, const JobsArgs& a, float2* smem)
{
    using C = SmallCfg<L>;
    const int g = threadIdx.x / C::T, t = threadIdx.x % C::T;
    const bool live = g < r.u.count;
    FrameDesc fd{nullptr, nullptr};
    if (live) fd = r.frames[g];
    const PaddedView view{smem + g * C::SLOT};
    if constexpr (OP == U_C2C_FWD) frame_c2c<L, false>(fd.in, fd.out, live, t, view, a.tw);
    else if constexpr (OP == U_C2C_INV) frame_c2c<L, true>(fd.in, fd.out, live, t, view, a.tw);
    else if constexpr (OP == U_R2C) frame_r2c<L>(fd.in, fd.out, live, t, view, a.tw);
    else frame_c2r<L>(fd.in, fd.out, live, t, view, a.tw);
}

// Real n = 1, 2, 4 closed forms (src/ckfft/fft_real.cpp:20-93), one frame per thread.
__device__ __noinline__ void run_rtiny(const UnitRec& r, bool inv)
{
    const int g = threadIdx.x;
    if (g >= r.u.count) return;
    const FrameDesc fd = r.frames[g];
    const int n = 1 << r.u.log2a;
    if (!inv) {
        const float* x = (const float*)fd.in;
        float2* y = fd.out;
        if (n == 1) {
            y[0] = make_float2(x[0] * 2.0f, 0.0f);
        } else if (n == 2) {
            y[0] = make_float2((x[0] + x[1]) * 2.0f, 0.0f);
            y[1] = make_float2((x[0] - x[1]) * 2.0f, 0.0f);
        } else {
            const float s02 = (x[0] + x[2]) * 2.0f, d02 = (x[0] - x[2]) * 2.0f;
            const float s13 = (x[1] + x[3]) * 2.0f, d13 = (x[1] - x[3]) * 2.0f;
            y[0] = make_float2(s02 + s13, 0.0f);
            y[1] = make_float2(d02, -d13);
            y[2] = make_float2(s02 - s13, 0.0f);
        }
    } else {
        const float2* x = fd.in;
        float* y = (float*)fd.out;
        if (n == 1) {
            y[0] = x[0].x;
        } else if (n == 2) {
            y[0] = x[0].x + x[1].x;
            y[1] = x[0].x - x[1].x;
        } else {
            const float s02 = x[0].x + x[2].x, s13 = 2.0f * x[1].x;
            const float d02 = x[0].x - x[2].x, d13 = 2.0f * x[1].y;
            y[0] = s02 + s13;
            y[1] = d02 - d13;
            y[2] = s02 - s13;
            y[3] = d02 + d13;
        }
    }
}

__device__ __forceinline__ float2* pick(const LargeDesc& d, int sel)
{
    return sel == B_IN ? const_cast<float2*>(d.in) : sel == B_OUT ? d.out : d.scratch;
}

// A pass unit carries kJobThreads / THREADS whole tiles, one per subgroup.
template <int OP, int LS>
__device__ __noinline__ void run_pass(const UnitRec& r, const JobsArgs& a, float2* smem)
{
    using P = PassCfg<LS, kJobThreads>;
    const Unit& u = r.u;
    const int s = threadIdx.x / P::THREADS, tid = threadIdx.x % P::THREADS;
    const LargeDesc d = r.big;
    const float2* src = pick(d, u.sel & 15);
    float2* dst = pick(d, u.sel >> 4);
    float2* my = smem + s * P::SLOTS;
    const long long tile = (long long)u.first + s;
    if constexpr (OP == U_COLS_FWD) pass_cols<LS, false, true, kJobThreads>(src, dst, u.log2b, tile, tid, my, a.tw);
    else if constexpr (OP == U_COLS_INV) pass_cols<LS, true, true, kJobThreads>(src, dst, u.log2b, tile, tid, my, a.tw);
    else if constexpr (OP == U_ROWS_FWD) pass_rows_xt<LS, false, true, kJobThreads>(src, dst, u.log2b, tile, tid, my, a.tw);
    else if constexpr (OP == U_ROWS_INV) pass_rows_xt<LS, true, true, kJobThreads>(src, dst, u.log2b, tile, tid, my, a.tw);
    else if constexpr (OP == U_COLS_MERGE)
        pass_cols_merge<LS, kJobThreads, 16, true>(src, dst, u.log2b, tile, tid, my, a.tw);
    else pass_rows_split<LS, kJobThreads, true>(src, dst, u.log2b, tile, tid, my, a.tw, u.log2b);
}

// ---------------------------------------------------------------- dispatch

#define CKG_SINGLE_CASES(OP)                                                          \
    switch (u.log2a) {                                                                \
    case 0: if constexpr (OP <= U_C2C_INV) run_single<OP, 0>(r, a, smem); break;      \
    case 1: if constexpr (OP <= U_C2C_INV) run_single<OP, 1>(r, a, smem); break;      \
    case 2: run_single<OP, 2>(r, a, smem); break;                                     \
    case 3: run_single<OP, 3>(r, a, smem); break;                                     \
    case 4: run_single<OP, 4>(r, a, smem); break;                                     \
    case 5: run_single<OP, 5>(r, a, smem); break;                                     \
    case 6: run_single<OP, 6>(r, a, smem); break;                                     \
    case 7: run_single<OP, 7>(r, a, smem); break;                                     \
    case 8: run_single<OP, 8>(r, a, smem); break;                                     \
    case 9: run_single<OP, 9>(r, a, smem); break;                                     \
    case 10: run_single<OP, 10>(r, a, smem); break;                                   \
    case 11: run_single<OP, 11>(r, a, smem); break;                                   \
    case 12: run_single<OP, 12>(r, a, smem); break;                                   \
    default: break;                                                                   \
    }

#define CKG_PASS_CASES(OP)                                                            \
    switch (u.log2a) {                                                                \
    case 6: run_pass<OP, 6>(r, a, smem); break;                                       \
    case 7: run_pass<OP, 7>(r, a, smem); break;                                       \
    case 8: run_pass<OP, 8>(r, a, smem); break;                                       \
    case 9: run_pass<OP, 9>(r, a, smem); break;                                       \
    case 10: run_pass<OP, 10>(r, a, smem); break;                                     \
    default: break;                                                                   \
    }

template <int OP>
__device__ __forceinline__ void single_switch(const UnitRec& r, const JobsArgs& a, float2* smem)
{
    const Unit& u = r.u;
    CKG_SINGLE_CASES(OP)
}

template <int OP>
__device__ __forceinline__ void pass_switch(const UnitRec& r, const JobsArgs& a, float2* smem)
{
    const Unit& u = r.u;
    CKG_PASS_CASES(OP)
}

__device__ __forceinline__ void dispatch(const UnitRec& r, const JobsArgs& a, float2* smem)
{
    switch (r.u.op) {
    case U_C2C_FWD: single_switch<U_C2C_FWD>(r, a, smem); break;
    case U_C2C_INV: single_switch<U_C2C_INV>(r, a, smem); break;
    case U_R2C: single_switch<U_R2C>(r, a, smem); break;
    case U_C2R: single_switch<U_C2R>(r, a, smem); break;
    case U_RTINY_FWD: run_rtiny(r, false); break;
    case U_RTINY_INV: run_rtiny(r, true); break;
    case U_COLS_FWD: pass_switch<U_COLS_FWD>(r, a, smem); break;
    case U_COLS_INV: pass_switch<U_COLS_INV>(r, a, smem); break;
    case U_ROWS_FWD: pass_switch<U_ROWS_FWD>(r, a, smem); break;
    case U_ROWS_INV: pass_switch<U_ROWS_INV>(r, a, smem); break;
    case U_COLS_MERGE: pass_switch<U_COLS_MERGE>(r, a, smem); break;
    case U_ROWS_SPLIT: pass_switch<U_ROWS_SPLIT>(r, a, smem); break;
    default: break;
    }
}

__global__ void __launch_bounds__(kJobThreads, kJobCtasPerSm) k_jobs(JobsArgs a)
{
    extern __shared__ __align__(128) float2 smem[];
    constexpr int kSlots = 3;
    __shared__ __align__(128) UnitRec s_rec[kSlots];
    __shared__ __align__(8) unsigned long long s_bar[kSlots];
    __shared__ int s_idx[kSlots];
    __shared__ int s_ok[kSlots];
    // Iteration `it` works on the unit in slot it % 3 (index, record, go /
    // no-go).  Thread 0 keeps two units ahead: while the CTA works on one
    // unit, the next unit's record is on its way into the following slot
    // (one bulk copy) and the claim after it (one atomic add) is in flight.
    // One CTA barrier per unit: with three slots, the slot being refilled was
    // last read two units ago, before the previous unit's barrier; a phase
    // unit's completion is counted per warp (every warp fences and adds one),
    // so no barrier waits for the slowest warp at the end of a unit.
    // Deadlock-free: a CTA claims in increasing order, so the lowest-indexed
    // unfinished unit is some CTA's current unit, and it depends only on lower
    // indices, all of which are finished.
    constexpr uint32_t kRecBytes = sizeof(UnitRec);
    int next = 0;                         // thread 0: the claim after the slot being filled
    int stuck = -1;                       // thread 0: slot whose copy never completed
    if (threadIdx.x == 0) {
        for (int k = 0; k < kSlots; ++k) mbar_init(smem_addr(&s_bar[k]), 1);
        fence_mbar_init();
        const int cur = atomicAdd(a.head, 1);
        if (cur < a.nunits) {
            mbar_arrive_expect_tx(smem_addr(&s_bar[0]), kRecBytes);
            bulk_load(smem_addr(&s_rec[0]), a.recs + cur, kRecBytes, smem_addr(&s_bar[0]));
        }
        s_idx[0] = cur;
        next = atomicAdd(a.head, 1);
    }
    __syncthreads();
#pragma unroll 1
    for (int it = 0, slot = 0;; ++it, slot = slot == kSlots - 1 ? 0 : slot + 1) {
        if (s_idx[slot] >= a.nunits) break;
        const int nslot = slot == kSlots - 1 ? 0 : slot + 1;
        if (threadIdx.x == 0) {
            const bool got = mbar_wait(smem_addr(&s_bar[slot]), (uint32_t)(it / kSlots) & 1u, a.err);
            if (got && next < a.nunits) {
                fence_proxy_async_shared();
                mbar_arrive_expect_tx(smem_addr(&s_bar[nslot]), kRecBytes);
                bulk_load(smem_addr(&s_rec[nslot]), a.recs + next, kRecBytes, smem_addr(&s_bar[nslot]));
                s_idx[nslot] = next;
                next = atomicAdd(a.head, 1);
            } else {
                s_idx[nslot] = a.nunits;         // no unit left: the loop ends after this one
            }
            if (!got) {
                stuck = slot;
                s_ok[slot] = -1;
            } else {
                const Unit& u = s_rec[slot].u;
                s_ok[slot] = (u.job >= 0 && u.need > 0) ? (int)wait_counter(a.done + u.job, u.need, a.err, a.wait_tries) : 1;
            }
        }
        __syncthreads();
        const int ok = s_ok[slot];
        if (ok < 0) break;                   // a record never arrived (error word set)
        if (ok) dispatch(s_rec[slot], a, smem);
        const int job = s_rec[slot].u.job;
        if (job >= 0) {
            __syncwarp();
            if ((threadIdx.x & 31) == 0) {
                __threadfence();
                atomicAdd(a.done + job, 1);
            }
        }
    }
    // after a timed-out copy, wait for it again (bounded) before the CTA's
    // shared memory goes away; on the normal path no copy is in flight
    if (threadIdx.x == 0 && stuck >= 0) {
        for (int k = 0; k < 2; ++k) mbar_wait(smem_addr(&s_bar[stuck]), (uint32_t)k, nullptr);
    }
}

// ------------------------------------------------------------------ host

template <int L>
constexpr size_t single_smem()
{
    return sizeof(float2) * (size_t)SmallCfg<L>::SLOT * (kJobThreads / SmallCfg<L>::T);
}
template <int LS>
constexpr size_t pass_smem()
{
    return PassCfg<LS, kJobThreads>::SMEM * (kJobThreads / PassCfg<LS, kJobThreads>::THREADS);
}
constexpr size_t cmax(size_t a, size_t b) { return a > b ? a : b; }

size_t jobs_smem_bytes()
{
    size_t m = 0;
    m = cmax(m, single_smem<0>()); m = cmax(m, single_smem<1>());
    m = cmax(m, single_smem<2>()); m = cmax(m, single_smem<3>()); m = cmax(m, single_smem<4>());
    m = cmax(m, single_smem<5>()); m = cmax(m, single_smem<6>()); m = cmax(m, single_smem<7>());
    m = cmax(m, single_smem<8>()); m = cmax(m, single_smem<9>()); m = cmax(m, single_smem<10>());
    m = cmax(m, single_smem<11>()); m = cmax(m, single_smem<12>());
    m = cmax(m, pass_smem<6>()); m = cmax(m, pass_smem<7>()); m = cmax(m, pass_smem<8>());
    m = cmax(m, pass_smem<9>()); m = cmax(m, pass_smem<10>());
    return (m + 127) / 128 * 128;
}

int jobs_grid();

cudaError_t prepare_jobs()
{
    cudaError_t e = cudaFuncSetAttribute(k_jobs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)jobs_smem_bytes());
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_jobs, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return e;
    jobs_grid();
    return cudaSuccess;
}

// Resident CTAs of the job kernel on the current device (cached per device;
// safe to call during stream capture once cached).
int jobs_grid()
{
    static int cache[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && cache[dev]) return cache[dev];
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_jobs, kJobThreads, jobs_smem_bytes()) != cudaSuccess || per < 1)
        per = 1;
    const int g = per * (sms > 0 ? sms : 1);
    if (dev >= 0 && dev < 64) cache[dev] = g;
    return g;
}

cudaError_t launch_jobs_one(const JobsArgs& a, cudaStream_t s)
{
    k_jobs<<<1, kJobThreads, jobs_smem_bytes(), s>>>(a);
    return cudaGetLastError();
}

// Enqueues the job kernel (the caller counts the launch).
cudaError_t launch_jobs(const JobsArgs& a, cudaStream_t s)
{
    if (a.nunits <= 0) return cudaSuccess;
    const int grid = jobs_grid();
    k_jobs<<<grid < a.nunits ? grid : a.nunits, kJobThreads, jobs_smem_bytes(), s>>>(a);
    return cudaGetLastError();
}

}  // namespace ckg
