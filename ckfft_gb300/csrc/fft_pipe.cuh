// fft_pipe.cuh -- persistent, bulk-copy pipelined single-CTA transforms.
//
// Same arithmetic as fft_small.cuh (Stockham stages in registers, exchanges in
// padded shared memory, fused real split / merge), arranged for GB300's
// memory system: a CTA stays resident and walks frame groups g, g + grid,
// g + 2 grid, ...; each group of TPB frames is contiguous in HBM and arrives
// in shared memory through one cp.async.bulk (1-D TMA) copy that completes on
// an mbarrier.  NBUF buffers rotate, so while the CTA transforms group i the
// copies for groups i+1 .. i+NBUF-1 are already in flight: HBM reads overlap
// compute without spending registers or warps on outstanding loads.
//
// A buffer is first the landing zone of its group (frames back to back) and
// then, once every thread has read its inputs, the padded exchange area of the
// same group.  After the group's results are stored, thread 0 re-arms the
// buffer's barrier and issues the copy of the group NBUF steps ahead.
//
// Groups must be whole: the launcher runs the last count % TPB frames through
// the plain kernel, and uses this path only when the input pointer is 16-byte
// aligned and a group's byte count is a multiple of 16.
#pragma once
#include "fft_small.cuh"
#include "tma.cuh"

namespace ckg {

template <int L, int KIND, int NBUF>
struct PipeCfg {
    using C = SmallCfg<L>;
    static constexpr int N = 1 << L;
    static constexpr bool INV = KIND == C2C_INV || KIND == C2R;
    static constexpr int FRAME_IN = KIND == C2R ? N + 1 : N;            // float2 per input frame
    static constexpr unsigned GROUP_BYTES = (unsigned)(C::TPB * FRAME_IN * sizeof(float2));
    // float2 per buffer, rounded to 128 bytes so every buffer is a valid
    // bulk-copy destination (16-byte alignment is required)
    static constexpr int BUF = (C::TPB * C::SLOT + 15) / 16 * 16;
    static constexpr size_t SMEM = sizeof(float2) * (size_t)BUF * NBUF;
    static constexpr bool FITS = SMEM <= 227 * 1024;                     // per-CTA shared-memory limit
    static_assert(BUF >= C::TPB * FRAME_IN, "landing zone must fit the buffer");
};

template <int L, int KIND, int NBUF>
__global__ void __launch_bounds__(SmallCfg<L>::THREADS, SmallCfg<L>::MINB)
k_pipe(const float2* __restrict__ in, float2* __restrict__ out, long long ngroups, long long out_dist,
       const float2* __restrict__ tw, unsigned* err)
{
    using P = PipeCfg<L, KIND, NBUF>;
    using C = SmallCfg<L>;
    constexpr int N = P::N;
    extern __shared__ __align__(128) float2 smem[];
    __shared__ __align__(8) unsigned long long bars[NBUF];
    const int g = threadIdx.x / C::T, t = threadIdx.x % C::T;
    pdl_start();

    if (threadIdx.x == 0) {
        for (int b = 0; b < NBUF; ++b) mbar_init(smem_addr(&bars[b]), 1);
        fence_mbar_init();
    }
    __syncthreads();
    auto issue = [&](int b, long long grp) {
        const uint32_t bar = smem_addr(&bars[b]);
        mbar_arrive_expect_tx(bar, P::GROUP_BYTES);
        bulk_load(smem_addr(smem + b * P::BUF), in + grp * (long long)(C::TPB * P::FRAME_IN), P::GROUP_BYTES, bar);
    };
    if (threadIdx.x == 0) {
        for (int b = 0; b < NBUF; ++b) {
            const long long grp = blockIdx.x + (long long)b * gridDim.x;
            if (grp < ngroups) issue(b, grp);
        }
    }

    long long failed_at = -1;
    for (long long i = 0;; ++i) {
        const long long grp = blockIdx.x + i * gridDim.x;
        if (grp >= ngroups) break;
        const int b = (int)(i % NBUF);
        const uint32_t phase = (uint32_t)((i / NBUF) & 1);
        float2* buf = smem + b * P::BUF;
        const bool ok = mbar_wait(smem_addr(&bars[b]), phase, err);
        const float2* land = buf + g * P::FRAME_IN;
        float2 v[C::R];
        if constexpr (KIND == C2R) {
            constexpr int M = N;
            const float2* twn = tw + 2 * M;
            const float2 w0 = __ldg(twn + t);
            static_for<0, C::R>([&](auto mc) {
                constexpr int m = decltype(mc)::value;
                const int p = t + m * C::T;
                v[m] = real_merge(land[p], land[M - p], split_twiddle<C::R, m, false>(w0, twn, p));
            });
        } else {
#pragma unroll
            for (int m = 0; m < C::R; ++m) v[m] = land[t + m * C::T];
        }
        // every input is in registers before exchanges reuse the buffer; a
        // timed-out wait anywhere stops the whole CTA
        if (__syncthreads_or(!ok)) { failed_at = i; break; }
        PaddedView view{buf + g * C::SLOT};
        stockham<L, C::LOG2R, P::INV, C::WARP>(v, t, tw, view);
        const long long f = grp * C::TPB + g;
        if constexpr (KIND == R2C) {
            constexpr int M = N;
#pragma unroll
            for (int m = 0; m < C::R; ++m) view.st(t + m * C::T, v[m]);
            xsync<C::WARP>();
            split_store<C, M>(view, RowOut{out + f * out_dist}, t, tw + 2 * M);
        } else {
            float2* dst = out + f * out_dist + t;
#pragma unroll
            for (int m = 0; m < C::R; ++m) __stcs(dst + m * C::T, v[m]);
        }
        __syncthreads();   // buffer b is free again
        if (threadIdx.x == 0) {
            const long long next = grp + (long long)NBUF * gridDim.x;
            if (next < ngroups) {
                fence_proxy_async_shared();
                issue(b, next);
            }
        }
    }
    if (failed_at >= 0 && threadIdx.x == 0) {
        // copies were issued for iterations failed_at .. failed_at + NBUF - 1;
        // give each a bounded chance to land before the CTA exits
        for (long long j = failed_at; j < failed_at + NBUF; ++j) {
            if (blockIdx.x + j * gridDim.x >= ngroups) break;
            const uint32_t bar = smem_addr(&bars[j % NBUF]);
            const uint32_t phase = (uint32_t)((j / NBUF) & 1);
            for (int it = 0; it < 4096 && !mbar_try_wait(bar, phase); ++it) {
            }
        }
    }
}

// Resident CTAs per SM for a pipelined kernel (cached per instantiation).
template <int L, int KIND, int NBUF>
int pipe_grid(long long ngroups)
{
    using P = PipeCfg<L, KIND, NBUF>;
    static int per_sm = -1, sms = 0;
    if (per_sm < 0) {
        int dev = 0, nb = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_pipe<L, KIND, NBUF>, SmallCfg<L>::THREADS, P::SMEM) != cudaSuccess)
            nb = 1;
        per_sm = nb > 0 ? nb : 1;
    }
    const long long cap = (long long)per_sm * sms;
    return (int)(ngroups < cap ? ngroups : cap);
}

template <int L, int KIND, int NBUF>
cudaError_t attr_pipe()
{
    using P = PipeCfg<L, KIND, NBUF>;
    if constexpr (!P::FITS) {
        return cudaSuccess;
    } else {
        cudaError_t e = cudaFuncSetAttribute(k_pipe<L, KIND, NBUF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P::SMEM);
        if (e != cudaSuccess) return e;
        return cudaFuncSetAttribute(k_pipe<L, KIND, NBUF>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    }
}

// Runs the whole groups of a batch through k_pipe; returns frames handled
// (0 when the pipelined path does not apply).  in_dist/out_dist in float2.
template <int L, int KIND, int NBUF>
cudaError_t launch_pipe(const void* in, void* out, long long count, long long in_dist, long long out_dist,
                        const float2* tw, unsigned* err, cudaStream_t s, long long* done)
{
    using P = PipeCfg<L, KIND, NBUF>;
    using C = SmallCfg<L>;
    *done = 0;
    if constexpr (!P::FITS) {
        return cudaSuccess;
    } else {
        const long long ngroups = count / C::TPB;
        if (ngroups < 1 || in_dist != P::FRAME_IN || ((uintptr_t)in & 15) || (P::GROUP_BYTES & 15) || !err)
            return cudaSuccess;
        const int grid = pipe_grid<L, KIND, NBUF>(ngroups);
        const cudaError_t e = launch_pdl(k_pipe<L, KIND, NBUF>, dim3(grid), dim3(C::THREADS), P::SMEM, s,
                                         (const float2*)in, (float2*)out, ngroups, out_dist, tw, err);
        *done = ngroups * C::TPB;
        return e;
    }
}

}  // namespace ckg
