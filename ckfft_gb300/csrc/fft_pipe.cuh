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

// ------------------------------------------------ split-exchange form
// The landing zone and the exchange area kept apart (kernel variant 8): one
// landing buffer the size of a group, and an exchange area that moves the x
// parts, then the y parts, through a float image padded every 32 elements.  For frames too large for one buffer to be both
// twice over (2^14: 128 KiB a frame, 68 KiB of exchange area, 196 KiB a
// CTA), and for sizes where the smaller footprint lets two persistent CTAs
// share an SM (2^13: 98 KiB).  The copy of the next group is issued as soon
// as every thread holds its inputs, so it lands while this group's stages
// and stores run.  Same stages, twiddles and positions as the other forms:
// the same results bit for bit.
template <int L, int KIND>
struct PipeSxCfg {
    using C = SmallCfg<L>;
    static constexpr int N = 1 << L;                                  // complex (half) length
    static constexpr bool REAL = KIND == R2C || KIND == C2R;
    // bytes of one bulk copy: the group's frames (complex, real forward), or
    // for the real inverse the N bins from the first 16-byte aligned one
    static constexpr unsigned COPY_BYTES = (unsigned)(C::TPB * N * sizeof(float2));
    // landing slots; the real inverse's bins sit from slot 2 on, with one slot
    // either side for the bin fetched by a plain load
    static constexpr int LAND = KIND == C2R ? N + 4 : C::TPB * N;
    static constexpr int XLEN = N + (N >> 5) + 1;                     // floats per frame image
    static constexpr int XBUF = (C::TPB * XLEN + 3) / 4 * 4;          // floats (16-byte multiple)
    static constexpr size_t SMEM = sizeof(float2) * (size_t)LAND + sizeof(float) * (size_t)XBUF;
    // 32 values per thread (stage spans 1, 32, 1024, ...: compile-time image
    // offsets), one CTA's shared memory; real kinds one frame per CTA
    static constexpr bool FITS = SMEM <= 227 * 1024 && C::T % 32 == 0 && C::R == 32 && (!REAL || C::TPB == 1);
};

__device__ __forceinline__ int pad32(int pos) { return pos + (pos >> 5); }

// One exchange of a stage's outputs through the float image xa: every thread
// writes the x parts of its outputs to their Stockham positions and reloads
// the x parts of positions t + mT, then the same for the y parts.
template <int LOG2N, int LOG2R, int LRS, int LNS, bool WARP>
__device__ __forceinline__ void exchange_split(float2 (&v)[1 << LOG2R], int t, float* xa)
{
    constexpr int R = 1 << LOG2R, RS = 1 << LRS, NS = 1 << LNS;
    constexpr int T = (1 << LOG2N) / R, U = R / RS;
    static_assert(T % 32 == 0 && RS <= 32 && (NS == 1 || NS % 32 == 0), "compile-time image offsets");
    static_for<0, 2>([&](auto cc) {
        constexpr int comp = decltype(cc)::value;
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int b = t + u * T;
            const int base = ((b >> LNS) << (LNS + LRS)) + (b & (NS - 1));
            // base + j NS -> pad32(base) + j (NS == 1, base a multiple of
            // RS <= 32 ... here of 32 when RS = 32) or + j (NS + NS / 32)
            float* p = xa + pad32(base);
#pragma unroll
            for (int j = 0; j < RS; ++j) {
                const int off = NS == 1 ? j : j * (NS + NS / 32);
                p[off] = comp ? v[u + j * U].y : v[u + j * U].x;
            }
        }
        xsync<WARP>();
        const float* q = xa + pad32(t);
#pragma unroll
        for (int m = 0; m < R; ++m) {
            const float f = q[m * (T + T / 32)];
            if constexpr (comp) v[m].y = f;
            else v[m].x = f;
        }
        xsync<WARP>();
    });
}

template <int LOG2N, int LOG2R, bool INV, bool WARP>
__device__ __forceinline__ void stockham_split(float2 (&v)[1 << LOG2R], int t, const float2* __restrict__ tw, float* xa)
{
    using S = Sched<LOG2N, LOG2R>;
    static_for<0, S::nstages>([&](auto sc) {
        constexpr int st = decltype(sc)::value;
        stage_compute<LOG2N, LOG2R, S::lrs(st), S::lns(st), INV>(v, t, tw);
        if constexpr (st + 1 < S::nstages) exchange_split<LOG2N, LOG2R, S::lrs(st), S::lns(st), WARP>(v, t, xa);
    });
}

// The real forward's last stage in the paired layout: thread t owns the
// butterflies b_{2i} = t + i T and b_{2i+1} = NS - i T - t (NS / 2 for
// t = i = 0) instead of t + u T.  Butterfly b's outputs sit at b + j NS and
// those of NS - b at (NS - b) + (RS - 1 - j) NS = N - (b + j NS), so every
// pair (k, N - k) of the split is in one thread's registers.  Each butterfly
// is computed exactly as by stage_compute (its twiddles from k = b).
template <int T, int NS>
__device__ __forceinline__ int paired_butterfly(int t, int u)
{
    const int i = u >> 1;
    if ((u & 1) == 0) return t + i * T;
    return (t == 0 && i == 0) ? NS / 2 : NS - i * T - t;
}

template <int LOG2N, int LOG2R, bool WARP>
__device__ __forceinline__ void stockham_split_paired(float2 (&v)[1 << LOG2R], int t, const float2* __restrict__ tw,
                                                      float* xa)
{
    using S = Sched<LOG2N, LOG2R>;
    constexpr int NST = S::nstages;
    constexpr int R = 1 << LOG2R, T = (1 << LOG2N) / R;
    constexpr int LRS = S::lrs(NST - 1), LNS = S::lns(NST - 1);
    constexpr int RS = 1 << LRS, NS = 1 << LNS, U = R / RS;
    static_assert(NST >= 2 && U % 2 == 0 && NS % 32 == 0 && NS == U * T, "paired last stage");
    static_for<0, NST - 1>([&](auto sc) {
        constexpr int st = decltype(sc)::value;
        stage_compute<LOG2N, LOG2R, S::lrs(st), S::lns(st), false>(v, t, tw);
        if constexpr (st + 2 < NST) {
            exchange_split<LOG2N, LOG2R, S::lrs(st), S::lns(st), WARP>(v, t, xa);
        } else {
            // the last exchange: written as by exchange_split, read back in
            // the paired layout, v[u + j U] = position b_u + j NS
            constexpr int LRS0 = S::lrs(st), LNS0 = S::lns(st);
            constexpr int RS0 = 1 << LRS0, NS0 = 1 << LNS0, U0 = R / RS0;
            static_for<0, 2>([&](auto cc) {
                constexpr int comp = decltype(cc)::value;
#pragma unroll
                for (int u = 0; u < U0; ++u) {
                    const int b = t + u * T;
                    const int base = ((b >> LNS0) << (LNS0 + LRS0)) + (b & (NS0 - 1));
                    float* p = xa + pad32(base);
#pragma unroll
                    for (int j = 0; j < RS0; ++j) {
                        const int off = NS0 == 1 ? j : j * (NS0 + NS0 / 32);
                        p[off] = comp ? v[u + j * U0].y : v[u + j * U0].x;
                    }
                }
                xsync<WARP>();
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const float* q = xa + pad32(paired_butterfly<T, NS>(t, u));
#pragma unroll
                    for (int j = 0; j < RS; ++j) {
                        const float f = q[j * (NS + NS / 32)];
                        if constexpr (comp) v[u + j * U].y = f;
                        else v[u + j * U].x = f;
                    }
                }
                xsync<WARP>();
            });
        }
    });
    // the last stage, butterfly by butterfly (stage_compute's arithmetic)
    static_for<0, U>([&](auto uc) {
        constexpr int u = decltype(uc)::value;
        float2 x[RS];
#pragma unroll
        for (int j = 0; j < RS; ++j) x[j] = v[u + j * U];
        const int k = paired_butterfly<T, NS>(t, u);
        float2 w[RS];
#pragma unroll
        for (int p = 1; p < RS; p <<= 1) w[p] = tw_load<false>(tw + NS * RS / p, k);
#pragma unroll
        for (int j = 3; j < RS; ++j) {
            if ((j & (j - 1)) == 0) continue;
            const int hb = 1 << (31 - __clz(j));
            w[j] = cmul(w[hb], w[j - hb]);
        }
#pragma unroll
        for (int j = 1; j < RS; ++j) x[j] = cmul(x[j], w[j]);
        dft<RS, false>(x);
#pragma unroll
        for (int j = 0; j < RS; ++j) v[u + j * U] = x[j];
    });
}

// in_dist / out_dist in float2 (real sides: packed pairs of reals).
// C2C_FWD / C2C_INV: frames of N values back to back (in_dist = N), 16-byte
// aligned.  R2C: N packed pairs in (in_dist = N, 16-byte aligned), N + 1 bins
// out, the split through the float image.  C2R: N + 1 bins in (any in_dist),
// N packed pairs out, the merge straight from the landing zone.
template <int L, int KIND>
__global__ void __launch_bounds__(SmallCfg<L>::THREADS, SmallCfg<L>::MINB)
k_pipe_sx(const float2* __restrict__ in, float2* __restrict__ out, long long ngroups, long long in_dist,
          long long out_dist, const float2* __restrict__ tw, unsigned* err)
{
    using P = PipeSxCfg<L, KIND>;
    using C = SmallCfg<L>;
    constexpr int N = P::N;
    constexpr bool INV = KIND == C2C_INV || KIND == C2R;
    extern __shared__ __align__(128) float2 smem[];
    __shared__ __align__(8) unsigned long long bar;
    float* xa = reinterpret_cast<float*>(smem + P::LAND);
    const int g = threadIdx.x / C::T, t = threadIdx.x % C::T;
    const uint32_t b = smem_addr(&bar);
    pdl_start();
    if (threadIdx.x == 0) {
        mbar_init(b, 1);
        fence_mbar_init();
    }
    __syncthreads();
    // real inverse: bin k of the frame at slot 2 + k - o, o = 1 when the
    // frame's first bin is not 16-byte aligned (bins in pairs of 16 bytes)
    auto odd = [&](long long grp) { return (int)(((uintptr_t)(in + grp * in_dist) >> 3) & 1); };
    auto issue = [&](long long grp) {
        const float2* src = in + grp * in_dist;
        mbar_arrive_expect_tx(b, P::COPY_BYTES);
        if constexpr (KIND == C2R) {
            // bins o .. o + N - 1 by bulk copy, the remaining one (N or 0) by
            // a plain load outside the copied slots
            const int o = odd(grp);
            bulk_load(smem_addr(smem + 2), src + o, P::COPY_BYTES, b);
            const int extra = o ? 0 : N;
            smem[2 + extra - o] = src[extra];
        } else {
            bulk_load(smem_addr(smem), src, P::COPY_BYTES, b);
        }
    };
    if (threadIdx.x == 0 && (long long)blockIdx.x < ngroups) issue(blockIdx.x);
    if constexpr (KIND == C2R) __syncthreads();            // the first frame's plain-loaded bin

    long long failed_at = -1;
    for (long long i = 0;; ++i) {
        const long long grp = blockIdx.x + i * gridDim.x;
        if (grp >= ngroups) break;
        const bool ok = mbar_wait(b, (uint32_t)(i & 1), err);
        float2 v[C::R];
        if constexpr (KIND == C2R) {
            // the merge of c2r_load, operands from the landing zone
            const float2* land = smem + 2 - odd(grp);
            const float2* twn = tw + 2 * N;
            const float2 w0 = __ldg(twn + t);
            static_for<0, C::R>([&](auto mc) {
                constexpr int m = decltype(mc)::value;
                const int p = t + m * C::T;
                v[m] = real_merge(land[p], land[N - p], split_twiddle<C::R, m, false>(w0, twn, p));
            });
        } else {
            const float2* land = smem + g * N;
#pragma unroll
            for (int m = 0; m < C::R; ++m) v[m] = land[t + m * C::T];
        }
        // every input is in registers before the next copy overwrites the
        // landing zone; a timed-out wait anywhere stops the whole CTA
        if (__syncthreads_or(!ok)) { failed_at = i; break; }
        if (threadIdx.x == 0) {
            const long long next = grp + gridDim.x;
            if (next < ngroups) {
                fence_proxy_async_shared();
                issue(next);
            }
        }
        float* img = xa + g * P::XLEN;
        if constexpr (KIND == R2C) {
            // the last stage in the paired layout: both members of every
            // split pair in this thread's registers; the split of split_store
            // (same operands, twiddle W_2N^k of k = min(p, N - p)) from them
            stockham_split_paired<L, C::LOG2R, C::WARP>(v, t, tw, img);
            using S = Sched<L, C::LOG2R>;
            constexpr int LRS = S::lrs(S::nstages - 1), LNS = S::lns(S::nstages - 1);
            constexpr int RS = 1 << LRS, NS = 1 << LNS, U = C::R / RS;
            float2* dst = out + grp * out_dist;
            const float2* twn = tw + 2 * N;
            auto split_pair = [&](int k, float2 z0, float2 z1) {
                const float2 w = tw_load<false>(twn, k);
                const float sx = z0.x + z1.x, sy = z0.y - z1.y;
                const float dx = z0.x - z1.x, dy = z0.y + z1.y;
                const float px = fmaf(w.x, dx, -w.y * dy), py = fmaf(w.x, dy, w.y * dx);
                __stcs(dst + k, make_float2(sx + py, sy - px));
                __stcs(dst + (N - k), make_float2(sx - py, -(sy + px)));
            };
            static_for<0, U / 2>([&](auto ic) {
                constexpr int i = decltype(ic)::value;
                constexpr int u = 2 * i;
                if (i == 0 && t == 0) {
                    // butterflies 0 and NS / 2 pair with themselves
#pragma unroll
                    for (int j = 0; j < RS / 2; ++j) {
                        split_pair(j * NS, v[u + j * U], v[u + ((RS - j) & (RS - 1)) * U]);
                        split_pair(NS / 2 + j * NS, v[u + 1 + j * U], v[u + 1 + (RS - 1 - j) * U]);
                    }
                    const float2 z = v[u + (RS / 2) * U];          // X[N/2] = 2 conj Z[N/2]
                    __stcs(dst + N / 2, make_float2(z.x + z.x, -(z.y + z.y)));
                } else {
                    const int b = paired_butterfly<C::T, NS>(t, u);
#pragma unroll
                    for (int j = 0; j < RS; ++j) {
                        const int p = b + j * NS;
                        const float2 zp = v[u + j * U], zq = v[u + 1 + (RS - 1 - j) * U];
                        if (p < N - p) split_pair(p, zp, zq);
                        else split_pair(N - p, zq, zp);
                    }
                }
            });
        } else {
            stockham_split<L, C::LOG2R, INV, C::WARP>(v, t, tw, img);
            float2* dst = out + (grp * C::TPB + g) * out_dist + t;
#pragma unroll
            for (int m = 0; m < C::R; ++m) __stcs(dst + m * C::T, v[m]);
        }
    }
    if (failed_at >= 0 && threadIdx.x == 0) {
        // the copy of iteration failed_at may still be in flight: give it a
        // bounded chance to land before the CTA exits
        for (int it = 0; it < 4096 && !mbar_try_wait(b, (uint32_t)(failed_at & 1)); ++it) {
        }
    }
}

template <int L, int KIND>
int pipe_sx_grid(long long ngroups)
{
    using P = PipeSxCfg<L, KIND>;
    static int per_sm = -1, sms = 0;
    if (per_sm < 0) {
        int dev = 0, nb = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_pipe_sx<L, KIND>, SmallCfg<L>::THREADS, P::SMEM) !=
            cudaSuccess)
            nb = 1;
        per_sm = nb > 0 ? nb : 1;
    }
    const long long cap = (long long)per_sm * sms;
    return (int)(ngroups < cap ? ngroups : cap);
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

template <int L, int KIND>
cudaError_t attr_pipe_sx()
{
    using X = PipeSxCfg<L, KIND>;
    if constexpr (!X::FITS) {
        return cudaSuccess;
    } else {
        cudaError_t e = cudaFuncSetAttribute(k_pipe_sx<L, KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)X::SMEM);
        if (e != cudaSuccess) return e;
        return cudaFuncSetAttribute(k_pipe_sx<L, KIND>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    }
}

// Runs the whole groups of a batch through k_pipe_sx; in_dist / out_dist in
// float2 (packed pairs on the real sides).  Frames handled in *done (0 when
// the form does not apply: complex and real forward inputs must be frames
// back to back, 16-byte aligned; real inverse bins 8-byte aligned).
template <int L, int KIND>
cudaError_t launch_pipe_sx(const void* in, void* out, long long count, long long in_dist, long long out_dist,
                           const float2* tw, unsigned* err, cudaStream_t s, long long* done)
{
    using X = PipeSxCfg<L, KIND>;
    using C = SmallCfg<L>;
    *done = 0;
    if constexpr (!X::FITS) {
        return cudaSuccess;
    } else {
        const long long ngroups = count / C::TPB;
        if (ngroups < 1 || !err || (X::COPY_BYTES & 15)) return cudaSuccess;
        if (KIND == C2R ? (in_dist < X::N + 1 || ((uintptr_t)in & 7)) : (in_dist != X::N || ((uintptr_t)in & 15)))
            return cudaSuccess;
        const int grid = pipe_sx_grid<L, KIND>(ngroups);
        const cudaError_t e = launch_pdl(k_pipe_sx<L, KIND>, dim3(grid), dim3(C::THREADS), X::SMEM, s,
                                         (const float2*)in, (float2*)out, ngroups, in_dist, out_dist, tw, err);
        *done = ngroups * C::TPB;
        return e;
    }
}

}  // namespace ckg
