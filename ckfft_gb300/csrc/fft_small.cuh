// fft_small.cuh -- single-CTA transforms (complex up to 2^14, real up to 2^15).
//
// One kernel launch covers a whole batch.  A CTA holds TPB transforms; each
// transform is owned by T = N/R threads with R values in registers.  Data is
// read from HBM once (coalesced over t) and written once, every intermediate
// stage exchanges through shared memory, and the real-input split / merge
// steps of the reference (src/ckfft/fft_real_default.cpp:23-62, 79-111) are
// fused into the kernel's last / first step.
#pragma once
#include "fft_core.cuh"
#include "kernels.h"
#include "tuning_table.h"

namespace ckg {

// Values per thread (log2) for a transform of 2^L points: the autotuned
// choice (tuning_table.h), the same for every kernel family of the size so
// that batched, pipelined, strided, fused and grouped kernels compute it
// with the same radices and produce the same bits.
__host__ __device__ constexpr int default_log2r(int L)
{
    return (L >= 0 && L < (int)(sizeof(kTunedLog2R) / sizeof(kTunedLog2R[0]))) ? kTunedLog2R[L] : 5;
}

// Per-size launch shape: R = 2^LR values per thread, T = n/R threads per
// transform, TPB transforms per CTA filling about CTH threads.  The default
// shape is the one most callers use; the batched kernels also come in the
// other shapes the autotuner measures (half / double the values per thread,
// 512- or 128-thread CTAs).
template <int L, int LR = default_log2r(L), int CTH = 256>
struct SmallCfg {
    static constexpr int LOG2R = LR;
    static constexpr int R = 1 << LOG2R;
    static constexpr int T = (1 << L) / R;
    static constexpr int TPB = T >= CTH ? 1 : CTH / T;
    static constexpr int THREADS = T * TPB;
    // resident CTAs asked of ptxas: 64 registers per thread for R <= 16, 128 for R = 32
    static constexpr int MINB = (R <= 16 ? 1024 : 512) / THREADS > 0 ? (R <= 16 ? 1024 : 512) / THREADS : 1;
    static constexpr bool WARP = T <= 32;                  // a transform never spans warps
    static constexpr int SLOT = padded_len(1 << L);        // shared slots per transform
    static constexpr size_t SMEM = sizeof(float2) * (size_t)SLOT * TPB;
};

// W_n^(t + m T) for the real split / merge, n = 2 R T: W_n^t * W_{2R}^m, the
// second factor a compile-time constant when 2R divides 32; else a table load.
template <int R, int M_, bool INV>
__device__ __forceinline__ float2 split_twiddle(float2 w_t, const float2* __restrict__ twn, int k)
{
    if constexpr (2 * R <= 32) return rot<2 * R, M_, INV>(w_t);
    else return tw_load<INV>(twn, k);
}

// ------------------------------------------------------------- accessors
// How a frame body reaches its input and output: element i of a frame (a
// complex value, or a packed pair of reals on the real side).

// Contiguous rows, streaming loads and stores (the batched layout).
struct RowIn {
    const float2* __restrict__ p;
    __device__ __forceinline__ float2 ld(long long i) const { return __ldcs(p + i); }
    __device__ __forceinline__ float2 ldg(long long i) const { return __ldg(p + i); }
};
struct RowOut {
    float2* __restrict__ p;
    __device__ __forceinline__ void st(long long i, float2 v) const { __stcs(p + i, v); }
};
// Complex element i at p[i * s].  Cached loads: with interleaved frames
// (small s, distance 1) the frames of one CTA share sectors.
struct StrideIn {
    const float2* __restrict__ p;
    long long s;
    __device__ __forceinline__ float2 ld(long long i) const { return __ldg(p + i * s); }
    __device__ __forceinline__ float2 ldg(long long i) const { return __ldg(p + i * s); }
};
struct StrideOut {
    float2* __restrict__ p;
    long long s;
    __device__ __forceinline__ void st(long long i, float2 v) const { p[i * s] = v; }
};
// Reals at p[j * s], read or written as packed pairs (x[2i], x[2i+1]).
struct PairIn {
    const float* __restrict__ p;
    long long s;
    __device__ __forceinline__ float2 ld(long long i) const
    {
        return make_float2(__ldg(p + 2 * i * s), __ldg(p + (2 * i + 1) * s));
    }
    __device__ __forceinline__ float2 ldg(long long i) const { return ld(i); }
};
struct PairOut {
    float* __restrict__ p;
    long long s;
    __device__ __forceinline__ void st(long long i, float2 v) const
    {
        p[2 * i * s] = v.x;
        p[(2 * i + 1) * s] = v.y;
    }
};

// Elements read from a frame's shared-memory slot.
struct SlotIn {
    PaddedView v;
    __device__ __forceinline__ float2 ld(long long i) const { return v.ld((int)i); }
    __device__ __forceinline__ float2 ldg(long long i) const { return v.ld((int)i); }
};

// Real forward split of a natural-order half-length spectrum Z held in the
// view, written as the n/2+1 = M+1 output bins.  Bins k and M-k come from the
// same pair: with S = z_k + conj z_{M-k}, D = z_k - conj z_{M-k}, P = W_n^k D,
//   X[k] = S - iP,   X[M-k] = conj(S + iP)
// (the reference's two per-bin formulas, src/ckfft/fft_real_default.cpp:30-58,
// share S, D and the twiddle because W_n^{M-k} = -conj W_n^k).  Thread t
// takes k = t + mT for m < R/2; thread 0 also takes the middle bin k = M/2.
template <class C, int M, class View, class Dst>
__device__ __forceinline__ void split_store(const View& view, const Dst& dst, int t,
                                            const float2* __restrict__ twn)
{
    const float2 w0 = __ldg(twn + t);
    static_for<0, C::R / 2>([&](auto mc) {
        constexpr int m = decltype(mc)::value;
        const int k = t + m * C::T;
        const float2 z0 = view.ld(k), z1 = view.ld((M - k) & (M - 1));
        const float2 w = split_twiddle<C::R, m, false>(w0, twn, k);
        const float sx = z0.x + z1.x, sy = z0.y - z1.y;
        const float dx = z0.x - z1.x, dy = z0.y + z1.y;
        const float px = fmaf(w.x, dx, -w.y * dy), py = fmaf(w.x, dy, w.y * dx);
        dst.st(k, make_float2(sx + py, sy - px));
        dst.st(M - k, make_float2(sx - py, -(sy + px)));
    });
    if (t == 0) {
        const float2 z = view.ld(M / 2);                // X[M/2] = 2 conj Z[M/2]
        dst.st(M / 2, make_float2(z.x + z.x, -(z.y + z.y)));
    }
}

// ------------------------------------------------------- one-frame bodies
// The T threads t = 0..T-1 of a group transform one frame between device
// pointers; `live == false` keeps the group in step (barriers) without
// touching memory.  Used by the batched kernels below and by the persistent
// job kernel (fft_jobs.cu).

template <int L, bool INV, class Src, class Dst, class C = SmallCfg<L>>
__device__ __forceinline__ void frame_c2c_at(const Src& src, const Dst& dst, bool live, int t,
                                             const PaddedView& view, const float2* __restrict__ tw)
{
    float2 v[C::R];
    if (live) {
#pragma unroll
        for (int m = 0; m < C::R; ++m) v[m] = src.ld(t + m * C::T);
    } else {
#pragma unroll
        for (int m = 0; m < C::R; ++m) v[m] = make_float2(0.f, 0.f);
    }
    stockham<L, C::LOG2R, INV, C::WARP>(v, t, tw, view);
    if (live) {
#pragma unroll
        for (int m = 0; m < C::R; ++m) dst.st(t + m * C::T, v[m]);
    }
}

template <int L, bool INV>
__device__ __forceinline__ void frame_c2c(const float2* __restrict__ src, float2* __restrict__ dst, bool live,
                                          int t, const PaddedView& view, const float2* __restrict__ tw)
{
    frame_c2c_at<L, INV>(RowIn{src}, RowOut{dst}, live, t, view, tw);
}

// Real forward: n = 2M reals (read as M packed pairs) -> M+1 complex bins (2 DFT).
template <int LM, class Src, class Dst, class C = SmallCfg<LM>>
__device__ __forceinline__ void frame_r2c_at(const Src& src, const Dst& dst, bool live, int t,
                                             const PaddedView& view, const float2* __restrict__ tw)
{
    constexpr int M = 1 << LM;
    float2 v[C::R];
    if (live) {
#pragma unroll
        for (int m = 0; m < C::R; ++m) v[m] = src.ld(t + m * C::T);
    } else {
#pragma unroll
        for (int m = 0; m < C::R; ++m) v[m] = make_float2(0.f, 0.f);
    }
    stockham<LM, C::LOG2R, false, C::WARP>(v, t, tw, view);
    // natural-order half-size spectrum Z to shared memory, then split
#pragma unroll
    for (int m = 0; m < C::R; ++m) view.st(t + m * C::T, v[m]);
    xsync<C::WARP>();
    if (live) split_store<C, M>(view, dst, t, tw + 2 * M);
}

template <int LM>
__device__ __forceinline__ void frame_r2c(const float2* __restrict__ src, float2* __restrict__ dst, bool live,
                                          int t, const PaddedView& view, const float2* __restrict__ tw)
{
    frame_r2c_at<LM>(RowIn{src}, RowOut{dst}, live, t, view, tw);
}

// Real inverse: M+1 complex bins -> n = 2M reals (written as M packed pairs).
// The real inverse's first step: v[m] = merge(X[p], X[M-p]) at p = t + mT.
template <int LM, class Src, class C = SmallCfg<LM>>
__device__ __forceinline__ void c2r_load(const Src& src, bool live, int t, const float2* __restrict__ tw,
                                         float2 (&v)[C::R])
{
    constexpr int M = 1 << LM;
    const float2* twn = tw + 2 * M;
    if (live) {
        // both merge operands straight from HBM: X[p] coalesced ascending and
        // X[M-p] coalesced descending (the second read of each line hits cache)
        float2 a[C::R], b[C::R];
#pragma unroll
        for (int m = 0; m < C::R; ++m) {
            a[m] = src.ldg(t + m * C::T);
            b[m] = src.ldg(M - t - m * C::T);
        }
        const float2 w0 = __ldg(twn + t);
        static_for<0, C::R>([&](auto mc) {
            constexpr int m = decltype(mc)::value;
            v[m] = real_merge(a[m], b[m], split_twiddle<C::R, m, false>(w0, twn, t + m * C::T));
        });
    } else {
#pragma unroll
        for (int m = 0; m < C::R; ++m) v[m] = make_float2(0.f, 0.f);
    }
}

template <int LM, class Src, class Dst, class C = SmallCfg<LM>>
__device__ __forceinline__ void frame_c2r_at(const Src& src, const Dst& dst, bool live, int t,
                                             const PaddedView& view, const float2* __restrict__ tw)
{
    float2 v[C::R];
    c2r_load<LM, Src, C>(src, live, t, tw, v);
    stockham<LM, C::LOG2R, true, C::WARP>(v, t, tw, view);
    if (live) {
#pragma unroll
        for (int m = 0; m < C::R; ++m) dst.st(t + m * C::T, v[m]);
    }
}

template <int LM>
__device__ __forceinline__ void frame_c2r(const float2* __restrict__ src, float2* __restrict__ dst, bool live,
                                          int t, const PaddedView& view, const float2* __restrict__ tw)
{
    frame_c2r_at<LM>(RowIn{src}, RowOut{dst}, live, t, view, tw);
}

// ------------------------------------------------------------ batched kernels

// Frames of one or two threads (n = 4 .. 32 complex) read and write their
// elements T apart: one warp access touches up to 32 sectors.  In a
// contiguous batch the CTA instead moves its whole block of TPB frames
// (TPB * n consecutive values) through shared memory with coalesced loads
// and stores; each frame reads its values from a slot of n + 1 elements (an
// odd stride: no bank conflicts).  Measured on GB300 (batches of 1 GiB):
// n = 16 2036 -> 7084 GB/s, n = 8 3555 -> 7145, n = 32 3527 -> 5355; at
// n = 64 (four threads a frame) and n <= 2 the direct loads stay faster.
template <int L, bool INV>
__device__ __forceinline__ void block_c2c(const float2* __restrict__ in, float2* __restrict__ out, long long count,
                                          float2* smem, const float2* __restrict__ tw)
{
    using C = SmallCfg<L>;
    constexpr int N = 1 << L, SL = N + 1;
    static_assert(SL <= C::SLOT, "staging slots fit the frame slots");
    const long long f0 = (long long)blockIdx.x * C::TPB;
    const long long left = count - f0;
    const int total = (left < C::TPB ? (int)left : C::TPB) * N;
    const float2* src = in + f0 * N;
    for (int i = threadIdx.x; i < total; i += C::THREADS) smem[(i >> L) * SL + (i & (N - 1))] = __ldcs(src + i);
    __syncthreads();
    const int g = threadIdx.x / C::T, t = threadIdx.x % C::T;
    float2 v[C::R];
#pragma unroll
    for (int m = 0; m < C::R; ++m) v[m] = smem[g * SL + t + m * C::T];
    __syncthreads();                  // the exchange slots overlap other frames' staging slots
    stockham<L, C::LOG2R, INV, C::WARP>(v, t, tw, PaddedView{smem + g * C::SLOT});
    __syncthreads();
#pragma unroll
    for (int m = 0; m < C::R; ++m) smem[g * SL + t + m * C::T] = v[m];
    __syncthreads();
    float2* dst = out + f0 * N;
    for (int i = threadIdx.x; i < total; i += C::THREADS) __stcs(dst + i, smem[(i >> L) * SL + (i & (N - 1))]);
}

// The same for the real kernels (n = 2M = 8 .. 64; n = 16: 3695 -> 6839,
// n = 32: 2490 -> 5920 GB/s forward): the frame slots hold the
// staged input (M pairs, or M+1 bins), the split writes its bins in place in
// the slot (every thread owns the pairs (k, M-k) it reads), and the block
// of bins or pairs leaves with coalesced stores.
template <int LM>
__device__ __forceinline__ void block_r2c(const float2* __restrict__ in, float2* __restrict__ out, long long count,
                                          float2* smem, const float2* __restrict__ tw)
{
    using C = SmallCfg<LM>;
    constexpr int M = 1 << LM;
    const long long f0 = (long long)blockIdx.x * C::TPB;
    const long long left = count - f0;
    const int frames = left < C::TPB ? (int)left : C::TPB;
    const float2* src = in + f0 * M;
    for (int i = threadIdx.x; i < frames * M; i += C::THREADS)
        smem[(i >> LM) * C::SLOT + PaddedView::pad(i & (M - 1))] = __ldcs(src + i);
    __syncthreads();
    const int g = threadIdx.x / C::T, t = threadIdx.x % C::T;
    const PaddedView view{smem + g * C::SLOT};
    float2 v[C::R];
#pragma unroll
    for (int m = 0; m < C::R; ++m) v[m] = view.ld(t + m * C::T);
    xsync<C::WARP>();
    stockham<LM, C::LOG2R, false, C::WARP>(v, t, tw, view);
#pragma unroll
    for (int m = 0; m < C::R; ++m) view.st(t + m * C::T, v[m]);
    xsync<C::WARP>();
    split_store<C, M>(view, view, t, tw + 2 * M);
    __syncthreads();
    float2* dst = out + f0 * (M + 1);
    for (int i = threadIdx.x; i < frames * (M + 1); i += C::THREADS) {
        const int fr = i / (M + 1), k = i - fr * (M + 1);
        __stcs(dst + i, smem[fr * C::SLOT + PaddedView::pad(k)]);
    }
}

template <int LM>
__device__ __forceinline__ void block_c2r(const float2* __restrict__ in, float2* __restrict__ out, long long count,
                                          float2* smem, const float2* __restrict__ tw)
{
    using C = SmallCfg<LM>;
    constexpr int M = 1 << LM;
    const long long f0 = (long long)blockIdx.x * C::TPB;
    const long long left = count - f0;
    const int frames = left < C::TPB ? (int)left : C::TPB;
    const float2* src = in + f0 * (M + 1);
    for (int i = threadIdx.x; i < frames * (M + 1); i += C::THREADS) {
        const int fr = i / (M + 1), k = i - fr * (M + 1);
        smem[fr * C::SLOT + PaddedView::pad(k)] = __ldcs(src + i);
    }
    __syncthreads();
    const int g = threadIdx.x / C::T, t = threadIdx.x % C::T;
    const PaddedView view{smem + g * C::SLOT};
    float2 v[C::R];
    c2r_load<LM>(SlotIn{view}, true, t, tw, v);
    xsync<C::WARP>();
    stockham<LM, C::LOG2R, true, C::WARP>(v, t, tw, view);
#pragma unroll
    for (int m = 0; m < C::R; ++m) view.st(t + m * C::T, v[m]);
    __syncthreads();
    float2* dst = out + f0 * M;
    for (int i = threadIdx.x; i < frames * M; i += C::THREADS)
        __stcs(dst + i, smem[(i >> LM) * C::SLOT + PaddedView::pad(i & (M - 1))]);
}

template <int L, bool INV, int LR = default_log2r(L), int CTH = 256>
__global__ void __launch_bounds__(SmallCfg<L, LR, CTH>::THREADS, SmallCfg<L, LR, CTH>::MINB)
k_c2c_small(const float2* __restrict__ in, float2* __restrict__ out, long long count,
            long long in_dist, long long out_dist, const float2* __restrict__ tw)
{
    using C = SmallCfg<L, LR, CTH>;
    pdl_start();
    extern __shared__ float2 smem[];
    if constexpr (C::T <= 2 && L >= 2) {
        if (in_dist == (1ll << L) && out_dist == (1ll << L)) {
            block_c2c<L, INV>(in, out, count, smem, tw);
            return;
        }
    }
    const int g = threadIdx.x / C::T, t = threadIdx.x % C::T;
    const long long f = (long long)blockIdx.x * C::TPB + g;
    frame_c2c_at<L, INV, RowIn, RowOut, C>(RowIn{in + f * in_dist}, RowOut{out + f * out_dist}, f < count, t,
                                           PaddedView{smem + g * C::SLOT}, tw);
}

template <int LM, int LR = default_log2r(LM), int CTH = 256>
__global__ void __launch_bounds__(SmallCfg<LM, LR, CTH>::THREADS, SmallCfg<LM, LR, CTH>::MINB)
k_r2c_small(const float2* __restrict__ in, float2* __restrict__ out, long long count,
            long long in_dist, long long out_dist, const float2* __restrict__ tw)
{
    using C = SmallCfg<LM, LR, CTH>;
    pdl_start();
    extern __shared__ float2 smem[];
    if constexpr (C::T <= 2) {
        if (in_dist == (1ll << LM) && out_dist == (1ll << LM) + 1) {
            block_r2c<LM>(in, out, count, smem, tw);
            return;
        }
    }
    const int g = threadIdx.x / C::T, t = threadIdx.x % C::T;
    const long long f = (long long)blockIdx.x * C::TPB + g;
    frame_r2c_at<LM, RowIn, RowOut, C>(RowIn{in + f * in_dist}, RowOut{out + f * out_dist}, f < count, t,
                                       PaddedView{smem + g * C::SLOT}, tw);
}

template <int LM, int LR = default_log2r(LM), int CTH = 256>
__global__ void __launch_bounds__(SmallCfg<LM, LR, CTH>::THREADS, SmallCfg<LM, LR, CTH>::MINB)
k_c2r_small(const float2* __restrict__ in, float2* __restrict__ out, long long count,
            long long in_dist, long long out_dist, const float2* __restrict__ tw)
{
    using C = SmallCfg<LM, LR, CTH>;
    pdl_start();
    extern __shared__ float2 smem[];
    if constexpr (C::T <= 2) {
        if (in_dist == (1ll << LM) + 1 && out_dist == (1ll << LM)) {
            block_c2r<LM>(in, out, count, smem, tw);
            return;
        }
    }
    const int g = threadIdx.x / C::T, t = threadIdx.x % C::T;
    const long long f = (long long)blockIdx.x * C::TPB + g;
    frame_c2r_at<LM, RowIn, RowOut, C>(RowIn{in + f * in_dist}, RowOut{out + f * out_dist}, f < count, t,
                                       PaddedView{smem + g * C::SLOT}, tw);
}

// ---------------------------------------------------------------- launch

template <class C>
inline unsigned small_grid(long long count)
{
    return (unsigned)((count + C::TPB - 1) / C::TPB);
}

template <int L, bool INV, int LR = default_log2r(L), int CTH = 256>
cudaError_t launch_c2c_L(const void* in, void* out, long long count, long long in_dist,
                         long long out_dist, const float2* tw, cudaStream_t s)
{
    using C = SmallCfg<L, LR, CTH>;
    return launch_pdl(k_c2c_small<L, INV, LR, CTH>, dim3(small_grid<C>(count)), dim3(C::THREADS), C::SMEM, s,
                      (const float2*)in, (float2*)out, count, in_dist, out_dist, tw);
}

template <int LM, int LR = default_log2r(LM), int CTH = 256>
cudaError_t launch_r2c_L(const void* in, void* out, long long count, long long in_dist,
                         long long out_dist, const float2* tw, cudaStream_t s)
{
    using C = SmallCfg<LM, LR, CTH>;
    return launch_pdl(k_r2c_small<LM, LR, CTH>, dim3(small_grid<C>(count)), dim3(C::THREADS), C::SMEM, s,
                      (const float2*)in, (float2*)out, count, in_dist / 2, out_dist, tw);
}

template <int LM, int LR = default_log2r(LM), int CTH = 256>
cudaError_t launch_c2r_L(const void* in, void* out, long long count, long long in_dist,
                         long long out_dist, const float2* tw, cudaStream_t s)
{
    using C = SmallCfg<LM, LR, CTH>;
    return launch_pdl(k_c2r_small<LM, LR, CTH>, dim3(small_grid<C>(count)), dim3(C::THREADS), C::SMEM, s,
                      (const float2*)in, (float2*)out, count, in_dist, out_dist / 2, tw);
}

template <int L, bool INV, int LR = default_log2r(L), int CTH = 256>
cudaError_t attr_c2c_L()
{
    return cudaFuncSetAttribute(k_c2c_small<L, INV, LR, CTH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)SmallCfg<L, LR, CTH>::SMEM);
}
template <int LM, int LR = default_log2r(LM), int CTH = 256>
cudaError_t attr_real_L()
{
    cudaError_t e = cudaFuncSetAttribute(k_r2c_small<LM, LR, CTH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)SmallCfg<LM, LR, CTH>::SMEM);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_c2r_small<LM, LR, CTH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)SmallCfg<LM, LR, CTH>::SMEM);
}

// ---------------------------------------------------------- tuned shapes
// Kernel variants of a single-CTA size (variant_for): 0 the default shape,
// 2 / 3 the pipelined kernel (fft_pipe.cuh), 4 half the values per thread,
// 5 twice the values per thread, 6 CTAs of about 512 threads, 7 of about 128.
constexpr int kVariantHalfR = 4, kVariantDoubleR = 5, kVariantCta512 = 6, kVariantCta128 = 7;

template <int L, int V>
struct ShapeOf {
    static constexpr int LR0 = default_log2r(L);
    static constexpr int LR = V == kVariantHalfR ? LR0 - 1 : V == kVariantDoubleR ? LR0 + 1 : LR0;
    static constexpr int CTH = V == kVariantCta512 ? 512 : V == kVariantCta128 ? 128 : 256;
    static constexpr int T0 = 1 << (L - LR0);
    // a shape exists when it differs from the default and fits: 2..32 values
    // per thread, at most 1024 threads per transform, room in shared memory
    static constexpr bool kValid =
        L >= 6 && LR >= 1 && LR <= 5 && LR <= L && (L - LR) <= 10 &&
        (V == kVariantHalfR || V == kVariantDoubleR || (V == kVariantCta512 && T0 < 512) ||
         (V == kVariantCta128 && T0 < 256)) &&
        SmallCfg<L, (LR >= 1 ? LR : 1), CTH>::SMEM <= 227 * 1024;
};

}  // namespace ckg
