// fft_inter.cu -- strided batches whose consecutive transforms are adjacent
// in memory (distance 1): interleaved channels, columns of a row-major
// matrix.  Element p of transform f sits at base[f + p * stride], so one
// transform's elements are a stride apart while G consecutive transforms
// share every row.  A CTA takes G consecutive transforms and moves the
// G-wide rows between HBM and its shared-memory slots with all of its
// threads, transform index fastest: each row segment is G * 8 bytes (G * 4
// for reals) of consecutive addresses, whole 32-byte sectors, instead of one
// sector per element.  The transforms then run from the slots exactly as in
// the batched kernels.
//
// Covered: complex 2^6 .. 2^13 (either side or both interleaved), real
// forward with interleaved reals, real inverse with interleaved reals, real
// n = 2^7 .. 2^14.  G is at least 16 (rows of 128 bytes and more) up to
// 2^10, then 8, 4 and 2 transforms per 1024-thread CTA at 2^11, 2^12, 2^13.
#include "fft_small.cuh"

namespace ckg {

template <int L>
struct InterCfg {
    using S = SmallCfg<L>;
    static constexpr int LOG2R = S::LOG2R, R = S::R, T = S::T;
    // transforms per CTA: rows of at least 128 bytes (G >= 16) where 1024
    // threads and the shared memory allow, else 4 (2 at 2^13)
    static constexpr int G = S::TPB >= 16 ? S::TPB : L <= 10 ? 16 : L == 11 ? 8 : L == 12 ? 4 : 2;
    static constexpr int THREADS = T * G;
    // resident CTAs asked of ptxas: 64 registers a thread up to 16 values, 128 for 32
    static constexpr int MINB = (R <= 16 ? 1024 : 512) / THREADS > 0 ? (R <= 16 ? 1024 : 512) / THREADS : 1;
    static constexpr bool WARP = S::WARP;
    static constexpr int SLOT = S::SLOT;
    static constexpr size_t SMEM = sizeof(float2) * (size_t)SLOT * G;
    static_assert(THREADS <= 1024, "one CTA");
};

// Rows [0, N) of G transforms (h < live) from `base` (transform h at
// base + h * dist) into the slots; missing transforms read as zero.
template <class C, int N>
__device__ __forceinline__ void rows_in(const float2* __restrict__ base, long long dist, long long stride, int live,
                                        float2* smem)
{
#pragma unroll
    for (int k = 0; k < N * C::G / C::THREADS; ++k) {
        const int idx = threadIdx.x + k * C::THREADS;
        const int h = idx % C::G, p = idx / C::G;
        float2 x = make_float2(0.f, 0.f);
        if (h < live) x = __ldcs(base + h * dist + (long long)p * stride);
        PaddedView{smem + h * C::SLOT}.st(p, x);
    }
}

template <class C, int N>
__device__ __forceinline__ void rows_out(float2* __restrict__ base, long long dist, long long stride, int live,
                                         const float2* smem)
{
#pragma unroll
    for (int k = 0; k < N * C::G / C::THREADS; ++k) {
        const int idx = threadIdx.x + k * C::THREADS;
        const int h = idx % C::G, p = idx / C::G;
        if (h < live) __stcs(base + h * dist + (long long)p * stride, PaddedView{(float2*)smem + h * C::SLOT}.ld(p));
    }
}

// The same for reals: sample j of a transform is component j & 1 of the
// packed pair j >> 1 in its slot.
template <class C, int N2>
__device__ __forceinline__ void reals_in(const float* __restrict__ base, long long dist, long long stride, int live,
                                         float2* smem)
{
#pragma unroll
    for (int k = 0; k < N2 * C::G / C::THREADS; ++k) {
        const int idx = threadIdx.x + k * C::THREADS;
        const int h = idx % C::G, j = idx / C::G;
        float x = 0.f;
        if (h < live) x = __ldcs(base + h * dist + (long long)j * stride);
        reinterpret_cast<float*>(smem + h * C::SLOT + PaddedView::pad(j >> 1))[j & 1] = x;
    }
}

template <class C, int N2>
__device__ __forceinline__ void reals_out(float* __restrict__ base, long long dist, long long stride, int live,
                                          const float2* smem)
{
#pragma unroll
    for (int k = 0; k < N2 * C::G / C::THREADS; ++k) {
        const int idx = threadIdx.x + k * C::THREADS;
        const int h = idx % C::G, j = idx / C::G;
        if (h < live)
            __stcs(base + h * dist + (long long)j * stride,
                   reinterpret_cast<const float*>(smem + h * C::SLOT + PaddedView::pad(j >> 1))[j & 1]);
    }
}

struct Group {
    int g, t, live;     // transform slot, thread within it, transforms present in this CTA
    long long f0, f;    // first transform of the CTA, this slot's transform (f0 when absent)
};

template <class C>
__device__ __forceinline__ Group group_of(long long count)
{
    Group q;
    q.g = threadIdx.x / C::T;
    q.t = threadIdx.x % C::T;
    q.f0 = (long long)blockIdx.x * C::G;
    const long long rem = count - q.f0;
    q.live = rem < C::G ? (int)rem : C::G;
    q.f = q.g < q.live ? q.f0 + q.g : q.f0;
    return q;
}

template <int L, bool INV, bool CIN, bool COUT>
__global__ void __launch_bounds__(InterCfg<L>::THREADS, InterCfg<L>::MINB)
k_c2c_inter(const float2* __restrict__ in, float2* __restrict__ out, long long count, Layout lay,
            const float2* __restrict__ tw)
{
    using C = InterCfg<L>;
    constexpr int N = 1 << L;
    extern __shared__ float2 smem[];
    const Group q = group_of<C>(count);
    const bool live = q.g < q.live;
    const PaddedView view{smem + q.g * C::SLOT};
    float2 v[C::R];
    if constexpr (CIN) {
        rows_in<C, N>(in + q.f0 * lay.in_dist, lay.in_dist, lay.in_stride, q.live, smem);
        __syncthreads();
#pragma unroll
        for (int m = 0; m < C::R; ++m) v[m] = view.ld(q.t + m * C::T);
        __syncthreads();                                   // the slots become exchange areas
    } else {
        const StrideIn src{in + q.f * lay.in_dist, lay.in_stride};
#pragma unroll
        for (int m = 0; m < C::R; ++m) v[m] = live ? src.ld(q.t + m * C::T) : make_float2(0.f, 0.f);
    }
    stockham<L, C::LOG2R, INV, C::WARP>(v, q.t, tw, view);
    if constexpr (COUT) {
        __syncthreads();
#pragma unroll
        for (int m = 0; m < C::R; ++m) view.st(q.t + m * C::T, v[m]);
        __syncthreads();
        rows_out<C, N>(out + q.f0 * lay.out_dist, lay.out_dist, lay.out_stride, q.live, smem);
    } else if (live) {
        const StrideOut dst{out + q.f * lay.out_dist, lay.out_stride};
#pragma unroll
        for (int m = 0; m < C::R; ++m) dst.st(q.t + m * C::T, v[m]);
    }
}

// Real forward, interleaved reals in; bins out through the strided accessor.
template <int LM>
__global__ void __launch_bounds__(InterCfg<LM>::THREADS, InterCfg<LM>::MINB)
k_r2c_inter(const float* __restrict__ in, float2* __restrict__ out, long long count, Layout lay,
            const float2* __restrict__ tw)
{
    using C = InterCfg<LM>;
    constexpr int M = 1 << LM;
    extern __shared__ float2 smem[];
    const Group q = group_of<C>(count);
    const PaddedView view{smem + q.g * C::SLOT};
    reals_in<C, 2 * M>(in + q.f0 * lay.in_dist, lay.in_dist, lay.in_stride, q.live, smem);
    __syncthreads();
    float2 v[C::R];
#pragma unroll
    for (int m = 0; m < C::R; ++m) v[m] = view.ld(q.t + m * C::T);
    __syncthreads();
    stockham<LM, C::LOG2R, false, C::WARP>(v, q.t, tw, view);
#pragma unroll
    for (int m = 0; m < C::R; ++m) view.st(q.t + m * C::T, v[m]);
    xsync<C::WARP>();
    if (q.g < q.live)
        split_store<typename C::S, M>(view, StrideOut{out + q.f * lay.out_dist, lay.out_stride}, q.t, tw + 2 * M);
}

// Real inverse, bins in through the strided accessor; interleaved reals out.
template <int LM>
__global__ void __launch_bounds__(InterCfg<LM>::THREADS, InterCfg<LM>::MINB)
k_c2r_inter(const float2* __restrict__ in, float* __restrict__ out, long long count, Layout lay,
            const float2* __restrict__ tw)
{
    using C = InterCfg<LM>;
    constexpr int M = 1 << LM;
    extern __shared__ float2 smem[];
    const Group q = group_of<C>(count);
    const PaddedView view{smem + q.g * C::SLOT};
    float2 v[C::R];
    c2r_load<LM>(StrideIn{in + q.f * lay.in_dist, lay.in_stride}, q.g < q.live, q.t, tw, v);
    stockham<LM, C::LOG2R, true, C::WARP>(v, q.t, tw, view);
    __syncthreads();
#pragma unroll
    for (int m = 0; m < C::R; ++m) view.st(q.t + m * C::T, v[m]);
    __syncthreads();
    reals_out<C, 2 * M>(out + q.f0 * lay.out_dist, lay.out_dist, lay.out_stride, q.live, smem);
}

// ---------------------------------------------------------------- launch

template <class C>
static unsigned inter_grid(long long count)
{
    return (unsigned)((count + C::G - 1) / C::G);
}

template <int L, bool INV>
static cudaError_t launch_c2c_inter_L(const void* in, void* out, long long count, const Layout& lay, bool cin,
                                      bool cout, const float2* tw, cudaStream_t s)
{
    using C = InterCfg<L>;
    const float2* i = (const float2*)in;
    float2* o = (float2*)out;
    if (cin && cout) k_c2c_inter<L, INV, true, true><<<inter_grid<C>(count), C::THREADS, C::SMEM, s>>>(i, o, count, lay, tw);
    else if (cin) k_c2c_inter<L, INV, true, false><<<inter_grid<C>(count), C::THREADS, C::SMEM, s>>>(i, o, count, lay, tw);
    else k_c2c_inter<L, INV, false, true><<<inter_grid<C>(count), C::THREADS, C::SMEM, s>>>(i, o, count, lay, tw);
    return cudaGetLastError();
}

template <int LM>
static cudaError_t launch_real_inter_L(bool inv, const void* in, void* out, long long count, const Layout& lay,
                                       const float2* tw, cudaStream_t s)
{
    using C = InterCfg<LM>;
    if (inv) k_c2r_inter<LM><<<inter_grid<C>(count), C::THREADS, C::SMEM, s>>>((const float2*)in, (float*)out, count, lay, tw);
    else k_r2c_inter<LM><<<inter_grid<C>(count), C::THREADS, C::SMEM, s>>>((const float*)in, (float2*)out, count, lay, tw);
    return cudaGetLastError();
}

bool inter_applies(Kind kind, int log2n, bool cin, bool cout)
{
    if (kind == R2C) return cin && log2n >= 7 && log2n <= 14;
    if (kind == C2R) return cout && log2n >= 7 && log2n <= 14;
    return (cin || cout) && log2n >= 6 && log2n <= 13;
}

cudaError_t launch_inter(Kind kind, int log2n, const void* in, void* out, long long count, const Layout& lay,
                         bool cin, bool cout, const float2* tw, cudaStream_t s)
{
    if (!inter_applies(kind, log2n, cin, cout)) return cudaErrorInvalidValue;
    if (count <= 0) return cudaSuccess;
    cudaError_t e = cudaErrorInvalidValue;
    if (kind == C2C_FWD || kind == C2C_INV) {
        const bool inv = kind == C2C_INV;
#define CKG_C2C_IN(L)                                                                              \
    case L:                                                                                        \
        e = inv ? launch_c2c_inter_L<L, true>(in, out, count, lay, cin, cout, tw, s)               \
                : launch_c2c_inter_L<L, false>(in, out, count, lay, cin, cout, tw, s);             \
        break;
        switch (log2n) {
            CKG_C2C_IN(6) CKG_C2C_IN(7) CKG_C2C_IN(8) CKG_C2C_IN(9)
            CKG_C2C_IN(10) CKG_C2C_IN(11) CKG_C2C_IN(12) CKG_C2C_IN(13)
        default: break;
        }
#undef CKG_C2C_IN
    } else {
        const bool inv = kind == C2R;
#define CKG_REAL_IN(LM)                                                                            \
    case LM + 1: e = launch_real_inter_L<LM>(inv, in, out, count, lay, tw, s); break;
        switch (log2n) {
            CKG_REAL_IN(6) CKG_REAL_IN(7) CKG_REAL_IN(8) CKG_REAL_IN(9)
            CKG_REAL_IN(10) CKG_REAL_IN(11) CKG_REAL_IN(12) CKG_REAL_IN(13)
        default: break;
        }
#undef CKG_REAL_IN
    }
    if (e == cudaSuccess) count_launch();
    return e;
}

template <int L>
static cudaError_t attr_inter()
{
    const int smem = (int)InterCfg<L>::SMEM;
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_c2c_inter<L, false, true, true>, a, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_c2c_inter<L, false, true, false>, a, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_c2c_inter<L, false, false, true>, a, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_c2c_inter<L, true, true, true>, a, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_c2c_inter<L, true, true, false>, a, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_c2c_inter<L, true, false, true>, a, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_r2c_inter<L>, a, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_c2r_inter<L>, a, smem);
    return e;
}

cudaError_t prepare_inter()
{
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = attr_inter<9>();
    if (e == cudaSuccess) e = attr_inter<10>();
    if (e == cudaSuccess) e = attr_inter<11>();
    if (e == cudaSuccess) e = attr_inter<12>();
    if (e == cudaSuccess) e = attr_inter<13>();
    return e;
}

}  // namespace ckg
