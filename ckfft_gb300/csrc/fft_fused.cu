// fft_fused.cu -- the steps either side of the real transforms, fused into
// the single-CTA kernels so that they cost no HBM pass of their own:
//   * k_stft: frame f = signal[f * hop + j] * window[j] (zero for j >=
//     frame_len), real forward transform, bins times `scale`;
//   * k_filter_c2r: bins times filter[k] times `scale`, real inverse
//     transform (spectral multiply + inverse of FFT convolution / filtering).
// Products are rounded one operation at a time (no contraction), so they
// equal the same products formed in FP32 before an unfused transform.
// Sizes outside the single-CTA range form the products in a row pass
// (k_window_rows / k_filter_rows) ahead of the contiguous path, and the
// forward scale in k_scale_rows after it.
#include <cstdint>

#include "fft_small.cuh"

namespace ckg {

// Reals of one frame, windowed, zero past `len`, as packed pairs.  VEC:
// whole frames (len == n) whose start and window sit on 8-byte boundaries,
// both read as pairs.
template <bool WIN, bool VEC>
struct WindowIn {
    const float* __restrict__ x;
    const float* __restrict__ w;
    long long len;
    __device__ __forceinline__ float2 ld(long long i) const
    {
        const long long j = 2 * i;
        float a, b;
        if constexpr (VEC) {
            const float2 v = __ldcs(reinterpret_cast<const float2*>(x) + i);
            a = v.x;
            b = v.y;
        } else {
            a = j < len ? __ldg(x + j) : 0.f;
            b = j + 1 < len ? __ldg(x + j + 1) : 0.f;
        }
        if constexpr (WIN && VEC) {
            const float2 u = __ldg(reinterpret_cast<const float2*>(w) + i);
            a = __fmul_rn(a, u.x);
            b = __fmul_rn(b, u.y);
        } else if constexpr (WIN) {
            a = __fmul_rn(a, __ldg(w + j));
            b = __fmul_rn(b, __ldg(w + j + 1));
        }
        return make_float2(a, b);
    }
    __device__ __forceinline__ float2 ldg(long long i) const { return ld(i); }
};

// Contiguous bins times a scale.
struct ScaledOut {
    float2* __restrict__ p;
    float s;
    __device__ __forceinline__ void st(long long i, float2 v) const
    {
        __stcs(p + i, make_float2(__fmul_rn(v.x, s), __fmul_rn(v.y, s)));
    }
};

__device__ __forceinline__ float2 cmul_rn(float2 a, float2 b)
{
    return make_float2(__fsub_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)),
                       __fadd_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}

// Bins of one frame times the filter's bins, times a scale.
template <bool FILT>
struct FilterIn {
    const float2* __restrict__ X;
    const float2* __restrict__ H;
    float s;
    __device__ __forceinline__ float2 ld(long long i) const
    {
        float2 v = __ldg(X + i);
        if constexpr (FILT) v = cmul_rn(v, __ldg(H + i));
        return make_float2(__fmul_rn(v.x, s), __fmul_rn(v.y, s));
    }
    __device__ __forceinline__ float2 ldg(long long i) const { return ld(i); }
};

template <int LM, bool WIN, bool VEC>
__global__ void __launch_bounds__(SmallCfg<LM>::THREADS, SmallCfg<LM>::MINB)
k_stft(const float* __restrict__ signal, long long hop, const float* __restrict__ window, long long frame_len,
       float scale, float2* __restrict__ out, long long count, const float2* __restrict__ tw)
{
    using C = SmallCfg<LM>;
    constexpr int M = 1 << LM;
    extern __shared__ float2 smem[];
    const int g = threadIdx.x / C::T, t = threadIdx.x % C::T;
    const long long f = (long long)blockIdx.x * C::TPB + g;
    const long long fc = f < count ? f : 0;
    frame_r2c_at<LM>(WindowIn<WIN, VEC>{signal + fc * hop, window, frame_len}, ScaledOut{out + fc * (M + 1), scale},
                     f < count, t, PaddedView{smem + g * C::SLOT}, tw);
}

template <int LM, bool FILT>
__global__ void __launch_bounds__(SmallCfg<LM>::THREADS, SmallCfg<LM>::MINB)
k_filter_c2r(const float2* __restrict__ spectra, const float2* __restrict__ filter, float scale,
             float2* __restrict__ out, long long count, const float2* __restrict__ tw)
{
    using C = SmallCfg<LM>;
    constexpr int M = 1 << LM;
    extern __shared__ float2 smem[];
    const int g = threadIdx.x / C::T, t = threadIdx.x % C::T;
    const long long f = (long long)blockIdx.x * C::TPB + g;
    const long long fc = f < count ? f : 0;
    frame_c2r_at<LM>(FilterIn<FILT>{spectra + fc * (M + 1), filter, scale}, RowOut{out + fc * M}, f < count, t,
                     PaddedView{smem + g * C::SLOT}, tw);
}

// Row passes of the generic route.
__global__ void k_window_rows(const float* __restrict__ signal, long long hop, const float* __restrict__ window,
                              long long frame_len, float* __restrict__ rows, long long count, long long n)
{
    const long long total = count * n;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long f = i / n, j = i - f * n;
        float v = j < frame_len ? __ldg(signal + f * hop + j) : 0.f;
        if (window) v = __fmul_rn(v, __ldg(window + j));
        rows[i] = v;
    }
}

__global__ void k_filter_rows(const float2* __restrict__ spectra, const float2* __restrict__ filter, float scale,
                              float2* __restrict__ rows, long long count, long long bins)
{
    const long long total = count * bins;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        float2 v = __ldg(spectra + i);
        if (filter) v = cmul_rn(v, __ldg(filter + i % bins));
        rows[i] = make_float2(__fmul_rn(v.x, scale), __fmul_rn(v.y, scale));
    }
}

__global__ void k_scale_rows(float2* __restrict__ p, long long total, float scale)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const float2 v = p[i];
        p[i] = make_float2(__fmul_rn(v.x, scale), __fmul_rn(v.y, scale));
    }
}

// ---------------------------------------------------------------- launch

template <int LM>
static cudaError_t launch_stft_L(const float* signal, long long hop, const float* window, long long frame_len,
                                 float scale, float2* out, long long count, const float2* tw, cudaStream_t s)
{
    using C = SmallCfg<LM>;
    const unsigned grid = (unsigned)((count + C::TPB - 1) / C::TPB);
    const bool vec = frame_len == (2ll << LM) && hop % 2 == 0 && ((uintptr_t)signal & 7) == 0 &&
                     ((uintptr_t)window & 7) == 0;
#define CKG_STFT(W, V) \
    k_stft<LM, W, V><<<grid, C::THREADS, C::SMEM, s>>>(signal, hop, window, frame_len, scale, out, count, tw)
    if (window) {
        if (vec) CKG_STFT(true, true);
        else CKG_STFT(true, false);
    } else {
        if (vec) CKG_STFT(false, true);
        else CKG_STFT(false, false);
    }
#undef CKG_STFT
    return cudaGetLastError();
}

template <int LM>
static cudaError_t launch_filter_L(const float2* spectra, const float2* filter, float scale, float2* out,
                                   long long count, const float2* tw, cudaStream_t s)
{
    using C = SmallCfg<LM>;
    const unsigned grid = (unsigned)((count + C::TPB - 1) / C::TPB);
    if (filter)
        k_filter_c2r<LM, true><<<grid, C::THREADS, C::SMEM, s>>>(spectra, filter, scale, out, count, tw);
    else
        k_filter_c2r<LM, false><<<grid, C::THREADS, C::SMEM, s>>>(spectra, filter, scale, out, count, tw);
    return cudaGetLastError();
}

bool fused_supported(int log2n) { return log2n >= 3 && log2n <= kSmallMaxLog2Real; }

#define CKG_FUSED_SWITCH(CALL)                                                                     \
    switch (log2n - 1) {                                                                           \
    case 2: e = CALL(2); break;                                                                    \
    case 3: e = CALL(3); break;                                                                    \
    case 4: e = CALL(4); break;                                                                    \
    case 5: e = CALL(5); break;                                                                    \
    case 6: e = CALL(6); break;                                                                    \
    case 7: e = CALL(7); break;                                                                    \
    case 8: e = CALL(8); break;                                                                    \
    case 9: e = CALL(9); break;                                                                    \
    case 10: e = CALL(10); break;                                                                  \
    case 11: e = CALL(11); break;                                                                  \
    case 12: e = CALL(12); break;                                                                  \
    case 13: e = CALL(13); break;                                                                  \
    case 14: e = CALL(14); break;                                                                  \
    default: return cudaErrorInvalidValue;                                                         \
    }

cudaError_t launch_stft(int log2n, const float* signal, long long hop, const float* window, long long frame_len,
                        float scale, void* out, long long count, const float2* tw, cudaStream_t s)
{
    if (count <= 0) return cudaSuccess;
    cudaError_t e;
#define CKG_CALL(LM) launch_stft_L<LM>(signal, hop, window, frame_len, scale, (float2*)out, count, tw, s)
    CKG_FUSED_SWITCH(CKG_CALL)
#undef CKG_CALL
    if (e == cudaSuccess) count_launch();
    return e;
}

cudaError_t launch_filter_inverse(int log2n, const void* spectra, const void* filter, float scale, float* out,
                                  long long count, const float2* tw, cudaStream_t s)
{
    if (count <= 0) return cudaSuccess;
    cudaError_t e;
#define CKG_CALL(LM) \
    launch_filter_L<LM>((const float2*)spectra, (const float2*)filter, scale, (float2*)out, count, tw, s)
    CKG_FUSED_SWITCH(CKG_CALL)
#undef CKG_CALL
    if (e == cudaSuccess) count_launch();
    return e;
}
#undef CKG_FUSED_SWITCH

static unsigned rows_grid(long long total)
{
    const long long want = (total + 255) / 256;
    return (unsigned)(want < 152 * 16 ? (want < 1 ? 1 : want) : 152 * 16);
}

cudaError_t launch_window_rows(const float* signal, long long hop, const float* window, long long frame_len,
                               float* rows, long long count, long long n, cudaStream_t s)
{
    if (count <= 0) return cudaSuccess;
    k_window_rows<<<rows_grid(count * n), 256, 0, s>>>(signal, hop, window, frame_len, rows, count, n);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_filter_rows(const void* spectra, const void* filter, float scale, void* rows, long long count,
                               long long bins, cudaStream_t s)
{
    if (count <= 0) return cudaSuccess;
    k_filter_rows<<<rows_grid(count * bins), 256, 0, s>>>((const float2*)spectra, (const float2*)filter, scale,
                                                          (float2*)rows, count, bins);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_scale_rows(void* p, long long total, float scale, cudaStream_t s)
{
    if (total <= 0) return cudaSuccess;
    k_scale_rows<<<rows_grid(total), 256, 0, s>>>((float2*)p, total, scale);
    count_launch();
    return cudaGetLastError();
}

template <int LM>
static cudaError_t attr_fused()
{
    const int smem = (int)SmallCfg<LM>::SMEM;
    cudaError_t e = cudaFuncSetAttribute(k_stft<LM, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_stft<LM, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_stft<LM, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_stft<LM, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_filter_c2r<LM, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_filter_c2r<LM, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    return e;
}

cudaError_t prepare_fused()
{
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = attr_fused<10>();
    if (e == cudaSuccess) e = attr_fused<11>();
    if (e == cudaSuccess) e = attr_fused<12>();
    if (e == cudaSuccess) e = attr_fused<13>();
    if (e == cudaSuccess) e = attr_fused<14>();
    return e;
}

}  // namespace ckg
