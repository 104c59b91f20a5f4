// fft_strided.cu -- advanced-layout batches: element p of transform f at
// in[f * in_dist + p * in_stride], written to out[f * out_dist + p * out_stride]
// (units: elements of the pointer's type, complex or float).
//
// Single-CTA sizes run the batched frame bodies of fft_small.cuh with strided
// accessors, so a strided batch moves every byte once, like a contiguous one:
// interleaved channels (stride = channels, distance 1), columns of a
// row-major matrix, frames at an odd hop.  Other sizes are gathered into
// contiguous rows, transformed by the contiguous path and scattered back
// (k_gather / k_scatter below).
#include "fft_small.cuh"

namespace ckg {

template <int L, bool INV>
__global__ void __launch_bounds__(SmallCfg<L>::THREADS, SmallCfg<L>::MINB)
k_c2c_strided(const float2* __restrict__ in, float2* __restrict__ out, long long count, Layout lay,
              const float2* __restrict__ tw)
{
    using C = SmallCfg<L>;
    extern __shared__ float2 smem[];
    const int g = threadIdx.x / C::T, t = threadIdx.x % C::T;
    const long long f = (long long)blockIdx.x * C::TPB + g;
    const long long fc = f < count ? f : 0;            // idle groups keep an in-range base
    frame_c2c_at<L, INV>(StrideIn{in + fc * lay.in_dist, lay.in_stride},
                         StrideOut{out + fc * lay.out_dist, lay.out_stride}, f < count, t,
                         PaddedView{smem + g * C::SLOT}, tw);
}

template <int LM>
__global__ void __launch_bounds__(SmallCfg<LM>::THREADS, SmallCfg<LM>::MINB)
k_r2c_strided(const float* __restrict__ in, float2* __restrict__ out, long long count, Layout lay,
              const float2* __restrict__ tw)
{
    using C = SmallCfg<LM>;
    extern __shared__ float2 smem[];
    const int g = threadIdx.x / C::T, t = threadIdx.x % C::T;
    const long long f = (long long)blockIdx.x * C::TPB + g;
    const long long fc = f < count ? f : 0;
    frame_r2c_at<LM>(PairIn{in + fc * lay.in_dist, lay.in_stride},
                     StrideOut{out + fc * lay.out_dist, lay.out_stride}, f < count, t,
                     PaddedView{smem + g * C::SLOT}, tw);
}

template <int LM>
__global__ void __launch_bounds__(SmallCfg<LM>::THREADS, SmallCfg<LM>::MINB)
k_c2r_strided(const float2* __restrict__ in, float* __restrict__ out, long long count, Layout lay,
              const float2* __restrict__ tw)
{
    using C = SmallCfg<LM>;
    extern __shared__ float2 smem[];
    const int g = threadIdx.x / C::T, t = threadIdx.x % C::T;
    const long long f = (long long)blockIdx.x * C::TPB + g;
    const long long fc = f < count ? f : 0;
    frame_c2r_at<LM>(StrideIn{in + fc * lay.in_dist, lay.in_stride},
                     PairOut{out + fc * lay.out_dist, lay.out_stride}, f < count, t,
                     PaddedView{smem + g * C::SLOT}, tw);
}

// Row f of `count` contiguous rows of `len` elements <-> the strided layout.
template <class E>
__global__ void k_gather(const E* __restrict__ src, long long stride, long long dist, E* __restrict__ dst,
                         long long count, long long len)
{
    const long long total = count * len;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long f = i / len, p = i - f * len;
        dst[i] = src[f * dist + p * stride];
    }
}

template <class E>
__global__ void k_scatter(const E* __restrict__ src, E* __restrict__ dst, long long stride, long long dist,
                          long long count, long long len)
{
    const long long total = count * len;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long f = i / len, p = i - f * len;
        dst[f * dist + p * stride] = src[i];
    }
}

// dst[c dp + r] = src[r sp + c] for r < rows, c < cols: 32 x 32 tiles through
// shared memory, so both sides move runs of 32 consecutive elements (128 or
// 256 bytes), and neighbouring CTAs take neighbouring tiles of the same rows.
// SS / SD: evict-first loads / stores for the side read or written once.
template <class E, bool SS, bool SD>
__global__ void __launch_bounds__(256) k_transpose(const E* __restrict__ src, long long sp, E* __restrict__ dst,
                                                   long long dp, long long rows, long long cols)
{
    __shared__ E tile[32][33];
    const long long tiles_c = (cols + 31) / 32, tiles = tiles_c * ((rows + 31) / 32);
    const int x = threadIdx.x & 31, y = threadIdx.x >> 5;
    pdl_start();
    for (long long b = blockIdx.x; b < tiles; b += gridDim.x) {
        const long long r0 = (b / tiles_c) * 32, c0 = (b % tiles_c) * 32;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const long long r = r0 + y + 8 * k, c = c0 + x;
            if (r < rows && c < cols) {
                const E* q = src + r * sp + c;
                tile[y + 8 * k][x] = SS ? __ldcs(q) : *q;
            }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const long long c = c0 + y + 8 * k, r = r0 + x;
            if (r < rows && c < cols) {
                E* q = dst + c * dp + r;
                if constexpr (SD) __stcs(q, tile[x][y + 8 * k]);
                else *q = tile[x][y + 8 * k];
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- launch

template <class C>
static unsigned strided_grid(long long count)
{
    return (unsigned)((count + C::TPB - 1) / C::TPB);
}

template <int L, bool INV>
static cudaError_t launch_c2c_st(const void* in, void* out, long long count, const Layout& lay,
                                 const float2* tw, cudaStream_t s)
{
    using C = SmallCfg<L>;
    k_c2c_strided<L, INV><<<strided_grid<C>(count), C::THREADS, C::SMEM, s>>>(
        (const float2*)in, (float2*)out, count, lay, tw);
    return cudaGetLastError();
}

template <int LM>
static cudaError_t launch_r2c_st(const void* in, void* out, long long count, const Layout& lay,
                                 const float2* tw, cudaStream_t s)
{
    using C = SmallCfg<LM>;
    k_r2c_strided<LM><<<strided_grid<C>(count), C::THREADS, C::SMEM, s>>>(
        (const float*)in, (float2*)out, count, lay, tw);
    return cudaGetLastError();
}

template <int LM>
static cudaError_t launch_c2r_st(const void* in, void* out, long long count, const Layout& lay,
                                 const float2* tw, cudaStream_t s)
{
    using C = SmallCfg<LM>;
    k_c2r_strided<LM><<<strided_grid<C>(count), C::THREADS, C::SMEM, s>>>(
        (const float2*)in, (float*)out, count, lay, tw);
    return cudaGetLastError();
}

bool strided_supported(Kind kind, int log2n)
{
    if (kind == R2C || kind == C2R) return log2n >= 3 && log2n <= kSmallMaxLog2Real;
    return log2n >= 0 && log2n <= kSmallMaxLog2Complex;
}

cudaError_t launch_strided(Kind kind, int log2n, const void* in, void* out, long long count, const Layout& lay,
                           const float2* tw, cudaStream_t s)
{
    if (!strided_supported(kind, log2n)) return cudaErrorInvalidValue;
    if (count <= 0) return cudaSuccess;
    cudaError_t e = cudaErrorInvalidValue;
#define CKG_C2C_ST(L)                                                                              \
    case L:                                                                                        \
        e = kind == C2C_INV ? launch_c2c_st<L, true>(in, out, count, lay, tw, s)                   \
                            : launch_c2c_st<L, false>(in, out, count, lay, tw, s);                 \
        break;
#define CKG_REAL_ST(LM)                                                                            \
    case LM + 1:                                                                                   \
        e = kind == C2R ? launch_c2r_st<LM>(in, out, count, lay, tw, s)                            \
                        : launch_r2c_st<LM>(in, out, count, lay, tw, s);                           \
        break;
    if (kind == C2C_FWD || kind == C2C_INV) {
        switch (log2n) {
            CKG_C2C_ST(0) CKG_C2C_ST(1) CKG_C2C_ST(2) CKG_C2C_ST(3) CKG_C2C_ST(4)
            CKG_C2C_ST(5) CKG_C2C_ST(6) CKG_C2C_ST(7) CKG_C2C_ST(8) CKG_C2C_ST(9)
            CKG_C2C_ST(10) CKG_C2C_ST(11) CKG_C2C_ST(12) CKG_C2C_ST(13) CKG_C2C_ST(14)
        default: break;
        }
    } else {
        switch (log2n) {
            CKG_REAL_ST(2) CKG_REAL_ST(3) CKG_REAL_ST(4) CKG_REAL_ST(5) CKG_REAL_ST(6)
            CKG_REAL_ST(7) CKG_REAL_ST(8) CKG_REAL_ST(9) CKG_REAL_ST(10) CKG_REAL_ST(11)
            CKG_REAL_ST(12) CKG_REAL_ST(13) CKG_REAL_ST(14)
        default: break;
        }
    }
#undef CKG_C2C_ST
#undef CKG_REAL_ST
    if (e == cudaSuccess) count_launch();
    return e;
}

static unsigned copy_grid(long long total)
{
    const long long want = (total + 255) / 256;
    return (unsigned)(want < 152 * 16 ? (want < 1 ? 1 : want) : 152 * 16);
}

cudaError_t launch_gather(const void* src, long long stride, long long dist, void* dst, long long count,
                          long long len, int esize, cudaStream_t s)
{
    if (count <= 0 || len <= 0) return cudaSuccess;
    const unsigned grid = copy_grid(count * len);
    if (esize == 8) k_gather<float2><<<grid, 256, 0, s>>>((const float2*)src, stride, dist, (float2*)dst, count, len);
    else if (esize == 4) k_gather<float><<<grid, 256, 0, s>>>((const float*)src, stride, dist, (float*)dst, count, len);
    else return cudaErrorInvalidValue;
    count_launch();
    return cudaGetLastError();
}

template <class E>
static cudaError_t launch_transpose_e(const void* src, long long sp, void* dst, long long dp, long long rows,
                                      long long cols, bool stream_src, bool stream_dst, cudaStream_t s)
{
    const long long tiles = ((rows + 31) / 32) * ((cols + 31) / 32);
    const unsigned grid = (unsigned)(tiles < 152 * 8 ? tiles : 152 * 8);
    const E* a = (const E*)src;
    E* b = (E*)dst;
    if (stream_src && stream_dst) return launch_pdl(k_transpose<E, true, true>, dim3(grid), dim3(256), 0, s, a, sp, b, dp, rows, cols);
    if (stream_src) return launch_pdl(k_transpose<E, true, false>, dim3(grid), dim3(256), 0, s, a, sp, b, dp, rows, cols);
    if (stream_dst) return launch_pdl(k_transpose<E, false, true>, dim3(grid), dim3(256), 0, s, a, sp, b, dp, rows, cols);
    return launch_pdl(k_transpose<E, false, false>, dim3(grid), dim3(256), 0, s, a, sp, b, dp, rows, cols);
}

cudaError_t launch_transpose(const void* src, long long sp, void* dst, long long dp, long long rows, long long cols,
                             int esize, bool stream_src, bool stream_dst, cudaStream_t s)
{
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    cudaError_t e;
    if (esize == 8) e = launch_transpose_e<float2>(src, sp, dst, dp, rows, cols, stream_src, stream_dst, s);
    else if (esize == 4) e = launch_transpose_e<float>(src, sp, dst, dp, rows, cols, stream_src, stream_dst, s);
    else return cudaErrorInvalidValue;
    if (e == cudaSuccess) count_launch();
    return e;
}

cudaError_t launch_scatter(const void* src, void* dst, long long stride, long long dist, long long count,
                           long long len, int esize, cudaStream_t s)
{
    if (count <= 0 || len <= 0) return cudaSuccess;
    const unsigned grid = copy_grid(count * len);
    if (esize == 8) k_scatter<float2><<<grid, 256, 0, s>>>((const float2*)src, (float2*)dst, stride, dist, count, len);
    else if (esize == 4) k_scatter<float><<<grid, 256, 0, s>>>((const float*)src, (float*)dst, stride, dist, count, len);
    else return cudaErrorInvalidValue;
    count_launch();
    return cudaGetLastError();
}

template <int L>
static cudaError_t attr_st_c2c()
{
    cudaError_t e = cudaFuncSetAttribute(k_c2c_strided<L, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)SmallCfg<L>::SMEM);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_c2c_strided<L, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)SmallCfg<L>::SMEM);
}

template <int LM>
static cudaError_t attr_st_real()
{
    cudaError_t e = cudaFuncSetAttribute(k_r2c_strided<LM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)SmallCfg<LM>::SMEM);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_c2r_strided<LM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)SmallCfg<LM>::SMEM);
}

cudaError_t prepare_strided()
{
    cudaError_t e = cudaSuccess;
    // sizes whose shared memory may exceed the 48 KB default
    if (e == cudaSuccess) e = attr_st_c2c<10>();
    if (e == cudaSuccess) e = attr_st_c2c<11>();
    if (e == cudaSuccess) e = attr_st_c2c<12>();
    if (e == cudaSuccess) e = attr_st_c2c<13>();
    if (e == cudaSuccess) e = attr_st_c2c<14>();
    if (e == cudaSuccess) e = attr_st_real<10>();
    if (e == cudaSuccess) e = attr_st_real<11>();
    if (e == cudaSuccess) e = attr_st_real<12>();
    if (e == cudaSuccess) e = attr_st_real<13>();
    if (e == cudaSuccess) e = attr_st_real<14>();
    return e;
}

}  // namespace ckg
