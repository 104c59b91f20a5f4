// fft_large.cu -- multi-pass transforms above the single-CTA size limit.
//
// Replaces the reference's recursion (src/ckfft/fft_default.cpp:168-266) for
// sizes whose data cannot stay on chip.  N = N1 * N2, x[n] viewed as N1 rows
// of N2 columns (n = N2*n1 + n2):
//
//   pass 1 (columns): for each column n2, Y[k1] = DFT_N1 over n1 of x[N2*n1 + n2],
//                     times W_N^(n2*k1), stored at scratch[N2*k1 + n2];
//   pass 2 (rows):    for each row k1, DFT_N2 over n2, X[k1 + N1*k2] stored
//                     transposed through shared memory.
//
// Both passes read and write HBM once, with C adjacent columns (pass 1) or
// rows (pass 2) per CTA so every warp access covers C*8 contiguous bytes.
// Real sizes run the half-length complex transform plus a split (forward) or
// merge (inverse) pass, the algebra of src/ckfft/fft_real_default.cpp.
#include "fft_core.cuh"
#include "kernels.h"

namespace ckg {

// Shape of a sub-transform of 2^LS points inside a pass: R values per thread,
// C sequences per CTA.
template <int LS>
struct PassCfg {
    static constexpr int LOG2R = LS < 4 ? LS : LS <= 10 ? 4 : 5;
    static constexpr int R = 1 << LOG2R;
    static constexpr int T = (1 << LS) / R;
    // at most 512 threads (so up to 128 registers) and ~140 KB of shared memory
    static constexpr int C = 512 / T < 16 ? 512 / T : 16;
    static constexpr int THREADS = C * T;
    // interleaved (pass 1 and pass-2 transpose) and per-row padded (pass 2) layouts
    static constexpr int INTERLEAVED = (1 << LS) * C + ((1 << LS) * C >> 4) + 1;
    static constexpr int BLOCKED = C * padded_len(1 << LS);
    static constexpr size_t SMEM = sizeof(float2) * (size_t)(INTERLEAVED > BLOCKED ? INTERLEAVED : BLOCKED);
};

// Element pos of sequence c in an interleaved tile, padded every 16 slots.
template <int C>
struct TileView {
    float2* base;
    int c;
    __device__ __forceinline__ static int slot(int pos, int c) { const int p = pos * C + c; return p + (p >> 4); }
    __device__ __forceinline__ void st(int pos, float2 x) const { base[slot(pos, c)] = x; }
    __device__ __forceinline__ float2 ld(int pos) const { return base[slot(pos, c)]; }
};

// W_N^p for 0 <= p < N = 2^ln from two short table levels:
// W_N^p = W_{N/2^s}^(p >> s) * W_N^(p mod 2^s), s = ceil(ln/2).
// Sizes on this path are at most 2^28, so p fits in 32 bits.
template <bool INV>
__device__ __forceinline__ float2 big_twiddle(const float2* __restrict__ tw, int ln, int p)
{
    const int s = (ln + 1) >> 1;
    const int hi = p >> s, lo = p & ((1 << s) - 1);
    const float2 a = __ldg(tw + (1 << (ln - s)) + hi);
    const float2 b = __ldg(tw + (1 << ln) + lo);
    const float2 w = cmul(a, b);
    return INV ? conjf2(w) : w;
}

// ------------------------------------------------------------ pass 1

template <int LA, bool INV>
__global__ void __launch_bounds__(PassCfg<LA>::THREADS)
k_cols(const float2* __restrict__ in, float2* __restrict__ out, long long count, int log2n2,
       long long in_dist, long long out_dist, const float2* __restrict__ tw)
{
    using P = PassCfg<LA>;
    extern __shared__ float2 smem[];
    const int c = threadIdx.x % P::C, t = threadIdx.x / P::C;
    const long long n2len = 1ll << log2n2;
    const long long tiles = n2len / P::C;
    const long long f = blockIdx.x / tiles;
    const long long n2 = (blockIdx.x % tiles) * P::C + c;
    const float2* src = in + f * in_dist + n2;
    float2 v[P::R];
#pragma unroll
    for (int m = 0; m < P::R; ++m) v[m] = __ldcs(src + (long long)(t + m * P::T) * n2len);
    TileView<P::C> view{smem, c};
    stockham<LA, P::LOG2R, INV, false>(v, t, tw, view);
    const int ln = LA + log2n2;
    float2* dst = out + f * out_dist + n2 + (long long)t * n2len;
    const long long step = (long long)P::T * n2len;
#pragma unroll
    for (int m = 0; m < P::R; ++m) {
        const int k1 = t + m * P::T;
        __stcs(dst + m * step, cmul(v[m], big_twiddle<INV>(tw, ln, (int)n2 * k1)));
        // keep the compiler from hoisting every twiddle load ahead of the
        // stores (that would need 4 more registers per value)
        if ((m & 3) == 3) asm volatile("" ::: "memory");
    }
}

// ------------------------------------------------------------ pass 2

template <int LB, bool INV>
__global__ void __launch_bounds__(PassCfg<LB>::THREADS)
k_rows(const float2* __restrict__ in, float2* __restrict__ out, long long count, int log2n1,
       long long in_dist, long long out_dist, const float2* __restrict__ tw)
{
    using P = PassCfg<LB>;
    constexpr int N2 = 1 << LB;
    extern __shared__ float2 smem[];
    const int r = threadIdx.x / P::T, t = threadIdx.x % P::T;
    const long long n1len = 1ll << log2n1;
    const long long tiles = n1len / P::C;
    const long long f = blockIdx.x / tiles;
    const long long row0 = (blockIdx.x % tiles) * P::C;
    const float2* src = in + f * in_dist + (row0 + r) * N2 + t;
    float2 v[P::R];
#pragma unroll
    for (int m = 0; m < P::R; ++m) v[m] = __ldcs(src + m * P::T);
    PaddedView view{smem + r * padded_len(N2)};
    stockham<LB, P::LOG2R, INV, (P::T <= 32)>(v, t, tw, view);
    __syncthreads();
    // transpose through shared memory so that stores run along rows k1
#pragma unroll
    for (int m = 0; m < P::R; ++m) smem[TileView<P::C>::slot(t + m * P::T, r)] = v[m];
    __syncthreads();
    const int r2 = threadIdx.x % P::C, t2 = threadIdx.x / P::C;
    float2* dst = out + f * out_dist + row0 + r2;
#pragma unroll
    for (int m = 0; m < P::R; ++m) {
        const int k2 = t2 + m * P::T;
        __stcs(dst + (long long)k2 * n1len, smem[TileView<P::C>::slot(k2, r2)]);
    }
}

// ------------------------------------------------- real split / merge passes

// In-place split of a natural-order half-length spectrum Z (M = 2^lm values,
// with room for M+1) into the real forward output X[0..M].
__global__ void k_split_inplace(float2* __restrict__ z, long long count, int lm, long long dist,
                                const float2* __restrict__ tw)
{
    const long long M = 1ll << lm;
    const long long half = M / 2;
    const long long per = half + 1;                   // pairs (k, M-k) for k = 0..M/2
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= count * per) return;
    const long long f = idx / per, k = idx % per;
    float2* zz = z + f * dist;
    const float2* twn = tw + 2 * M;                   // level n = 2M
    if (k == 0) {
        const float2 z0 = zz[0];
        zz[0] = real_split(z0, z0, __ldg(twn));
        zz[M] = real_split(z0, z0, __ldg(twn + M));
    } else if (k == half) {
        const float2 zk = zz[k];
        zz[k] = real_split(zk, zk, __ldg(twn + k));
    } else {
        const float2 a = zz[k], b = zz[M - k];
        zz[k] = real_split(a, b, __ldg(twn + k));
        zz[M - k] = real_split(b, a, __ldg(twn + (M - k)));
    }
}

// Y[k] = merge(X[k], X[M-k]) for k < M, written as M complex values.
__global__ void k_merge(const float2* __restrict__ x, float2* __restrict__ y, long long count, int lm,
                        long long in_dist, long long out_dist, const float2* __restrict__ tw)
{
    const long long M = 1ll << lm;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= count * M) return;
    const long long f = idx >> lm, k = idx & (M - 1);
    const float2* xx = x + f * in_dist;
    y[f * out_dist + k] = real_merge(__ldcs(xx + k), __ldcs(xx + (M - k)), __ldg(tw + 2 * M + k));
}

// ---------------------------------------------------------------- launch

template <int LA, bool INV>
static cudaError_t launch_cols_L(const float2* in, float2* out, long long count, int log2n2,
                                 long long in_dist, long long out_dist, const float2* tw, cudaStream_t s)
{
    using P = PassCfg<LA>;
    const long long blocks = count * ((1ll << log2n2) / P::C);
    k_cols<LA, INV><<<(unsigned)blocks, P::THREADS, P::SMEM, s>>>(in, out, count, log2n2, in_dist, out_dist, tw);
    return cudaGetLastError();
}

template <int LB, bool INV>
static cudaError_t launch_rows_L(const float2* in, float2* out, long long count, int log2n1,
                                 long long in_dist, long long out_dist, const float2* tw, cudaStream_t s)
{
    using P = PassCfg<LB>;
    const long long blocks = count * ((1ll << log2n1) / P::C);
    k_rows<LB, INV><<<(unsigned)blocks, P::THREADS, P::SMEM, s>>>(in, out, count, log2n1, in_dist, out_dist, tw);
    return cudaGetLastError();
}

#define CKG_SUB_SWITCH(L, FN, ...)                                                                 \
    switch (L) {                                                                                   \
    case 7: return FN<7, INV>(__VA_ARGS__);                                                        \
    case 8: return FN<8, INV>(__VA_ARGS__);                                                        \
    case 9: return FN<9, INV>(__VA_ARGS__);                                                        \
    case 10: return FN<10, INV>(__VA_ARGS__);                                                      \
    case 11: return FN<11, INV>(__VA_ARGS__);                                                      \
    case 12: return FN<12, INV>(__VA_ARGS__);                                                      \
    case 13: return FN<13, INV>(__VA_ARGS__);                                                      \
    case 14: return FN<14, INV>(__VA_ARGS__);                                                      \
    default: return cudaErrorInvalidValue;                                                         \
    }

template <bool INV>
static cudaError_t launch_cols(int la, const float2* in, float2* out, long long count, int log2n2,
                               long long in_dist, long long out_dist, const float2* tw, cudaStream_t s)
{
    CKG_SUB_SWITCH(la, launch_cols_L, in, out, count, log2n2, in_dist, out_dist, tw, s)
}

template <bool INV>
static cudaError_t launch_rows(int lb, const float2* in, float2* out, long long count, int log2n1,
                               long long in_dist, long long out_dist, const float2* tw, cudaStream_t s)
{
    CKG_SUB_SWITCH(lb, launch_rows_L, in, out, count, log2n1, in_dist, out_dist, tw, s)
}

LargePlan large_plan(int log2n)
{
    LargePlan p;
    p.log2n = log2n;
    p.log2n1 = log2n / 2;
    p.log2n2 = log2n - p.log2n1;
    return p;
}

static bool large_supported(int log2n)
{
    const LargePlan p = large_plan(log2n);
    return log2n > kSmallMaxLog2Complex && p.log2n1 >= 7 && p.log2n2 <= 14;
}

size_t large_scratch_bytes(Kind kind, int log2n)
{
    // complex: one N-point intermediate; real: one (N/2)-point intermediate
    const int lc = (kind == R2C || kind == C2R) ? log2n - 1 : log2n;
    return sizeof(float2) << lc;
}

cudaError_t launch_large_c2c(bool inverse, int log2n, const void* in, void* out, long long count,
                             long long in_dist, long long out_dist, const float2* tw,
                             void* scratch, size_t scratch_bytes, cudaStream_t s)
{
    if (!large_supported(log2n)) return cudaErrorInvalidValue;
    if (count <= 0) return cudaSuccess;
    const LargePlan p = large_plan(log2n);
    const long long n = 1ll << log2n;
    const long long group = (long long)(scratch_bytes / (sizeof(float2) * (size_t)n));
    if (group < 1) return cudaErrorInvalidValue;
    const float2* src = (const float2*)in;
    float2* dst = (float2*)out;
    float2* tmp = (float2*)scratch;
    for (long long off = 0; off < count; off += group) {
        const long long cnt = count - off < group ? count - off : group;
        cudaError_t e = inverse
            ? launch_cols<true>(p.log2n1, src + off * in_dist, tmp, cnt, p.log2n2, in_dist, n, tw, s)
            : launch_cols<false>(p.log2n1, src + off * in_dist, tmp, cnt, p.log2n2, in_dist, n, tw, s);
        if (e != cudaSuccess) return e;
        e = inverse
            ? launch_rows<true>(p.log2n2, tmp, dst + off * out_dist, cnt, p.log2n1, n, out_dist, tw, s)
            : launch_rows<false>(p.log2n2, tmp, dst + off * out_dist, cnt, p.log2n1, n, out_dist, tw, s);
        if (e != cudaSuccess) return e;
        count_launch(2);
    }
    return cudaSuccess;
}

cudaError_t launch_large_r2c(int log2n, const void* in, void* out, long long count,
                             long long in_dist, long long out_dist, const float2* tw,
                             void* scratch, size_t scratch_bytes, cudaStream_t s)
{
    // in: n floats per frame (n/2 packed complex), out: n/2+1 complex per frame
    const int lm = log2n - 1;
    const long long M = 1ll << lm;
    cudaError_t e = launch_large_c2c(false, lm, in, out, count, in_dist / 2, out_dist, tw, scratch,
                                     scratch_bytes, s);
    if (e != cudaSuccess) return e;
    const long long work = count * (M / 2 + 1);
    const int threads = 256;
    k_split_inplace<<<(unsigned)((work + threads - 1) / threads), threads, 0, s>>>(
        (float2*)out, count, lm, out_dist, tw);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_large_c2r(int log2n, const void* in, void* out, long long count,
                             long long in_dist, long long out_dist, const float2* tw,
                             void* scratch, size_t scratch_bytes, cudaStream_t s)
{
    // in: n/2+1 complex per frame, out: n floats per frame (n/2 packed complex)
    const int lm = log2n - 1;
    const long long M = 1ll << lm;
    const long long work = count * M;
    const int threads = 256;
    k_merge<<<(unsigned)((work + threads - 1) / threads), threads, 0, s>>>(
        (const float2*)in, (float2*)out, count, lm, in_dist, out_dist / 2, tw);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // inverse complex transform of the merged values, in place through scratch
    return launch_large_c2c(true, lm, out, out, count, out_dist / 2, out_dist / 2, tw, scratch,
                            scratch_bytes, s);
}

template <int L>
static cudaError_t attr_pass()
{
    using P = PassCfg<L>;
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_cols<L, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P::SMEM)) != cudaSuccess) return e;
    if ((e = cudaFuncSetAttribute(k_cols<L, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P::SMEM)) != cudaSuccess) return e;
    if ((e = cudaFuncSetAttribute(k_rows<L, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P::SMEM)) != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_rows<L, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P::SMEM);
}

cudaError_t prepare_large()
{
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = attr_pass<7>();
    if (e == cudaSuccess) e = attr_pass<8>();
    if (e == cudaSuccess) e = attr_pass<9>();
    if (e == cudaSuccess) e = attr_pass<10>();
    if (e == cudaSuccess) e = attr_pass<11>();
    if (e == cudaSuccess) e = attr_pass<12>();
    if (e == cudaSuccess) e = attr_pass<13>();
    if (e == cudaSuccess) e = attr_pass<14>();
    return e;
}

}  // namespace ckg
