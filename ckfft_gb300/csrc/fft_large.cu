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
// Real sizes run the half-length complex transform with the split (forward)
// fused into its last pass and the merge (inverse) into its first, the
// algebra of src/ckfft/fft_real_default.cpp; a separate split / merge kernel
// remains for scratch arrays that are not 128-byte aligned.
#include <cstdint>

#include "fft_passes.cuh"
#include "jobs.h"
#include "kernels.h"

namespace ckg {

// ------------------------------------------------------------ pass kernels

// Thread budget of the batched pass kernels: 1024 for sub-lengths above 2^10
// (16 values per thread, 64 registers), 512 below.
template <int LS>
struct BatchMaxT {
    static constexpr int value = LS > 10 ? 1024 : 512;
};
// Widest tile of the batched passes: 16 sequences (128-byte row accesses).
// 32 (256-byte rows) up to sub-length 2^8 measured slower on GB300: batched
// 2^17 2604 vs 2740 GB/s, 2^24 1723 vs 1942 (twice the shared memory per
// CTA, half the CTAs per SM).
template <int LS>
struct BatchCMax {
    static constexpr int value = 16;
};
template <int LS>
using BPass = PassCfg<LS, BatchMaxT<LS>::value, BatchCMax<LS>::value>;
// Resident CTAs asked of the compiler for the column kernels: at most 64
// registers a thread, so that at sub-lengths 2^9 / 2^10 (512 threads) two
// CTAs share an SM and one's loads overlap the other's butterflies.
template <int LS>
struct ColsMinBlocks {
    static constexpr int value = 65536 / (BPass<LS>::THREADS * 64);
};

template <int LA, bool INV>
__global__ void __launch_bounds__(BPass<LA>::THREADS, ColsMinBlocks<LA>::value)
k_cols(const float2* __restrict__ in, float2* __restrict__ out, long long count, int log2n2,
       long long in_dist, long long out_dist, const float2* __restrict__ tw)
{
    using P = BPass<LA>;
    extern __shared__ float2 smem[];
    pdl_start();
    const long long tiles = (1ll << log2n2) / P::C;
    const long long f = blockIdx.x / tiles;
    pass_cols<LA, INV, false, BatchMaxT<LA>::value, BatchCMax<LA>::value>(in + f * in_dist, out + f * out_dist, log2n2,
                                                                          blockIdx.x % tiles, threadIdx.x, smem, tw);
}

template <int LB, bool INV>
__global__ void __launch_bounds__(BPass<LB>::THREADS)
k_rows(const float2* __restrict__ in, float2* __restrict__ out, long long count, int log2n1,
       long long in_dist, long long out_dist, const float2* __restrict__ tw)
{
    using P = BPass<LB>;
    extern __shared__ float2 smem[];
    pdl_start();
    const long long tiles = (1ll << log2n1) / P::C;
    const long long f = blockIdx.x / tiles;
    pass_rows_xt<LB, INV, false, BatchMaxT<LB>::value, true, BatchCMax<LB>::value>(
        in + f * in_dist, out + f * out_dist, log2n1, blockIdx.x % tiles, threadIdx.x, smem, tw);
}

// Third pass of the three-pass transform (N = N1 N2 N3, sub-lengths 2^l1,
// 2^l2, 2^LB): block (f, k2, tile) runs DFT_N3 along the C rows k1 of the
// tile, row (k1, k2) of transform f at in[f N + k1 N2 N3 + k2 N3 ..], and
// stores X[k1 + N1 k2 + N1 N2 k3] -- C consecutive outputs per k3.
template <int LB, bool INV>
__global__ void __launch_bounds__(BPass<LB>::THREADS)
k_rows3(const float2* __restrict__ in, float2* __restrict__ out, int l1, int l2, long long out_dist,
        const float2* __restrict__ tw)
{
    using P = BPass<LB>;
    extern __shared__ float2 smem[];
    pdl_start();
    const long long tiles = (1ll << l1) / P::C;
    const long long b = blockIdx.x;
    const long long tile = b % tiles;
    const long long k2 = (b / tiles) & ((1ll << l2) - 1);
    const long long f = b / (tiles << l2);
    const long long n = 1ll << (l1 + l2 + LB);
    pass_rows_xt<LB, INV, false, BatchMaxT<LB>::value, true, BatchCMax<LB>::value>(
        in + f * n + (k2 << LB), out + f * out_dist + (k2 << l1), l1 + l2, tile, threadIdx.x, smem, tw, l2 + LB);
}

// Row pass of a real forward transform with the split fused: block
// (f, tile) writes the M+1 output bins of its row pairs (pass_rows_split).
template <int LB>
__global__ void __launch_bounds__(BPass<LB>::THREADS)
k_rows_split(const float2* __restrict__ in, float2* __restrict__ out, int log2n1, int log2k1, long long in_dist,
             long long out_dist, const float2* __restrict__ tw)
{
    using P = BPass<LB>;
    extern __shared__ float2 smem[];
    pdl_start();
    const long long tiles = (1ll << log2n1) / P::C;
    const long long f = blockIdx.x / tiles;
    pass_rows_split<LB, BatchMaxT<LB>::value>(in + f * in_dist, out + f * out_dist, log2n1, blockIdx.x % tiles,
                                              threadIdx.x, smem, tw, log2k1);
}

// Column pass of a real inverse transform with the merge fused: block
// (f, tile) reads the M+1 bins of its column pairs (pass_cols_merge).
template <int LA>
__global__ void __launch_bounds__(BPass<LA>::THREADS, ColsMinBlocks<LA>::value)
k_cols_merge(const float2* __restrict__ in, float2* __restrict__ out, int log2n2, long long in_dist,
             long long out_dist, const float2* __restrict__ tw)
{
    using P = BPass<LA>;
    extern __shared__ float2 smem[];
    pdl_start();
    const long long tiles = (1ll << log2n2) / P::C;
    const long long f = blockIdx.x / tiles;
    pass_cols_merge<LA, BatchMaxT<LA>::value, BatchCMax<LA>::value>(in + f * in_dist, out + f * out_dist, log2n2,
                                                                    blockIdx.x % tiles, threadIdx.x, smem, tw);
}

// --------------------------- real split / merge as passes of their own
// (used only when the scratch array is not 128-byte aligned)

// In-place split of a natural-order half-length spectrum Z (M = 2^lm values,
// with room for M+1) into the real forward output X[0..M].
__global__ void k_split_inplace(float2* __restrict__ z, long long count, int lm, long long dist,
                                const float2* __restrict__ tw)
{
    pdl_start();
    const long long M = 1ll << lm;
    const long long per = M / 2 + 1;                 // pairs (k, M-k) for k = 0..M/2
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= count * per) return;
    const long long f = idx / per, k = idx % per;
    split_pair_inplace<false>(z + f * dist, M, k, tw + 2 * M);
}

// Y[k] = merge(X[k], X[M-k]) for k < M, written as M complex values.
__global__ void k_merge(const float2* __restrict__ x, float2* __restrict__ y, long long count, int lm,
                        long long in_dist, long long out_dist, const float2* __restrict__ tw)
{
    pdl_start();
    const long long M = 1ll << lm;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= count * M) return;
    const long long f = idx >> lm, k = idx & (M - 1);
    merge_elem<false>(x + f * in_dist, y + f * out_dist, M, k, tw + 2 * M);
}

// ---------------------------------------------------------------- launch

template <int LA, bool INV>
static cudaError_t launch_cols_L(const float2* in, float2* out, long long count, int log2n2,
                                 long long in_dist, long long out_dist, const float2* tw, cudaStream_t s)
{
    using P = BPass<LA>;
    const long long blocks = count * ((1ll << log2n2) / P::C);
    return launch_pdl(k_cols<LA, INV>, dim3((unsigned)blocks), dim3(P::THREADS), P::SMEM, s, in, out, count, log2n2,
                      in_dist, out_dist, tw);
}

template <int LB, bool INV>
static cudaError_t launch_rows_L(const float2* in, float2* out, long long count, int log2n1,
                                 long long in_dist, long long out_dist, const float2* tw, cudaStream_t s)
{
    using P = BPass<LB>;
    const long long blocks = count * ((1ll << log2n1) / P::C);
    return launch_pdl(k_rows<LB, INV>, dim3((unsigned)blocks), dim3(P::THREADS), P::SMEM, s, in, out, count, log2n1,
                      in_dist, out_dist, tw);
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

template <int LB, bool INV>
static cudaError_t launch_rows3_L(const float2* in, float2* out, long long count, int l1, int l2, long long out_dist,
                                  const float2* tw, cudaStream_t s)
{
    using P = BPass<LB>;
    const long long blocks = count * ((1ll << l1) / P::C) << l2;
    return launch_pdl(k_rows3<LB, INV>, dim3((unsigned)blocks), dim3(P::THREADS), P::SMEM, s, in, out, l1, l2, out_dist,
                      tw);
}

template <bool INV>
static cudaError_t launch_rows3(int l3, const float2* in, float2* out, long long count, int l1, int l2,
                                long long out_dist, const float2* tw, cudaStream_t s)
{
    switch (l3) {
    case 7: return launch_rows3_L<7, INV>(in, out, count, l1, l2, out_dist, tw, s);
    case 8: return launch_rows3_L<8, INV>(in, out, count, l1, l2, out_dist, tw, s);
    case 9: return launch_rows3_L<9, INV>(in, out, count, l1, l2, out_dist, tw, s);
    case 10: return launch_rows3_L<10, INV>(in, out, count, l1, l2, out_dist, tw, s);
    default: return cudaErrorInvalidValue;
    }
}

// Three sub-lengths of at most 2^10 (each >= 2^7), as equal as possible.
static bool plan3(int log2n, int* l1, int* l2, int* l3)
{
    if (log2n < 21 || log2n > 30) return false;
    *l3 = (log2n + 2) / 3;
    *l2 = (log2n - *l3 + 1) / 2;
    *l1 = log2n - *l3 - *l2;
    return *l1 >= 7 && *l3 <= 10 && *l2 <= 10;
}

// Sizes from 2^kThreePassMinLog2 on run as three passes whose tiles are all
// 16 columns / rows wide (128-byte accesses); two passes there would need
// sub-lengths above 2^10, whose tiles are 4 or 8 wide.
constexpr int kThreePassMinLog2 = 21;

static cudaError_t launch_rows_split(int lb, const float2* in, float2* out, long long count, int log2n1, int log2k1,
                                     long long in_dist, long long out_dist, const float2* tw, cudaStream_t s);
static cudaError_t launch_cols_merge(int la, const float2* in, float2* out, long long count, int log2n2,
                                     long long in_dist, long long out_dist, const float2* tw, cudaStream_t s);

// kind C2C_FWD / C2C_INV: complex transforms of 2^log2n points.  R2C: real
// forward of 2^(log2n+1) reals read as 2^log2n packed pairs, the split fused
// into the third pass (2^log2n + 1 bins out).  C2R: real inverse from
// 2^log2n + 1 bins, the merge fused into the first pass.  Distances in float2.
static cudaError_t launch_three_pass(Kind kind, int log2n, const float2* in, float2* out, long long count,
                                     long long in_dist, long long out_dist, const float2* tw, float2* tmp,
                                     long long group, cudaStream_t s)
{
    int l1, l2, l3;
    if (!plan3(log2n, &l1, &l2, &l3)) return cudaErrorInvalidValue;
    const bool inverse = kind == C2C_INV || kind == C2R;
    const long long n = 1ll << log2n, M = 1ll << (l2 + l3);
    for (long long off = 0; off < count; off += group) {
        const long long cnt = count - off < group ? count - off : group;
        const float2* src = in + off * in_dist;
        float2* dst = out + off * out_dist;
        // pass 1: columns of length N1 over the M = N2 N3 columns -> tmp
        cudaError_t e = kind == C2R       ? launch_cols_merge(l1, src, tmp, cnt, l2 + l3, in_dist, n, tw, s)
                        : inverse         ? launch_cols<true>(l1, src, tmp, cnt, l2 + l3, in_dist, n, tw, s)
                                          : launch_cols<false>(l1, src, tmp, cnt, l2 + l3, in_dist, n, tw, s);
        // pass 2: in every row k1, columns of length N2 over the N3 columns, in place
        if (e == cudaSuccess)
            e = inverse ? launch_cols<true>(l2, tmp, tmp, cnt << l1, l3, M, M, tw, s)
                        : launch_cols<false>(l2, tmp, tmp, cnt << l1, l3, M, M, tw, s);
        // pass 3: rows of length N3, C consecutive k1 per tile -> out (real
        // forward: row pairs k, N1 N2 - k with the split)
        if (e == cudaSuccess)
            e = kind == R2C ? launch_rows_split(l3, tmp, dst, cnt, l1 + l2, l1, n, out_dist, tw, s)
                : inverse   ? launch_rows3<true>(l3, tmp, dst, cnt, l1, l2, out_dist, tw, s)
                            : launch_rows3<false>(l3, tmp, dst, cnt, l1, l2, out_dist, tw, s);
        if (e != cudaSuccess) return e;
        count_launch(3);
    }
    return cudaSuccess;
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
    // 2^15, 2^16: both passes inside one persistent CTA per transform
    // (fft_mid.cu), or inside one cluster per transform (fft_l2pass.cu); the
    // intermediate kept in L2 either way
    if (mid_supported(log2n) && mid_enabled(log2n) && ((uintptr_t)scratch & 127) == 0 && ((uintptr_t)in & 15) == 0 &&
        (in_dist & 1) == 0 && scratch_bytes >= mid_scratch_bytes(log2n, count))
        return launch_mid(inverse ? 1 : 0, log2n, in, out, count, in_dist, out_dist, tw, scratch, scratch_bytes, s);
    if (l2pass_supported(log2n) && ((uintptr_t)scratch & 127) == 0)
        return launch_l2pass(inverse ? 1 : 0, log2n, in, out, count, in_dist, out_dist, tw, scratch, scratch_bytes, s);
    const LargePlan p = large_plan(log2n);
    const long long n = 1ll << log2n;
    const long long group = (long long)(scratch_bytes / (sizeof(float2) * (size_t)n));
    if (group < 1) return cudaErrorInvalidValue;
    const float2* src = (const float2*)in;
    float2* dst = (float2*)out;
    float2* tmp = (float2*)scratch;
    if (log2n >= kThreePassMinLog2 && ((uintptr_t)scratch & 127) == 0)
        return launch_three_pass(inverse ? C2C_INV : C2C_FWD, log2n, src, dst, count, in_dist, out_dist, tw, tmp,
                                 group, s);
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

template <int LB>
static cudaError_t launch_rows_split_L(const float2* in, float2* out, long long count, int log2n1, int log2k1,
                                       long long in_dist, long long out_dist, const float2* tw, cudaStream_t s)
{
    using P = BPass<LB>;
    const long long blocks = count * ((1ll << log2n1) / P::C);
    return launch_pdl(k_rows_split<LB>, dim3((unsigned)blocks), dim3(P::THREADS), P::SMEM, s, in, out, log2n1,
                      log2k1, in_dist, out_dist, tw);
}

// Row pass with the real split fused, row sub-length 2^lb (7 .. 10).
static cudaError_t launch_rows_split(int lb, const float2* in, float2* out, long long count, int log2n1, int log2k1,
                                     long long in_dist, long long out_dist, const float2* tw, cudaStream_t s)
{
    switch (lb) {
    case 7: return launch_rows_split_L<7>(in, out, count, log2n1, log2k1, in_dist, out_dist, tw, s);
    case 8: return launch_rows_split_L<8>(in, out, count, log2n1, log2k1, in_dist, out_dist, tw, s);
    case 9: return launch_rows_split_L<9>(in, out, count, log2n1, log2k1, in_dist, out_dist, tw, s);
    case 10: return launch_rows_split_L<10>(in, out, count, log2n1, log2k1, in_dist, out_dist, tw, s);
    default: return cudaErrorInvalidValue;
    }
}

// Two-pass real forward with the split fused into the row pass, for half
// lengths whose row sub-length is 2^8 .. 2^10 below the three-pass sizes.
static bool rows_split_supported(int lm)
{
    const LargePlan p = large_plan(lm);
    return lm > kSmallMaxLog2Complex && lm < kThreePassMinLog2 && p.log2n1 >= 7 && p.log2n2 >= 8 && p.log2n2 <= 10;
}

static cudaError_t launch_r2c_rows_split(int lm, const float2* in, float2* out, long long count, long long in_dist,
                                         long long out_dist, const float2* tw, float2* tmp, size_t scratch_bytes,
                                         cudaStream_t s)
{
    const LargePlan p = large_plan(lm);
    const long long M = 1ll << lm;
    const long long group = (long long)(scratch_bytes / (sizeof(float2) * (size_t)M));
    if (group < 1) return cudaErrorInvalidValue;
    for (long long off = 0; off < count; off += group) {
        const long long cnt = count - off < group ? count - off : group;
        cudaError_t e = launch_cols<false>(p.log2n1, in + off * in_dist, tmp, cnt, p.log2n2, in_dist, M, tw, s);
        if (e == cudaSuccess)
            e = launch_rows_split(p.log2n2, tmp, out + off * out_dist, cnt, p.log2n1, p.log2n1, M, out_dist, tw, s);
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
    // (half lengths 2^15 / 2^16: the cluster kernel with the split fused into
    // its row tiles, 2749 / 2621 GB/s batched at n = 2^16 / 2^17 against 2507
    // / 2609 for the fused two-pass form through HBM)
    const int lm = log2n - 1;
    const long long M = 1ll << lm;
    if (count <= 0) return cudaSuccess;
    if (l2pass_supported(lm) && ((uintptr_t)scratch & 127) == 0)
        return launch_l2pass(2, lm, in, out, count, in_dist / 2, out_dist, tw, scratch, scratch_bytes, s);
    if (rows_split_supported(lm) && ((uintptr_t)scratch & 127) == 0)
        return launch_r2c_rows_split(lm, (const float2*)in, (float2*)out, count, in_dist / 2, out_dist, tw,
                                     (float2*)scratch, scratch_bytes, s);
    int l1, l2, l3;
    if (lm >= kThreePassMinLog2 && plan3(lm, &l1, &l2, &l3) && ((uintptr_t)scratch & 127) == 0) {
        const long long group = (long long)(scratch_bytes / (sizeof(float2) * (size_t)M));
        if (group < 1) return cudaErrorInvalidValue;
        return launch_three_pass(R2C, lm, (const float2*)in, (float2*)out, count, in_dist / 2, out_dist, tw,
                                 (float2*)scratch, group, s);
    }
    cudaError_t e = launch_large_c2c(false, lm, in, out, count, in_dist / 2, out_dist, tw, scratch,
                                     scratch_bytes, s);
    if (e != cudaSuccess) return e;
    const long long work = count * (M / 2 + 1);
    const int threads = 256;
    e = launch_pdl(k_split_inplace, dim3((unsigned)((work + threads - 1) / threads)), dim3(threads), 0, s,
                   (float2*)out, count, lm, out_dist, tw);
    count_launch();
    return e;
}

template <int LA>
static cudaError_t launch_cols_merge_L(const float2* in, float2* out, long long count, int log2n2,
                                       long long in_dist, long long out_dist, const float2* tw, cudaStream_t s)
{
    using P = BPass<LA>;
    const long long blocks = count * ((1ll << log2n2) / P::C);
    return launch_pdl(k_cols_merge<LA>, dim3((unsigned)blocks), dim3(P::THREADS), P::SMEM, s, in, out, log2n2,
                      in_dist, out_dist, tw);
}

// Column pass with the real merge fused, column sub-length 2^la (7 .. 10).
static cudaError_t launch_cols_merge(int la, const float2* in, float2* out, long long count, int log2n2,
                                     long long in_dist, long long out_dist, const float2* tw, cudaStream_t s)
{
    switch (la) {
    case 7: return launch_cols_merge_L<7>(in, out, count, log2n2, in_dist, out_dist, tw, s);
    case 8: return launch_cols_merge_L<8>(in, out, count, log2n2, in_dist, out_dist, tw, s);
    case 9: return launch_cols_merge_L<9>(in, out, count, log2n2, in_dist, out_dist, tw, s);
    case 10: return launch_cols_merge_L<10>(in, out, count, log2n2, in_dist, out_dist, tw, s);
    default: return cudaErrorInvalidValue;
    }
}

// Two-pass real inverse with the merge fused into the column pass, for half
// lengths whose column sub-length is 2^7 .. 2^10 below the three-pass sizes.
static bool cols_merge_supported(int lm)
{
    const LargePlan p = large_plan(lm);
    return lm > kSmallMaxLog2Complex && lm < kThreePassMinLog2 && p.log2n1 >= 7 && p.log2n1 <= 10 &&
           p.log2n2 <= 14;
}

static cudaError_t launch_c2r_cols_merge(int lm, const float2* in, float2* out, long long count, long long in_dist,
                                         long long out_dist, const float2* tw, float2* tmp, size_t scratch_bytes,
                                         cudaStream_t s)
{
    const LargePlan p = large_plan(lm);
    const long long M = 1ll << lm;
    const long long group = (long long)(scratch_bytes / (sizeof(float2) * (size_t)M));
    if (group < 1) return cudaErrorInvalidValue;
    for (long long off = 0; off < count; off += group) {
        const long long cnt = count - off < group ? count - off : group;
        cudaError_t e = launch_cols_merge(p.log2n1, in + off * in_dist, tmp, cnt, p.log2n2, in_dist, M, tw, s);
        if (e != cudaSuccess) return e;
        e = launch_rows<true>(p.log2n2, tmp, out + off * out_dist, cnt, p.log2n1, M, out_dist, tw, s);
        if (e != cudaSuccess) return e;
        count_launch(2);
    }
    return cudaSuccess;
}

cudaError_t launch_large_c2r(int log2n, const void* in, void* out, long long count,
                             long long in_dist, long long out_dist, const float2* tw,
                             void* scratch, size_t scratch_bytes, cudaStream_t s)
{
    // in: n/2+1 complex per frame, out: n floats per frame (n/2 packed complex)
    // (half lengths 2^15 / 2^16: the cluster kernel with the merge fused into
    // its column tiles, 2780 / 2656 GB/s batched at n = 2^16 / 2^17 against
    // 2714 / 2554 for the fused two-pass form through HBM)
    const int lm = log2n - 1;
    const long long M = 1ll << lm;
    if (count <= 0) return cudaSuccess;
    if (l2pass_supported(lm) && ((uintptr_t)scratch & 127) == 0)
        return launch_l2pass(3, lm, in, out, count, in_dist, out_dist / 2, tw, scratch, scratch_bytes, s);
    if (cols_merge_supported(lm) && ((uintptr_t)scratch & 127) == 0)
        return launch_c2r_cols_merge(lm, (const float2*)in, (float2*)out, count, in_dist, out_dist / 2, tw,
                                     (float2*)scratch, scratch_bytes, s);
    int l1, l2, l3;
    if (lm >= kThreePassMinLog2 && plan3(lm, &l1, &l2, &l3) && ((uintptr_t)scratch & 127) == 0) {
        const long long group = (long long)(scratch_bytes / (sizeof(float2) * (size_t)M));
        if (group < 1) return cudaErrorInvalidValue;
        return launch_three_pass(C2R, lm, (const float2*)in, (float2*)out, count, in_dist, out_dist / 2, tw,
                                 (float2*)scratch, group, s);
    }
    const long long work = count * M;
    const int threads = 256;
    cudaError_t e = launch_pdl(k_merge, dim3((unsigned)((work + threads - 1) / threads)), dim3(threads), 0, s,
                               (const float2*)in, (float2*)out, count, lm, in_dist, out_dist / 2, tw);
    count_launch();
    if (e != cudaSuccess) return e;
    // inverse complex transform of the merged values, in place through scratch
    return launch_large_c2c(true, lm, out, out, count, out_dist / 2, out_dist / 2, tw, scratch,
                            scratch_bytes, s);
}

template <int L>
static cudaError_t attr_pass()
{
    using P = BPass<L>;
    cudaError_t e;
    if constexpr (L <= 10) {
        if ((e = cudaFuncSetAttribute(k_rows3<L, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P::SMEM)) != cudaSuccess) return e;
        if ((e = cudaFuncSetAttribute(k_rows3<L, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P::SMEM)) != cudaSuccess) return e;
    }
    if constexpr (L >= 7 && L <= 10) {
        if ((e = cudaFuncSetAttribute(k_rows_split<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P::SMEM)) != cudaSuccess) return e;
    }
    if constexpr (L >= 7 && L <= 10) {
        if ((e = cudaFuncSetAttribute(k_cols_merge<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P::SMEM)) != cudaSuccess) return e;
    }
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
