// fft_l2pass.cu -- complex 2^15 and 2^16 in two passes whose intermediate
// never reaches HBM.
//
// The multi-pass transform of fft_large.cu (columns, then rows, see
// fft_passes.cuh) runs here inside one thread-block cluster of K CTAs per
// transform: the cluster's CTAs share the column tiles, meet at a cluster
// barrier (release / acquire at cluster scope), share the row tiles, and each
// row tile's CTA drops the intermediate's L2 lines once it has read them.
// The intermediate of the transforms in flight (resident clusters x 8n
// bytes, 38 MB at both sizes) stays in the 129 MB L2, so HBM sees the input
// read once and the output written once -- the traffic of a single pass --
// while the batched two-pass kernels move every value through HBM twice.
// Measured on GB300 (batches of 1 GiB): 2^15 3929 GB/s, 2^16 3851, against
// 3145 / 3105 for the two-pass kernels through HBM; the kernel is bound by
// the two passes' instructions, not by HBM (43 % DRAM throughput, no
// intermediate bytes in DRAM).  At 2^17 (8-CTA clusters, 76 MB of
// intermediate in flight) it ties with the two HBM passes (2935 / 2963
// against 2928 / 2926 GB/s forward / inverse) and is not used there.  Real transforms of 2^16 / 2^17 points (these half
// lengths) run here too, the split fused into the row tiles and the merge
// into the column tiles (pass_rows_split, pass_cols_merge): forward 2749 /
// 2621 GB/s, inverse 2780 / 2656, against 2507 / 2609 and 2714 / 2554 for
// the same fused passes through HBM.
#include <cooperative_groups.h>

#include "fft_passes.cuh"
#include "jobs.h"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace ckg {

constexpr int kL2Threads = 256;

template <int LA, int LB, int KIND = 0>
struct L2Cfg {
    // CTAs per transform: 4 at 2^15, 8 at 2^16 and for the real forward
    // (measured on GB300, batches of 1 GiB: complex 2^15 3663 GB/s with 4,
    // 3513 with 8, 3474 with 2; 2^16 3591 with 8, 3424 with 4, 3121 with 2;
    // real n = 2^16 forward 2749 with 8, 2584 with 4, inverse 2777 with 4,
    // 2689 with 8)
    static constexpr int K = LA + LB <= 15 && KIND != 2 ? 4 : 8;
    using PA = PassCfg<LA, kL2Threads>;
    using PB = PassCfg<LB, kL2Threads>;
    static constexpr int SGA = kL2Threads / PA::THREADS;     // column tiles at once
    static constexpr int SGB = kL2Threads / PB::THREADS;     // row tiles at once
    static constexpr int TILES_A = (1 << LB) / PA::C;        // column tiles of one transform
    static constexpr int TILES_B = (1 << LA) / PB::C;        // row tiles
    static constexpr int ITER_A = TILES_A / (K * SGA);
    static constexpr int ITER_B = TILES_B / (K * SGB);
    static constexpr size_t SMEM_A = PA::SMEM * SGA, SMEM_B = PB::SMEM * SGB;
    static constexpr size_t SMEM = SMEM_A > SMEM_B ? SMEM_A : SMEM_B;
    static_assert(PA::THREADS * SGA == kL2Threads && PB::THREADS * SGB == kL2Threads, "whole CTAs per phase");
    static_assert(ITER_A >= 1 && ITER_A * K * SGA == TILES_A, "column tiles split evenly");
    static_assert(ITER_B >= 1 && ITER_B * K * SGB == TILES_B, "row tiles split evenly");
};

__device__ __forceinline__ void cluster_barrier(cg::cluster_group& cluster)
{
    // global stores before the barrier are seen by the peers' loads after it:
    // the arrive releases and the wait acquires at cluster scope (no separate
    // fence: one cost a membar stall of about 1 per issued instruction)
    (void)cluster;
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// One transform per cluster: blockIdx.x / K.  scratch holds 2^(LA+LB) values
// per transform of the launch (128-byte aligned rows).
// KIND 0 / 1: complex forward / inverse of n = 2^(LA+LB) points.
// KIND 2: real forward of 2n reals (read as n packed complex values) to
// n + 1 bins, the split fused into the row tiles (pass_rows_split).
// KIND 3: real inverse of n + 1 bins to 2n reals, the merge fused into the
// column tiles (pass_cols_merge).
// fr != nullptr: transform f reads fr[f].in and writes fr[f].out (a grouped
// launch of a job run) instead of in + f in_dist, out + f out_dist.
template <int LA, int LB, int KIND>
__global__ void __cluster_dims__(L2Cfg<LA, LB, KIND>::K, 1, 1) __launch_bounds__(kL2Threads, 4)
k_l2_c2c(const float2* __restrict__ in, float2* __restrict__ out, float2* __restrict__ scratch, long long in_dist,
         long long out_dist, const float2* __restrict__ tw, const FrameDesc* __restrict__ fr)
{
    using C = L2Cfg<LA, LB, KIND>;
    constexpr bool INV = KIND == 1 || KIND == 3;
    constexpr long long n = 1ll << (LA + LB);
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const long long f = blockIdx.x / C::K;
    extern __shared__ __align__(128) float2 smem[];
    pdl_start();
    const float2* x = fr ? fr[f].in : in + f * in_dist;
    float2* y = fr ? fr[f].out : out + f * out_dist;
    float2* s = scratch + f * n;
    // columns: the input -> s
    const int sga = threadIdx.x / C::PA::THREADS, ta = threadIdx.x % C::PA::THREADS;
#pragma unroll 1
    for (int i = 0; i < C::ITER_A; ++i) {
        const int tile = (i * C::K + rank) * C::SGA + sga;
        if constexpr (KIND == 3) pass_cols_merge<LA, kL2Threads>(x, s, LB, tile, ta, smem + sga * C::PA::SLOTS, tw);
        else pass_cols<LA, INV, false, kL2Threads>(x, s, LB, tile, ta, smem + sga * C::PA::SLOTS, tw);
        __syncthreads();                             // the tile's shared memory is reused
    }
    // every column tile of the transform is in L2 before any row tile reads it
    cluster_barrier(cluster);
    const int sgb = threadIdx.x / C::PB::THREADS, tb = threadIdx.x % C::PB::THREADS;
    // the row pass reloads its twiddles: at 2^16 its second stage needs the
    // same table entries as the column pass's, and keeping those live
    // across the barrier spills registers
    const float2* twb = tw;
    asm volatile("" : "+l"(twb));
#pragma unroll 1
    for (int i = 0; i < C::ITER_B; ++i) {
        const int tile = (i * C::K + rank) * C::SGB + sgb;
        if constexpr (KIND == 2)
            pass_rows_split<LB, kL2Threads, true>(s, y, LA, tile, tb, smem + sgb * C::PB::SLOTS, twb, LA);
        else pass_rows_xt<LB, INV, true, kL2Threads, true>(s, y, LA, tile, tb, smem + sgb * C::PB::SLOTS, twb);
        __syncthreads();
    }
}

template <int LA, int LB, int KIND>
static cudaError_t launch_l2_L(const float2* in, float2* out, float2* scratch, long long count, long long in_dist,
                               long long out_dist, const float2* tw, cudaStream_t s, const FrameDesc* fr = nullptr)
{
    using C = L2Cfg<LA, LB, KIND>;
    return launch_pdl(k_l2_c2c<LA, LB, KIND>, dim3((unsigned)(count * C::K)), dim3(kL2Threads), C::SMEM, s, in,
                      out, scratch, in_dist, out_dist, tw, fr);
}

bool l2pass_supported(int log2n) { return log2n >= 15 && log2n <= 16; }

// kind: 0 / 1 complex forward / inverse, 2 / 3 real forward / inverse of
// 2^(log2n+1) reals (log2n: the complex half length); dists in complex units.
cudaError_t launch_l2pass(int kind, int log2n, const void* in, void* out, long long count, long long in_dist,
                          long long out_dist, const float2* tw, void* scratch, size_t scratch_bytes, cudaStream_t s)
{
    if (!l2pass_supported(log2n) || kind < 0 || kind > 3) return cudaErrorInvalidValue;
    if (count <= 0) return cudaSuccess;
    const long long n = 1ll << log2n;
    const long long group = (long long)(scratch_bytes / (sizeof(float2) * (size_t)n));
    if (group < 1 || ((uintptr_t)scratch & 127)) return cudaErrorInvalidValue;
    const float2* src = (const float2*)in;
    float2* dst = (float2*)out;
    float2* tmp = (float2*)scratch;
    for (long long off = 0; off < count; off += group) {
        const long long cnt = count - off < group ? count - off : group;
        const float2* a = src + off * in_dist;
        float2* b = dst + off * out_dist;
        cudaError_t e;
#define CKG_L2_KIND(LA, LB)                                                                        \
    switch (kind) {                                                                                \
    case 0: e = launch_l2_L<LA, LB, 0>(a, b, tmp, cnt, in_dist, out_dist, tw, s); break;           \
    case 1: e = launch_l2_L<LA, LB, 1>(a, b, tmp, cnt, in_dist, out_dist, tw, s); break;           \
    case 2: e = launch_l2_L<LA, LB, 2>(a, b, tmp, cnt, in_dist, out_dist, tw, s); break;           \
    default: e = launch_l2_L<LA, LB, 3>(a, b, tmp, cnt, in_dist, out_dist, tw, s); break;          \
    }
        if (log2n == 15) { CKG_L2_KIND(7, 8) }
        else { CKG_L2_KIND(8, 8) }
#undef CKG_L2_KIND
        if (e != cudaSuccess) return e;
        count_launch();
    }
    return cudaSuccess;
}

// The same over a table of transforms (a grouped launch of a job run).
cudaError_t launch_l2pass_table(int kind, int log2n, const FrameDesc* fr, long long count, const float2* tw,
                                void* scratch, size_t scratch_bytes, cudaStream_t s)
{
    if (!l2pass_supported(log2n) || kind < 0 || kind > 3) return cudaErrorInvalidValue;
    if (count <= 0) return cudaSuccess;
    const long long n = 1ll << log2n;
    const long long group = (long long)(scratch_bytes / (sizeof(float2) * (size_t)n));
    if (group < 1 || ((uintptr_t)scratch & 127)) return cudaErrorInvalidValue;
    float2* tmp = (float2*)scratch;
    for (long long off = 0; off < count; off += group) {
        const long long cnt = count - off < group ? count - off : group;
        const FrameDesc* g = fr + off;
        cudaError_t e;
#define CKG_L2_KIND(LA, LB)                                                                              \
    switch (kind) {                                                                                      \
    case 0: e = launch_l2_L<LA, LB, 0>(nullptr, nullptr, tmp, cnt, 0, 0, tw, s, g); break;               \
    case 1: e = launch_l2_L<LA, LB, 1>(nullptr, nullptr, tmp, cnt, 0, 0, tw, s, g); break;               \
    case 2: e = launch_l2_L<LA, LB, 2>(nullptr, nullptr, tmp, cnt, 0, 0, tw, s, g); break;               \
    default: e = launch_l2_L<LA, LB, 3>(nullptr, nullptr, tmp, cnt, 0, 0, tw, s, g); break;              \
    }
        if (log2n == 15) { CKG_L2_KIND(7, 8) }
        else { CKG_L2_KIND(8, 8) }
#undef CKG_L2_KIND
        if (e != cudaSuccess) return e;
        count_launch();
    }
    return cudaSuccess;
}

template <int LA, int LB>
static cudaError_t attr_l2()
{
    const int smem = (int)L2Cfg<LA, LB>::SMEM;
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = cudaFuncSetAttribute(k_l2_c2c<LA, LB, 0>, a, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_l2_c2c<LA, LB, 1>, a, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_l2_c2c<LA, LB, 2>, a, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_l2_c2c<LA, LB, 3>, a, smem);
    return e;
}

cudaError_t prepare_l2pass()
{
    cudaError_t e = attr_l2<7, 8>();
    if (e == cudaSuccess) e = attr_l2<8, 8>();
    return e;
}

}  // namespace ckg
