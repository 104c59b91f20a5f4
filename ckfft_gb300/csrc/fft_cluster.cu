// fft_cluster.cu -- single-pass complex transforms of 2^14 .. 2^16 points on
// thread-block clusters (distributed shared memory).
//
// N = K * M with M = 2^13 points per CTA and K = 2, 4 or 8 CTAs per cluster
// (one transform per cluster).  With n = c*M + m and k = K*k2 + k1:
//   X[K k2 + k1] = sum_m W_M^(m k2) [ W_N^(m k1) sum_c x[c M + m] W_K^(c k1) ]
//   1. CTA c loads the contiguous chunk x[cM .. cM+M) into shared memory A;
//   2. cluster barrier; CTA r takes positions m in [rM/K, (r+1)M/K), reads
//      x[cM + m] from every CTA's A, runs DFT_K in registers, multiplies
//      output k1 by W_N^(m k1) and writes it to CTA k1's A[m] -- in place:
//      position m of every CTA is read and written only by CTA r;
//   3. cluster barrier; each CTA runs the M-point Stockham transform of its A
//      (A is also the exchange area), giving X[K k2 + c] for k2 = 0 .. M-1;
//   4. the results go back to A, cluster barrier, and CTA c gathers the
//      contiguous output chunk X[cM .. cM+M) from the cluster (element g
//      lives in CTA g mod K at g / K) and stores it coalesced;
//   5. a last cluster barrier keeps every CTA's shared memory alive until its
//      peers have finished reading it.
// Every value is read from and written to HBM once (the two-pass path moves
// it twice); the exchanges run over the cluster's shared-memory network.
#include <cooperative_groups.h>

#include "fft_small.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace ckg {

constexpr int kClLog2M = 13;
constexpr int kClM = 1 << kClLog2M;
constexpr int kClThreads = kClM / 16;                              // 512: 16 values per thread
constexpr int kClA = (padded_len(kClM) + 31) / 32 * 32;            // exchange area (padded)
constexpr size_t kClSmem = sizeof(float2) * (size_t)kClA;           // 70 KB: two CTAs per SM

template <int K, bool INV>
__global__ void __cluster_dims__(K, 1, 1) __launch_bounds__(kClThreads, 2)
k_cluster_c2c(const float2* __restrict__ in, float2* __restrict__ out, long long in_dist, long long out_dist,
              const float2* __restrict__ tw)
{
    constexpr int M = kClM, T = kClThreads, R = 16;
    constexpr int N = K * M;
    constexpr int PER = M / K / T;                                 // positions per thread in step 2
    cg::cluster_group cluster = cg::this_cluster();
    const int c = (int)cluster.block_rank();
    const long long f = blockIdx.x / K;
    const int t = threadIdx.x;
    extern __shared__ __align__(128) float2 smem[];
    float2* A = smem;

    // 1. contiguous chunk c of transform f
    const float2* src = in + f * in_dist + (long long)c * M;
#pragma unroll
    for (int j = 0; j < R; ++j) A[t + j * T] = __ldcs(src + t + j * T);
    cluster.sync();

    // 2. radix-K step across the cluster
    const float2* lvl = tw + N;                                    // W_N^p at lvl[p]
#pragma unroll
    for (int p = 0; p < PER; ++p) {
        const int m = c * (M / K) + t + p * T;
        float2 x[K];
#pragma unroll
        for (int q = 0; q < K; ++q) x[q] = cluster.map_shared_rank(A, q)[m];
        dft<K, INV>(x);
#pragma unroll
        for (int k1 = 0; k1 < K; ++k1) {
            const float2 y = k1 == 0 ? x[0] : cmul(x[k1], tw_load<INV>(lvl, m * k1));
            cluster.map_shared_rank(A, k1)[m] = y;
        }
    }
    cluster.sync();

    // 3. local M-point transform of y_c (peers are done with this CTA's A)
    float2 v[R];
#pragma unroll
    for (int j = 0; j < R; ++j) v[j] = A[t + j * T];
    __syncthreads();                                       // A becomes the exchange area
    PaddedView view{A};
    stockham<kClLog2M, 4, INV, false>(v, t, tw, view);
    // 4. X[K k2 + c] for k2 = t + jT back to A (the last exchange ended with a
    //    barrier after its reads), then gather contiguous outputs
#pragma unroll
    for (int j = 0; j < R; ++j) A[t + j * T] = v[j];
    cluster.sync();
    float2* dst = out + f * out_dist + (long long)c * M;
#pragma unroll
    for (int j = 0; j < R; ++j) {
        const int g = c * M + t + j * T;
        __stcs(dst + t + j * T, cluster.map_shared_rank(A, g % K)[g / K]);
    }
    // 5. peers may still be reading this CTA's A
    cluster.sync();
}

template <int K, bool INV>
static cudaError_t launch_cl(const void* in, void* out, long long count, long long in_dist, long long out_dist,
                             const float2* tw, cudaStream_t s)
{
    k_cluster_c2c<K, INV><<<(unsigned)(count * K), kClThreads, kClSmem, s>>>(
        (const float2*)in, (float2*)out, in_dist, out_dist, tw);
    return cudaGetLastError();
}

bool cluster_supported(int log2n) { return log2n >= kClLog2M + 1 && log2n <= kClLog2M + 3; }

cudaError_t launch_cluster_c2c(bool inverse, int log2n, const void* in, void* out, long long count,
                               long long in_dist, long long out_dist, const float2* tw, cudaStream_t s)
{
    if (count <= 0) return cudaSuccess;
    cudaError_t e;
    switch (log2n - kClLog2M) {
    case 1: e = inverse ? launch_cl<2, true>(in, out, count, in_dist, out_dist, tw, s)
                        : launch_cl<2, false>(in, out, count, in_dist, out_dist, tw, s); break;
    case 2: e = inverse ? launch_cl<4, true>(in, out, count, in_dist, out_dist, tw, s)
                        : launch_cl<4, false>(in, out, count, in_dist, out_dist, tw, s); break;
    case 3: e = inverse ? launch_cl<8, true>(in, out, count, in_dist, out_dist, tw, s)
                        : launch_cl<8, false>(in, out, count, in_dist, out_dist, tw, s); break;
    default: return cudaErrorInvalidValue;
    }
    if (e == cudaSuccess) count_launch();
    return e;
}

template <int K, bool INV>
static cudaError_t attr_cl()
{
    return cudaFuncSetAttribute(k_cluster_c2c<K, INV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kClSmem);
}

cudaError_t prepare_cluster()
{
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = attr_cl<2, false>();
    if (e == cudaSuccess) e = attr_cl<2, true>();
    if (e == cudaSuccess) e = attr_cl<4, false>();
    if (e == cudaSuccess) e = attr_cl<4, true>();
    if (e == cudaSuccess) e = attr_cl<8, false>();
    if (e == cudaSuccess) e = attr_cl<8, true>();
    return e;
}

}  // namespace ckg
