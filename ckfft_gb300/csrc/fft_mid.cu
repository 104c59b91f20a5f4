// fft_mid.cu -- complex 2^15 and 2^16: one persistent CTA per SM, each CTA
// transforming whole transforms one after another, both passes of the
// two-pass decomposition (fft_passes.cuh) inside the CTA, the intermediate in
// L2, and every tile arriving in shared memory by bulk copies (1-D TMA).
//
// n = N1 N2.  Column pass ("A tiles"): DFT_N1 down CA adjacent columns and the
// twiddle W_n^(n2 k1); row pass ("B tiles"): DFT_N2 along RB rows, stored
// transposed.  A tile holds 4096 values (32 KiB): CA = 4096 / N1 columns,
// RB = 4096 / N2 rows.
//
// Thread roles (576 threads):
//   group A (warps 0-7)   column tiles of transform i+1 (from the input in HBM)
//   group B (warps 8-15)  row tiles of transform i (from the intermediate in L2)
//   warp 16               bulk copies of the column tiles into ring A
//   warp 17               bulk copies of the row tiles into ring B
// The two groups work on consecutive transforms at once, so the column pass
// of one transform overlaps the row pass of the previous one; the
// intermediate has two slots per CTA.  Each ring has two 32 KiB landing
// buffers: a group copies its tile into registers and releases the buffer
// at once, so the next tile's copy is in flight while the group computes.
//
// Intermediate layout (per slot): A tile a writes its 4096 values
// contiguously as [k1][c] (n2 = a CA + c), so a row tile (rows k1 = b RB ..
// b RB + RB-1) is TA contiguous chunks of RB x CA values, one bulk copy each;
// the row tile drops the chunks' L2 lines once they have landed.
//
// Ordering:
//   full[b]   the producer's expect_tx + copies -> the group's wait;
//   empty[b]  every thread of the group arrives after reading its values;
//   adone[s]  group A arrives once all column tiles of slot s are stored
//             (each storing thread fences generic -> async proxy first);
//             ring B's producer waits before copying row tiles of slot s;
//   bdone[s]  group B arrives once every row-tile copy of slot s has landed;
//             group A waits before writing slot s again.
// Every wait is bounded (tma.cuh); a wait that runs out sets the device
// error word and the abort flag, all roles leave their loops, and the
// producers wait (bounded) for copies still in flight before the CTA exits.
//
// Replaces, for these sizes, the reference's radix-4 recursion
// (src/ckfft/fft_default.cpp:168-266); same transform, Stockham order.
#include "fft_passes.cuh"
#include "jobs.h"
#include "kernels.h"
#include "tma.cuh"

namespace ckg {

constexpr int kMidGroup = 256;                      // threads per compute group
constexpr int kMidThreads = 2 * kMidGroup + 64;     // + two producer warps
constexpr int kMidTile = 4096;                      // values per tile
constexpr int kMidRing = 2;                         // landing buffers per ring

template <int LA, int LB>
struct MidCfg {
    static constexpr int N1 = 1 << LA, N2 = 1 << LB;
    static constexpr long long N = (long long)N1 * N2;
    static constexpr int CA = kMidTile / N1;         // columns per column tile
    static constexpr int RB = kMidTile / N2;         // rows per row tile
    static constexpr int TA = N2 / CA;               // column tiles per transform
    static constexpr int TB = N1 / RB;               // row tiles per transform
    static constexpr int RA = 16, RBV = 16;          // values per thread
    static constexpr int THA = N1 / RA;              // threads per column
    static constexpr int THB = N2 / RBV;             // threads per row
    static_assert(CA * THA == kMidGroup && RB * THB == kMidGroup, "a tile is one value set per group thread x16");
    static_assert(TA >= 1 && TB >= 1, "whole tiles");
    // shared memory (float2 units)
    static constexpr int XA = kMidTile + kMidTile / 16 + 1;                 // TileView<CA> exchange
    static constexpr int XB0 = RB * padded_len(N2);                          // padded rows
    static constexpr int XB = XB0 > XA ? XB0 : XA;                           // + transpose
    static constexpr int XA_AL = (XA + 15) / 16 * 16, XB_AL = (XB + 15) / 16 * 16;
    static constexpr size_t SMEM = sizeof(float2) * ((size_t)2 * kMidRing * kMidTile + XA_AL + XB_AL);
    static constexpr unsigned TILE_BYTES = kMidTile * sizeof(float2);
    static constexpr unsigned SEG_A = CA * sizeof(float2);                   // one row of a column tile
    static constexpr unsigned SEG_B = RB * CA * sizeof(float2);              // one chunk of a row tile
    static_assert(SEG_A % 16 == 0 && SEG_B % 16 == 0, "bulk copies move multiples of 16 bytes");
};

struct MidBars {
    unsigned long long fullA[kMidRing], emptyA[kMidRing], fullB[kMidRing], emptyB[kMidRing];
    unsigned long long adone[2], bdone[2];
    int abort;
};

__device__ __forceinline__ void group_sync(int id)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(kMidGroup) : "memory");
}

// Every thread of the group learns whether all of them had `ok` (a barrier).
__device__ __forceinline__ bool group_all(bool ok, int id)
{
    int r;
    asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.s32 p, %1, 0;\n\t"
                 "bar.red.and.pred q, %2, %3, p;\n\tselp.s32 %0, 1, 0, q;\n\t}"
                 : "=r"(r) : "r"((int)ok), "r"(id), "r"(kMidGroup) : "memory");
    return r != 0;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void fence_proxy_async_global()
{
    asm volatile("fence.proxy.async.global;" ::: "memory");
}

// Bounded wait that also watches the CTA's abort flag; false: stop.
__device__ __forceinline__ bool mid_wait(uint32_t bar, uint32_t phase, unsigned* err, volatile int* abort)
{
#pragma unroll 1
    for (int it = 0; it < kWaitTries; ++it) {
        if (mbar_try_wait(bar, phase)) return true;
        if ((it & 255) == 255 && *abort) return false;
    }
    if (err) *(volatile unsigned*)err = kErrWaitTimeout;
    *abort = 1;
    return false;
}

// Transform pointers: contiguous batch or a pointer table.
struct MidIO {
    const float2* in;
    float2* out;
    long long in_dist, out_dist;
    const FrameDesc* fr;
    __device__ __forceinline__ const float2* src(long long f) const { return fr ? fr[f].in : in + f * in_dist; }
    __device__ __forceinline__ float2* dst(long long f) const { return fr ? fr[f].out : out + f * out_dist; }
};

// Column tile: v[m] = x[n1 = t + m THA][column c] from the landing buffer
// ([n1][c] rows of CA values), DFT_N1, twiddle W_n^(n2 k1), stored to the
// slot's chunk a as [k1][c].
template <int LA, int LB, bool INV>
__device__ __forceinline__ void mid_cols(const float2* land, float2* xch, float2* chunk, int a, int tid,
                                         const float2* __restrict__ tw, uint32_t empty_bar)
{
    using M = MidCfg<LA, LB>;
    const int c = tid % M::CA, t = tid / M::CA;
    float2 v[M::RA];
#pragma unroll
    for (int m = 0; m < M::RA; ++m) v[m] = land[(t + m * M::THA) * M::CA + c];
    mbar_arrive(empty_bar);                        // the landing buffer may be refilled
    stockham<LA, 4, INV, false, 1, kMidGroup>(v, t, tw, TileView<M::CA>{xch, c});
    // W_n^(n2 k1), k1 = t + m THA = t + (4q + r) THA: the factors of
    // cols_twiddle_store (fft_passes.cuh)
    constexpr int ln = LA + LB;
    constexpr int mask = (1 << ln) - 1;
    const int n2 = a * M::CA + c;
    const int p0 = n2 * t, pT = (n2 * M::THA) & mask;
    const float2 w0 = big_twiddle<INV>(tw, ln, p0 & mask);
    const float2 b1 = big_twiddle<INV>(tw, ln, pT), b2 = big_twiddle<INV>(tw, ln, (2 * pT) & mask);
    const float2 b3 = cmul(b1, b2);
    const float2 l0 = big_twiddle<INV>(tw, ln, (pT << 2) & mask);
    const float2 l1 = big_twiddle<INV>(tw, ln, (pT << 3) & mask);
    float2* dst = chunk + t * M::CA + c;
    static_for<0, 4>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        float2 aq = w0;
        if constexpr (q & 1) aq = cmul(aq, l0);
        if constexpr (q & 2) aq = cmul(aq, l1);
        constexpr int step = M::THA * M::CA;
        dst[(4 * q + 0) * step] = cmul(v[4 * q + 0], aq);
        dst[(4 * q + 1) * step] = cmul(v[4 * q + 1], cmul(aq, b1));
        dst[(4 * q + 2) * step] = cmul(v[4 * q + 2], cmul(aq, b2));
        dst[(4 * q + 3) * step] = cmul(v[4 * q + 3], cmul(aq, b3));
    });
}

// Row tile b: rows k1 = b RB + r; v[m] = row element n2 = t + m THB from the
// landing buffer (TA chunks of [RB][CA]), DFT_N2, transposed through shared
// memory and stored at X[k1 + N1 k2].
template <int LA, int LB, bool INV>
__device__ __forceinline__ void mid_rows(const float2* land, float2* xch, float2* __restrict__ y, int b, int tid,
                                         const float2* __restrict__ tw, uint32_t empty_bar, int bar_id)
{
    using M = MidCfg<LA, LB>;
    const int r = tid / M::THB, t = tid % M::THB;
    float2 v[M::RBV];
#pragma unroll
    for (int m = 0; m < M::RBV; ++m) {
        const int n2 = t + m * M::THB;
        v[m] = land[(n2 / M::CA) * (M::RB * M::CA) + r * M::CA + (n2 % M::CA)];
    }
    mbar_arrive(empty_bar);
    PaddedView view{xch + r * padded_len(M::N2)};
    stockham<LB, 4, INV, (M::THB <= 32)>(v, t, tw, view);
    group_sync(bar_id);                            // the exchange area becomes the transpose area
#pragma unroll
    for (int m = 0; m < M::RBV; ++m) xch[TileView<M::RB>::slot(t + m * M::THB, r)] = v[m];
    group_sync(bar_id);
    const int r2 = tid % M::RB, t2 = tid / M::RB;
    float2* dst = y + (long long)b * M::RB + r2;
    constexpr int T2 = kMidGroup / M::RB;
#pragma unroll
    for (int m = 0; m < M::N2 / T2; ++m) {
        const int k2 = t2 + m * T2;
        __stcs(dst + (long long)k2 * M::N1, xch[TileView<M::RB>::slot(k2, r2)]);
    }
    group_sync(bar_id);                            // the transpose area is free for the next tile
}

// scratch: 2 slots of n values per CTA (gridDim.x CTAs), 128-byte aligned.
template <int LA, int LB, int KIND>
// 576 threads x 112 registers fit the SM's 64 K registers (one CTA per SM)
__global__ void __maxnreg__(112)
k_mid(MidIO io, long long count, float2* __restrict__ scratch, const float2* __restrict__ tw, unsigned* err)
{
    using M = MidCfg<LA, LB>;
    constexpr bool INV = KIND == 1;
    extern __shared__ __align__(128) float2 smem[];
    __shared__ MidBars sb;
    float2* ringA = smem;
    float2* ringB = smem + kMidRing * kMidTile;
    float2* xchA = smem + 2 * kMidRing * kMidTile;
    float2* xchB = xchA + M::XA_AL;
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const long long mine = count > blockIdx.x ? (count - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    float2* slots = scratch + (long long)blockIdx.x * 2 * M::N;
    volatile int* abort = &sb.abort;

    if (tid == 0) {
        for (int i = 0; i < kMidRing; ++i) {
            mbar_init(smem_addr(&sb.fullA[i]), 1);
            mbar_init(smem_addr(&sb.fullB[i]), 1);
            mbar_init(smem_addr(&sb.emptyA[i]), kMidGroup);
            mbar_init(smem_addr(&sb.emptyB[i]), kMidGroup);
        }
        for (int s = 0; s < 2; ++s) {
            mbar_init(smem_addr(&sb.adone[s]), 1);
            mbar_init(smem_addr(&sb.bdone[s]), 1);
        }
        sb.abort = 0;
        fence_mbar_init();
    }
    __syncthreads();
    pdl_start();

    if (warp == 16) {
        // ---- producer of ring A: column tiles (rows of CA values, N1 of them)
        long long k = 0;
        for (long long i = 0; i < mine && !*abort; ++i) {
            const float2* x = io.src(blockIdx.x + i * gridDim.x);
            for (int a = 0; a < M::TA; ++a, ++k) {
                const int buf = (int)(k % kMidRing);
                const bool ok = k < kMidRing || mid_wait(smem_addr(&sb.emptyA[buf]), (uint32_t)((k / kMidRing - 1) & 1), err, abort);
                if (!__all_sync(0xffffffffu, ok)) break;
                const uint32_t full = smem_addr(&sb.fullA[buf]);
                if (lane == 0) mbar_arrive_expect_tx(full, M::TILE_BYTES);
                __syncwarp();
                const uint32_t dst = smem_addr(ringA + buf * kMidTile);
                for (int n1 = lane; n1 < M::N1; n1 += 32)
                    bulk_load(dst + n1 * M::SEG_A, x + (long long)n1 * M::N2 + a * M::CA, M::SEG_A, full);
            }
        }
        // copies still in flight land before the CTA may exit
        if (*abort) {
            for (long long j = (k > kMidRing ? k - kMidRing : 0); j < k; ++j)
                for (int it = 0; it < 4096 && !mbar_try_wait(smem_addr(&sb.fullA[j % kMidRing]), (uint32_t)((j / kMidRing) & 1)); ++it) {
                }
        }
    } else if (warp == 17) {
        // ---- producer of ring B: row tiles (TA chunks of RB x CA values)
        long long k = 0;
        for (long long i = 0; i < mine && !*abort; ++i) {
            const int s = (int)(i & 1);
            if (!__all_sync(0xffffffffu, mid_wait(smem_addr(&sb.adone[s]), (uint32_t)((i >> 1) & 1), err, abort))) break;
            fence_proxy_async_global();
            const float2* slot = slots + s * M::N;
            for (int b = 0; b < M::TB; ++b, ++k) {
                const int buf = (int)(k % kMidRing);
                const bool ok = k < kMidRing || mid_wait(smem_addr(&sb.emptyB[buf]), (uint32_t)((k / kMidRing - 1) & 1), err, abort);
                if (!__all_sync(0xffffffffu, ok)) break;
                const uint32_t full = smem_addr(&sb.fullB[buf]);
                if (lane == 0) mbar_arrive_expect_tx(full, M::TILE_BYTES);
                __syncwarp();
                const uint32_t dst = smem_addr(ringB + buf * kMidTile);
                for (int a = lane; a < M::TA; a += 32)
                    bulk_load(dst + a * M::SEG_B, slot + (long long)a * kMidTile + (long long)b * M::RB * M::CA,
                              M::SEG_B, full);
            }
            if (*abort) break;
        }
        if (*abort) {
            for (long long j = (k > kMidRing ? k - kMidRing : 0); j < k; ++j)
                for (int it = 0; it < 4096 && !mbar_try_wait(smem_addr(&sb.fullB[j % kMidRing]), (uint32_t)((j / kMidRing) & 1)); ++it) {
                }
        }
    } else if (warp < 8) {
        // ---- group A: column tiles into the slot of transform i
        const int g = tid;
        long long k = 0;
        for (long long i = 0; i < mine; ++i) {
            const int s = (int)(i & 1);
            // the slot's previous transform (i - 2) must have been copied out
            if (!group_all(i < 2 || mid_wait(smem_addr(&sb.bdone[s]), (uint32_t)(((i - 2) >> 1) & 1), err, abort), 1))
                break;
            float2* slot = slots + s * M::N;
            bool ok = true;
            for (int a = 0; a < M::TA; ++a, ++k) {
                const int buf = (int)(k % kMidRing);
                if (!group_all(mid_wait(smem_addr(&sb.fullA[buf]), (uint32_t)((k / kMidRing) & 1), err, abort), 1)) {
                    ok = false;
                    break;
                }
                // stockham's last exchange ends with a group barrier: the
                // exchange area is free for the next tile when this returns
                mid_cols<LA, LB, INV>(ringA + buf * kMidTile, xchA, slot + (long long)a * kMidTile, a, g, tw,
                                      smem_addr(&sb.emptyA[buf]));
            }
            if (!ok) break;
            fence_proxy_async_global();            // the stores above are read next by bulk copies
            group_sync(1);
            if (g == 0) mbar_arrive(smem_addr(&sb.adone[s]));
        }
    } else {
        // ---- group B: row tiles of transform i, results to the output
        const int g = tid - kMidGroup;
        long long k = 0;
        for (long long i = 0; i < mine; ++i) {
            const int s = (int)(i & 1);
            float2* y = io.dst(blockIdx.x + i * gridDim.x);
            const float2* slot = slots + s * M::N;
            bool ok = true;
            for (int b = 0; b < M::TB; ++b, ++k) {
                const int buf = (int)(k % kMidRing);
                if (!group_all(mid_wait(smem_addr(&sb.fullB[buf]), (uint32_t)((k / kMidRing) & 1), err, abort), 2)) {
                    ok = false;
                    break;
                }
                // the chunks of this row tile are dead: drop their L2 lines
                {
                    constexpr int lines = (int)(M::SEG_B / 128);
                    for (int l = g; l < M::TA * lines; l += kMidGroup) {
                        const int a = l / lines, o = l % lines;
                        const char* p = (const char*)(slot + (long long)a * kMidTile + (long long)b * M::RB * M::CA) + 128 * o;
                        asm volatile("discard.global.L2 [%0], 128;" ::"l"(p) : "memory");
                    }
                }
                mid_rows<LA, LB, INV>(ringB + buf * kMidTile, xchB, y, b, g, tw, smem_addr(&sb.emptyB[buf]), 2);
            }
            if (!ok) break;
            // every copy out of slot s has landed and its lines were dropped
            // (mid_rows ends with a group barrier): group A may refill it
            if (g == 0) mbar_arrive(smem_addr(&sb.bdone[s]));
        }
    }
}

template <int LA, int LB, int KIND>
static cudaError_t attr_mid()
{
    return cudaFuncSetAttribute(k_mid<LA, LB, KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)MidCfg<LA, LB>::SMEM);
}

static int mid_sms()
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

bool mid_supported(int log2n) { return log2n == 15 || log2n == 16; }

size_t mid_scratch_bytes(int log2n, long long count)
{
    const long long ctas = count < mid_sms() ? count : mid_sms();
    return (size_t)ctas * 2 * sizeof(float2) * ((size_t)1 << log2n);
}

template <int LA, int LB>
static cudaError_t launch_mid_L(int kind, const MidIO& io, long long count, const float2* tw, float2* scratch,
                                cudaStream_t s)
{
    using M = MidCfg<LA, LB>;
    const unsigned grid = (unsigned)(count < mid_sms() ? count : mid_sms());
    unsigned* err = device_error_word();
    return kind == 0 ? launch_pdl(k_mid<LA, LB, 0>, dim3(grid), dim3(kMidThreads), M::SMEM, s, io, count, scratch, tw, err)
                     : launch_pdl(k_mid<LA, LB, 1>, dim3(grid), dim3(kMidThreads), M::SMEM, s, io, count, scratch, tw, err);
}

static cudaError_t launch_mid_io(int kind, int log2n, const MidIO& io, long long count, const float2* tw,
                                 void* scratch, size_t scratch_bytes, cudaStream_t s)
{
    if (!mid_supported(log2n) || (kind != 0 && kind != 1)) return cudaErrorInvalidValue;
    if (count <= 0) return cudaSuccess;
    if (scratch_bytes < mid_scratch_bytes(log2n, count) || ((uintptr_t)scratch & 127)) return cudaErrorInvalidValue;
    cudaError_t e = log2n == 15 ? launch_mid_L<7, 8>(kind, io, count, tw, (float2*)scratch, s)
                                : launch_mid_L<8, 8>(kind, io, count, tw, (float2*)scratch, s);
    if (e == cudaSuccess) count_launch();
    return e;
}

// Contiguous batch; in / out 16-byte aligned and dists multiples of 2 values.
cudaError_t launch_mid(int kind, int log2n, const void* in, void* out, long long count, long long in_dist,
                       long long out_dist, const float2* tw, void* scratch, size_t scratch_bytes, cudaStream_t s)
{
    if (((uintptr_t)in & 15) || (in_dist & 1)) return cudaErrorInvalidValue;
    MidIO io{(const float2*)in, (float2*)out, in_dist, out_dist, nullptr};
    return launch_mid_io(kind, log2n, io, count, tw, scratch, scratch_bytes, s);
}

// A table of transforms (grouped launches of a job run); every input 16-byte aligned.
cudaError_t launch_mid_table(int kind, int log2n, const FrameDesc* fr, long long count, const float2* tw,
                             void* scratch, size_t scratch_bytes, cudaStream_t s)
{
    MidIO io{nullptr, nullptr, 0, 0, fr};
    return launch_mid_io(kind, log2n, io, count, tw, scratch, scratch_bytes, s);
}

cudaError_t prepare_mid()
{
    cudaError_t e = attr_mid<7, 8, 0>();
    if (e == cudaSuccess) e = attr_mid<7, 8, 1>();
    if (e == cudaSuccess) e = attr_mid<8, 8, 0>();
    if (e == cudaSuccess) e = attr_mid<8, 8, 1>();
    return e;
}

}  // namespace ckg
