// fft_mid.cu -- complex 2^15 and 2^16: persistent CTAs (one per SM), each
// cluster of CL CTAs transforming whole transforms one after another, both
// passes of the two-pass decomposition (fft_passes.cuh) inside the cluster,
// the intermediate in L2, and every tile arriving in shared memory by
// asynchronous copies while the previous tile computes.
//
// n = N1 N2.  Column pass ("A tiles"): DFT_N1 down CA adjacent columns and the
// twiddle W_n^(n2 k1); row pass ("B tiles"): DFT_N2 along RB rows, stored
// transposed.  A tile holds 4096 values (32 KiB): CA = 4096 / N1 columns,
// RB = 4096 / N2 rows.
//
// Thread roles (576 threads):
//   group A (warps 0-7)   column tiles of transform i+1 (from the input in HBM)
//   group B (warps 8-15)  row tiles of transform i (from the intermediate in L2)
//   warp 16               copies of the column tiles into ring A: 16-byte
//                         cp.async pieces (a column tile is N1 rows of 128 or
//                         256 bytes; one bulk copy per row measured 1.6-2.8x
//                         slower: the copy engine's cost per operation, not
//                         the bytes, set the rate)
//   warp 17               copies of the row tiles into ring B: one bulk copy
//                         (1-D TMA) per 2-4 KiB chunk
// The two groups work on consecutive transforms at once, so the column pass
// of one transform overlaps the row pass of the previous one; the
// intermediate has two slots per cluster.  Each ring has two 32 KiB landing
// buffers: a group copies its tile into registers and releases the buffer
// at once, so the next tile's copy is in flight while the group computes.
// With CL = 2 (complex 2^16) the two CTAs of a cluster split every
// transform's tiles, which halves the intermediate each SM keeps in L2.
//
// Intermediate layout (per slot): A tile a writes its 4096 values
// contiguously as [k1][c] (n2 = a CA + c), so a row tile (rows k1 = b RB ..
// b RB + RB-1) is TA contiguous chunks of RB x CA values, one bulk copy each;
// the row tile drops the chunks' L2 lines once they have landed.
//
// Ordering:
//   full[b]   ring A: every producer lane's cp.async arrival; ring B: the
//             producer's expect_tx + bulk copies -> the group's wait;
//   empty[b]  every thread of the group arrives after reading its values;
//   adone[s]  group A of every CTA of the cluster arrives once its column
//             tiles of slot s are stored (each storing thread fences generic
//             -> async proxy first); ring B's producers wait before copying
//             row tiles of slot s;
//   bdone[s]  group B of every CTA arrives once its row-tile copies of slot
//             s have landed and their lines were dropped; group A waits
//             before writing slot s again.
// Every mbarrier wait is bounded (tma.cuh); a wait that runs out sets the
// device error word and the abort flag, all roles leave their loops
// (decisions are made uniform inside a warp or group first), and the
// producers wait (bounded) for copies still in flight before the CTA exits.
//
// Replaces, for these sizes, the reference's radix-4 recursion
// (src/ckfft/fft_default.cpp:168-266); same transform, Stockham order.
#include "fft_passes.cuh"
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
    static_assert(CA * THA == kMidGroup && RB * THB == kMidGroup, "a tile is 16 values per group thread");
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
    static_assert(SEG_A % 16 == 0 && SEG_B % 16 == 0, "copies move multiples of 16 bytes");
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

// L2 eviction policies: inputs are read once (evict first), the
// intermediate should stay in L2 until the row pass has read it (evict last).
__device__ __forceinline__ uint64_t policy_evict_first()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint64_t policy_evict_last()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

// 16-byte asynchronous copy global -> shared (L2 only, with an L2 policy),
// and an arrival on `bar` once all of this thread's earlier such copies
// have landed.
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint64_t pol)
{
    asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "l"(pol)
                 : "memory");
}

__device__ __forceinline__ void cp_async_arrive(uint32_t bar)
{
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void st_hint(float2* p, float2 v, uint64_t pol)
{
    asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(v.x), "f"(v.y), "l"(pol)
                 : "memory");
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

// Cluster-scope forms: a CTA of a cluster arrives on the barriers of every
// CTA of the cluster (the intermediate is shared), and waits with acquire
// at cluster scope.
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t bar, int rank)
{
    uint32_t remote;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(bar), "r"(rank));
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(remote) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait_cluster(uint32_t bar, uint32_t phase)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(bar), "r"(phase) : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mid_wait_cluster(uint32_t bar, uint32_t phase, unsigned* err, volatile int* abort)
{
#pragma unroll 1
    for (int it = 0; it < kWaitTries; ++it) {
        if (mbar_try_wait_cluster(bar, phase)) return true;
        if ((it & 255) == 255 && *abort) return false;
    }
    if (err) *(volatile unsigned*)err = kErrWaitTimeout;
    *abort = 1;
    return false;
}

__device__ __forceinline__ void cluster_sync_all()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// DFT of 2^LS points (LS = 7, 8) held as 16 values by each of 2^LS / 16
// threads: a radix-16 stage without twiddles, one exchange, and a last stage
// whose table twiddles the thread loaded once (they depend on the thread
// only, not on the tile).
template <int LS, bool INV>
struct Dft2 {
    static_assert(Sched<LS, 4>::nstages == 2, "two stages");
    static constexpr int L1 = Sched<LS, 4>::lrs(1);
    static constexpr int U = 16 >> L1;
    float2 wb[U][L1];
    __device__ __forceinline__ void load(int t, const float2* __restrict__ tw)
    {
        stage_twiddles<LS, 4, L1, 4, INV>(t, tw, wb);
    }
    template <bool WARP, int BAR_ID, int BAR_N, class View>
    __device__ __forceinline__ void run(float2 (&v)[16], int t, const View& view) const
    {
        stage_compute<LS, 4, 4, 0, INV>(v, t, nullptr);
        stage_exchange<LS, 4, 4, 0, WARP, BAR_ID, BAR_N>(v, t, view);
        stage_compute_pre<LS, 4, L1, 4, INV>(v, wb);
    }
};

// Column-pass twiddle factors of one thread for one column tile.
struct ColTw {
    float2 w0, b1, b2, l0, l1;
};

// Transform pointers of a contiguous batch.
struct MidIO {
    const float2* in;
    float2* out;
    long long in_dist, out_dist;
    __device__ __forceinline__ const float2* src(long long f) const { return in + f * in_dist; }
    __device__ __forceinline__ float2* dst(long long f) const { return out + f * out_dist; }
};

// W_n^(n2 k1) for k1 = t + m THA, m = 4q + r, as W_n^(n2 t) W_n^(4q n2 THA)
// W_n^(r n2 THA); the factors are single table entries (level 2^q holds
// W_(2^q)^j at 2^q + j): W_n^(n2 THA) = W_(n/THA)^n2, ..., W_n^(8 n2 THA) =
// W_(2 N2)^n2.  Loaded one tile ahead so that their latency is hidden.
template <int LA, int LB, bool INV>
__device__ __forceinline__ ColTw col_twiddles(int a, int tid, const float2* __restrict__ tw)
{
    using M = MidCfg<LA, LB>;
    constexpr long long n = M::N;
    static_assert(4 * M::N2 == n / (4 * M::THA), "THA = N1 / 16");
    const int c = tid % M::CA, t = tid / M::CA;
    const int n2 = a * M::CA + c;
    ColTw w;
    w.w0 = tw_load<INV>(tw + n, (int)(((long long)n2 * t) & (n - 1)));
    w.b1 = tw_load<INV>(tw + n / M::THA, n2);
    w.b2 = tw_load<INV>(tw + n / (2 * M::THA), n2);
    w.l0 = tw_load<INV>(tw + 4 * M::N2, n2);
    w.l1 = tw_load<INV>(tw + 2 * M::N2, n2);
    return w;
}

// Column tile: v[m] = x[n1 = t + m THA][column c] from the landing buffer
// ([n1][c] rows of CA values), DFT_N1, twiddle W_n^(n2 k1) (factors `w`),
// stored to the slot's chunk a as [k1][c] (kept in L2: policy `pol`).  The
// exchange's last barrier precedes the stores, so the exchange area is free
// for the next tile when this returns.
template <int LA, int LB, bool INV>
__device__ __forceinline__ void mid_cols(const float2* land, float2* xch, float2* chunk, int tid,
                                         const Dft2<LA, INV>& dft, const ColTw& w, uint32_t empty_bar,
                                         uint64_t pol)
{
    using M = MidCfg<LA, LB>;
    const int c = tid % M::CA, t = tid / M::CA;
    float2 v[M::RA];
#pragma unroll
    for (int m = 0; m < M::RA; ++m) v[m] = land[(t + m * M::THA) * M::CA + c];
    mbar_arrive(empty_bar);                        // the landing buffer may be refilled
    dft.template run<false, 1, kMidGroup>(v, t, TileView<M::CA>{xch, c});
    const float2 b3 = cmul(w.b1, w.b2);
    float2* dst = chunk + t * M::CA + c;
    static_for<0, 4>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        float2 aq = w.w0;
        if constexpr (q & 1) aq = cmul(aq, w.l0);
        if constexpr (q & 2) aq = cmul(aq, w.l1);
        constexpr int step = M::THA * M::CA;
        st_hint(dst + (4 * q + 0) * step, cmul(v[4 * q + 0], aq), pol);
        st_hint(dst + (4 * q + 1) * step, cmul(v[4 * q + 1], cmul(aq, w.b1)), pol);
        st_hint(dst + (4 * q + 2) * step, cmul(v[4 * q + 2], cmul(aq, w.b2)), pol);
        st_hint(dst + (4 * q + 3) * step, cmul(v[4 * q + 3], cmul(aq, b3)), pol);
    });
}

// Row tile b: rows k1 = b RB + r; v[m] = row element n2 = t + m THB from the
// landing buffer (TA chunks of [RB][CA]), DFT_N2, transposed through shared
// memory and stored at X[k1 + N1 k2].
template <int LA, int LB, bool INV>
__device__ __forceinline__ void mid_rows(const float2* land, float2* xch, float2* __restrict__ y, int b, int tid,
                                         const Dft2<LB, INV>& dft, uint32_t empty_bar, int bar_id)
{
    using M = MidCfg<LA, LB>;
    static_assert(M::THB <= 32, "a row stays inside one warp");
    const int r = tid / M::THB, t = tid % M::THB;
    float2 v[M::RBV];
#pragma unroll
    for (int m = 0; m < M::RBV; ++m) {
        const int n2 = t + m * M::THB;
        v[m] = land[(n2 / M::CA) * (M::RB * M::CA) + r * M::CA + (n2 % M::CA)];
    }
    mbar_arrive(empty_bar);
    dft.template run<true, 0, 0>(v, t, PaddedView{xch + r * padded_len(M::N2)});
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

// One transform per cluster of CL CTAs at a time: CTA `rank` takes column
// tiles a = rank, rank + CL, ... and row tiles b = rank, rank + CL, ...;
// the cluster's two intermediate slots are shared.  scratch: 2 slots of n
// values per cluster, 128-byte aligned.  18 warps over the SM's four 16 K
// register partitions (at most 5 on one): at most 102 registers a thread,
// 96 in allocation units.
template <int LA, int LB, int KIND, int CL>
__global__ void __cluster_dims__(CL, 1, 1) __maxnreg__(96)
k_mid(MidIO io, long long count, float2* __restrict__ scratch, const float2* __restrict__ tw, unsigned* err)
{
    using M = MidCfg<LA, LB>;
    static_assert(M::TA % CL == 0 && M::TB % CL == 0, "tiles split evenly over the cluster");
    constexpr bool INV = KIND == 1;
    constexpr int TAC = M::TA / CL, TBC = M::TB / CL;     // tiles per CTA per transform
    extern __shared__ __align__(128) float2 smem[];
    __shared__ MidBars sb;
    float2* ringA = smem;
    float2* ringB = smem + kMidRing * kMidTile;
    float2* xchA = smem + 2 * kMidRing * kMidTile;
    float2* xchB = xchA + M::XA_AL;
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int rank = (int)(blockIdx.x % CL);
    const long long cid = blockIdx.x / CL, ncl = gridDim.x / CL;
    const long long mine = count > cid ? (count - 1 - cid) / ncl + 1 : 0;
    float2* slots = scratch + cid * 2 * M::N;
    volatile int* abort = &sb.abort;

    if (tid == 0) {
        for (int i = 0; i < kMidRing; ++i) {
            mbar_init(smem_addr(&sb.fullA[i]), 32);          // one cp.async arrival per producer lane
            mbar_init(smem_addr(&sb.fullB[i]), 1);
            mbar_init(smem_addr(&sb.emptyA[i]), kMidGroup);
            mbar_init(smem_addr(&sb.emptyB[i]), kMidGroup);
        }
        for (int s = 0; s < 2; ++s) {
            mbar_init(smem_addr(&sb.adone[s]), CL);
            mbar_init(smem_addr(&sb.bdone[s]), CL);
        }
        sb.abort = 0;
        fence_mbar_init();
    }
    // every CTA's barriers exist before any CTA of the cluster arrives on them
    if constexpr (CL > 1) cluster_sync_all();
    else __syncthreads();
    pdl_start();

    if (warp == 16) {
        // ---- producer of ring A: column tiles (N1 rows of CA values), 16-byte pieces
        const uint64_t pol_in = policy_evict_first();
        long long k = 0;
        for (long long i = 0; i < mine && !*abort; ++i) {
            const float2* x = io.src(cid + i * ncl);
            for (int j = 0; j < TAC; ++j, ++k) {
                const int a = rank + CL * j;
                const int buf = (int)(k % kMidRing);
                const bool ok = k < kMidRing || mid_wait(smem_addr(&sb.emptyA[buf]), (uint32_t)((k / kMidRing - 1) & 1), err, abort);
                if (!__all_sync(0xffffffffu, ok)) break;
                const uint32_t full = smem_addr(&sb.fullA[buf]);
                const uint32_t dst = smem_addr(ringA + buf * kMidTile);
                constexpr int PPR = (int)(M::SEG_A / 16);     // pieces per row
#pragma unroll 4
                for (int p = lane; p < M::N1 * PPR; p += 32) {
                    const int n1 = p / PPR, q = p % PPR;
                    cp_async16(dst + n1 * M::SEG_A + 16 * q,
                               (const char*)(x + (long long)n1 * M::N2 + a * M::CA) + 16 * q, pol_in);
                }
                cp_async_arrive(full);
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
            if (!__all_sync(0xffffffffu, mid_wait_cluster(smem_addr(&sb.adone[s]), (uint32_t)((i >> 1) & 1), err, abort)))
                break;
            fence_proxy_async_global();
            const float2* slot = slots + s * M::N;
            for (int j = 0; j < TBC; ++j, ++k) {
                const int b = rank + CL * j;
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
        const uint64_t pol_mid = policy_evict_last();
        Dft2<LA, INV> dft;
        dft.load(g / M::CA, tw);
        ColTw cur = col_twiddles<LA, LB, INV>(rank, g, tw);
        long long k = 0;
        for (long long i = 0; i < mine; ++i) {
            const int s = (int)(i & 1);
            // the slot's previous transform (i - 2) must have been copied out by every CTA
            if (!group_all(i < 2 || mid_wait_cluster(smem_addr(&sb.bdone[s]), (uint32_t)(((i - 2) >> 1) & 1), err, abort), 1))
                break;
            float2* slot = slots + s * M::N;
            bool ok = true;
            for (int j = 0; j < TAC; ++j, ++k) {
                const int a = rank + CL * j;
                // the next tile's column twiddles (tiles cycle through the same columns)
                const ColTw nxt = col_twiddles<LA, LB, INV>(j + 1 < TAC ? a + CL : rank, g, tw);
                const int buf = (int)(k % kMidRing);
                if (!group_all(mid_wait(smem_addr(&sb.fullA[buf]), (uint32_t)((k / kMidRing) & 1), err, abort), 1)) {
                    ok = false;
                    break;
                }
                mid_cols<LA, LB, INV>(ringA + buf * kMidTile, xchA, slot + (long long)a * kMidTile, g, dft, cur,
                                      smem_addr(&sb.emptyA[buf]), pol_mid);
                cur = nxt;
            }
            if (!ok) break;
            fence_proxy_async_global();            // the stores above are read next by bulk copies
            group_sync(1);
            if (g < CL) mbar_arrive_cluster(smem_addr(&sb.adone[s]), g);
        }
    } else {
        // ---- group B: row tiles of transform i, results to the output
        const int g = tid - kMidGroup;
        Dft2<LB, INV> dft;
        dft.load(g % M::THB, tw);
        long long k = 0;
        for (long long i = 0; i < mine; ++i) {
            const int s = (int)(i & 1);
            float2* y = io.dst(cid + i * ncl);
            const float2* slot = slots + s * M::N;
            bool ok = true;
            for (int j = 0; j < TBC; ++j, ++k) {
                const int b = rank + CL * j;
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
                mid_rows<LA, LB, INV>(ringB + buf * kMidTile, xchB, y, b, g, dft, smem_addr(&sb.emptyB[buf]), 2);
            }
            if (!ok) break;
            // every copy out of slot s by this CTA has landed and its lines
            // were dropped (mid_rows ends with a group barrier)
            if (g < CL) mbar_arrive_cluster(smem_addr(&sb.bdone[s]), g);
        }
    }
    // no CTA leaves while another may still arrive on its barriers
    if constexpr (CL > 1) {
        __syncwarp();
        cluster_sync_all();
    }
}

template <int LA, int LB, int KIND, int CL>
static cudaError_t attr_mid()
{
    cudaError_t e = cudaFuncSetAttribute(k_mid<LA, LB, KIND, CL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)MidCfg<LA, LB>::SMEM);
    if (e == cudaSuccess && CL > 1)
        e = cudaFuncSetAttribute(k_mid<LA, LB, KIND, CL>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return e;
}

// Clusters of CL CTAs resident at once (one CTA per SM).
template <int LA, int LB, int CL>
static long long mid_clusters()
{
    static long long n = 0;
    if (!n) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(CL * 1024);
        cfg.blockDim = dim3(kMidThreads);
        cfg.dynamicSmemBytes = MidCfg<LA, LB>::SMEM;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = CL;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int c = 0;
        if (cudaOccupancyMaxActiveClusters(&c, k_mid<LA, LB, 0, CL>, &cfg) != cudaSuccess || c < 1) {
            cudaGetLastError();
            c = 1;
        }
        n = c;
    }
    return n;
}

// Cluster size per size: complex 2^16 shares each transform between two SMs,
// which halves the intermediate each SM keeps in L2 (one SM per transform
// measured 3179 GB/s with the intermediate spilling to HBM, two 3429).
static int mid_cl(int log2n) { return log2n == 16 ? 2 : 1; }

bool mid_supported(int log2n) { return log2n == 15 || log2n == 16; }

static long long mid_nclusters(int log2n, long long count)
{
    const long long c = log2n == 15 ? mid_clusters<7, 8, 1>() : mid_clusters<8, 8, 2>();
    return count < c ? count : c;
}

size_t mid_scratch_bytes(int log2n, long long count)
{
    return (size_t)mid_nclusters(log2n, count) * 2 * sizeof(float2) * ((size_t)1 << log2n);
}

template <int LA, int LB, int CL>
static cudaError_t launch_mid_CL(int kind, const MidIO& io, long long count, const float2* tw, float2* scratch,
                                 long long ncl, cudaStream_t s)
{
    using M = MidCfg<LA, LB>;
    const dim3 grid((unsigned)(ncl * CL));
    unsigned* err = device_error_word();
    return kind == 0
        ? launch_pdl(k_mid<LA, LB, 0, CL>, grid, dim3(kMidThreads), M::SMEM, s, io, count, scratch, tw, err)
        : launch_pdl(k_mid<LA, LB, 1, CL>, grid, dim3(kMidThreads), M::SMEM, s, io, count, scratch, tw, err);
}

// Contiguous batch; in 16-byte aligned and in_dist a multiple of 2 values.
cudaError_t launch_mid(int kind, int log2n, const void* in, void* out, long long count, long long in_dist,
                       long long out_dist, const float2* tw, void* scratch, size_t scratch_bytes, cudaStream_t s)
{
    if (!mid_supported(log2n) || (kind != 0 && kind != 1)) return cudaErrorInvalidValue;
    if (count <= 0) return cudaSuccess;
    if (((uintptr_t)in & 15) || (in_dist & 1)) return cudaErrorInvalidValue;
    if (scratch_bytes < mid_scratch_bytes(log2n, count) || ((uintptr_t)scratch & 127)) return cudaErrorInvalidValue;
    const MidIO io{(const float2*)in, (float2*)out, in_dist, out_dist};
    const long long ncl = mid_nclusters(log2n, count);
    cudaError_t e = log2n == 15 ? launch_mid_CL<7, 8, 1>(kind, io, count, tw, (float2*)scratch, ncl, s)
                                : launch_mid_CL<8, 8, 2>(kind, io, count, tw, (float2*)scratch, ncl, s);
    if (e == cudaSuccess) count_launch();
    return e;
}

cudaError_t prepare_mid()
{
    cudaError_t e = attr_mid<7, 8, 0, 1>();
    if (e == cudaSuccess) e = attr_mid<7, 8, 1, 1>();
    if (e == cudaSuccess) e = attr_mid<8, 8, 0, 2>();
    if (e == cudaSuccess) e = attr_mid<8, 8, 1, 2>();
    return e;
}

}  // namespace ckg
