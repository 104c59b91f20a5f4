// fft_passes.cuh -- the two passes of the multi-pass transform as device
// functions (used by the batched kernels in fft_large.cu and by the persistent
// job kernel in fft_jobs.cu).
//
// N = N1 * N2, x[n] viewed as N1 rows of N2 columns (n = N2*n1 + n2):
//   columns: for each column n2, Y[k1] = DFT_N1 over n1 of x[N2*n1 + n2], times
//            W_N^(n2*k1), stored at scratch[N2*k1 + n2];
//   rows:    for each row k1, DFT_N2 over n2, X[k1 + N1*k2] stored transposed
//            through shared memory.
// A tile is C adjacent columns (or rows), so each warp access covers C*8
// contiguous bytes.  CG selects L2-only loads (ld.global.cg) for data that
// another CTA wrote earlier in the same launch.
#pragma once
#include <cstdint>

#include "fft_core.cuh"

namespace ckg {

// Shape of a sub-transform of 2^LS points inside a pass: R values per thread,
// C sequences per tile.
// MAXT: thread budget of the CTA (or CTA subgroup) running the tile.  With
// 512 threads, sub-lengths above 2^10 take 32 values per thread (128
// registers); with 1024 threads they keep 16 values (64 registers) and twice
// the resident warps.
// CMAX: widest tile (C * 8 bytes per row access).
template <int LS, int MAXT = 512, int CMAX = 16>
struct PassCfg {
    static constexpr int LOG2R = LS < 4 ? LS : (LS <= 10 || MAXT >= 1024) ? 4 : 5;
    static constexpr int R = 1 << LOG2R;
    static constexpr int T = (1 << LS) / R;
    static constexpr int C = MAXT / T < CMAX ? MAXT / T : CMAX;
    static constexpr int THREADS = C * T;
    // interleaved (pass 1 and pass-2 transpose) and per-row padded (pass 2) layouts
    static constexpr int INTERLEAVED = (1 << LS) * C + ((1 << LS) * C >> 4) + 1;
    static constexpr int BLOCKED = C * padded_len(1 << LS);
    static constexpr int SLOTS = INTERLEAVED > BLOCKED ? INTERLEAVED : BLOCKED;
    static constexpr size_t SMEM = sizeof(float2) * (size_t)SLOTS;
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

template <bool CG>
__device__ __forceinline__ float2 ld_data(const float2* p)
{
    if constexpr (CG) return __ldcg(p);
    else return __ldcs(p);
}

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

// Tail of the column pass: v[m] = Y[k1] of column n2 at k1 = t + m T,
// multiplied by W_N^(n2 k1) and stored at out[N2 k1 + n2].
template <int LA, bool INV, int MAXT, int CMAX>
__device__ __forceinline__ void cols_twiddle_store(float2 (&v)[PassCfg<LA, MAXT, CMAX>::R], float2* __restrict__ out,
                                                   int log2n2, long long n2, int t, const float2* __restrict__ tw,
                                                   bool live)
{
    using P = PassCfg<LA, MAXT, CMAX>;
    const long long n2len = 1ll << log2n2;
    const int ln = LA + log2n2;
    float2* dst = out + n2 + (long long)t * n2len;
    const long long step = (long long)P::T * n2len;
    // W_N^(n2 k1) for k1 = t + m T, m = 4q + r:  W^(n2 t) * W^(4 n2 T q) * W^(n2 T r).
    // 3 + log2(R/4) table lookups per thread instead of R; each twiddle is a
    // product of at most 2 + log2(R/4) rounded factors.
    const int mask = (1 << ln) - 1;
    const int p0 = (int)n2 * t, pT = ((int)n2 * P::T) & mask;
    const float2 a = big_twiddle<INV>(tw, ln, p0 & mask);
    const float2 b1 = big_twiddle<INV>(tw, ln, pT), b2 = big_twiddle<INV>(tw, ln, (2 * pT) & mask);
    const float2 b3 = cmul(b1, b2);
    constexpr int Q = P::R / 4;
    float2 ladder[Q > 1 ? ilog2(Q) : 1];
#pragma unroll
    for (int i = 0; (1 << i) < Q; ++i) ladder[i] = big_twiddle<INV>(tw, ln, (int)(((long long)pT << (2 + i)) & mask));
    if (!live) return;
    static_for<0, Q>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        float2 aq = a;
        static_for<0, (Q > 1 ? ilog2(Q) : 0)>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            if constexpr ((q >> i) & 1) aq = cmul(aq, ladder[i]);
        });
        __stcs(dst + (4 * q + 0) * step, cmul(v[4 * q + 0], aq));
        __stcs(dst + (4 * q + 1) * step, cmul(v[4 * q + 1], cmul(aq, b1)));
        __stcs(dst + (4 * q + 2) * step, cmul(v[4 * q + 2], cmul(aq, b2)));
        __stcs(dst + (4 * q + 3) * step, cmul(v[4 * q + 3], cmul(aq, b3)));
    });
}

// Column pass for tile `tile` of one transform, by threads tid = 0..THREADS-1.
// live == false: the threads take part in the barriers only (no memory
// access outside the tile's shared memory).
template <int LA, bool INV, bool CG, int MAXT = 512, int CMAX = 16>
__device__ __forceinline__ void pass_cols(const float2* __restrict__ in, float2* __restrict__ out, int log2n2,
                                          long long tile, int tid, float2* smem, const float2* __restrict__ tw,
                                          bool live = true)
{
    using P = PassCfg<LA, MAXT, CMAX>;
    const int c = tid % P::C, t = tid / P::C;
    const long long n2len = 1ll << log2n2;
    const long long n2 = tile * P::C + c;
    const float2* src = in + n2;
    float2 v[P::R];
#pragma unroll
    for (int m = 0; m < P::R; ++m)
        v[m] = live ? ld_data<CG>(src + (long long)(t + m * P::T) * n2len) : make_float2(0.f, 0.f);
    TileView<P::C> view{smem, c};
    stockham<LA, P::LOG2R, INV, false>(v, t, tw, view);
    cols_twiddle_store<LA, INV, MAXT, CMAX>(v, out, log2n2, n2, t, tw, live);
}

// Column pass of a real inverse transform with the merge fused (M = N1 N2
// complex values from the M+1 input bins X): tile u holds columns
// n2 = u C/2 + j and their mirrors N2 - n2 (j < C/2; tile 0 holds column
// N2/2 in place of the mirror of column 0), so for every element
// k = N2 n1 + n2 its partner M - k = N2 (N1 - 1 - n1) + (N2 - n2) is in the
// same tile (column 0 pairs with itself at row N1 - n1, and with X[M] at
// row 0).  The tile's raw bins are staged in shared memory and merged into
// registers (the algebra of merge_elem) before the column DFTs: no merge
// pass over HBM.  CG: L2-only loads, as in pass_cols.
template <int LA, int MAXT = 512, int CMAX = 16, bool CG = false>
__device__ __forceinline__ void pass_cols_merge(const float2* __restrict__ in, float2* __restrict__ out, int log2n2,
                                                long long tile, int tid, float2* smem, const float2* __restrict__ tw)
{
    using P = PassCfg<LA, MAXT, CMAX>;
    constexpr int N1 = 1 << LA, H = P::C / 2;
    static_assert(P::C >= 2 && P::C % 2 == 0, "tiles of column pairs");
    const int c = tid % P::C, t = tid / P::C;
    const int n2len = 1 << log2n2;
    const long long M = (long long)N1 << log2n2;
    const float2* twn = tw + 2 * M;
    const int u = (int)tile;
    // column of tile slot `slot`
    auto col = [&](int slot) {
        if (slot < H) return u * H + slot;
        return (u == 0 && slot == H) ? n2len / 2 : n2len - (u * H + (slot - H));
    };
    const int n2 = col(c);
#pragma unroll
    for (int m = 0; m < P::R; ++m) {
        const int n1 = t + m * P::T;
        smem[TileView<P::C>::slot(n1, c)] = ld_data<CG>(in + (long long)n1 * n2len + n2);
    }
    const float2 xm = (u == 0 && tid == 0) ? ld_data<CG>(in + M) : make_float2(0.f, 0.f);   // X[M]
    __syncthreads();
    // Each thread merges its own elements k = N2 n1 + n2 (rows n1 = t + mT of
    // column n2) into registers, reading the partner X[M - k] from the
    // staged tile: row N1 - 1 - n1 of the mirror column (column 0: row
    // N1 - n1, and X[M] at row 0).  Twiddle W_2M^k = W_2N1^n1 * W_2M^n2: a
    // row factor from the short 2N1 level of the table, one column factor
    // per thread.
    const bool edge = u == 0 && (c == 0 || c == H);       // columns 0 and N2/2 mirror themselves
    const int mc = edge ? c : (c < H ? c + H : c - H);     // slot of the mirror column
    const float2* twr = tw + 2 * N1;                       // W_2N1^n1
    const float2 wcol = __ldg(twn + n2);
    float2 v[P::R];
#pragma unroll
    for (int m = 0; m < P::R; ++m) {
        const int n1 = t + m * P::T;
        const float2 a = smem[TileView<P::C>::slot(n1, c)];
        float2 b;
        if (u == 0 && c == 0) b = n1 == 0 ? xm : smem[TileView<P::C>::slot(N1 - n1, 0)];
        else b = smem[TileView<P::C>::slot(N1 - 1 - n1, mc)];
        v[m] = real_merge(a, b, cmul(__ldg(twr + n1), wcol));
    }
    __syncthreads();
    TileView<P::C> view{smem, c};
    stockham<LA, P::LOG2R, true, false>(v, t, tw, view);
    cols_twiddle_store<LA, true, MAXT, CMAX>(v, out, log2n2, n2, t, tw, true);
}

// Row pass for tile `tile` (rows tile*C .. tile*C+C-1) of one transform.
// DISCARD: the input is a dead intermediate (scratch) whose L2 lines may be
// dropped without write-back once read; it must be 128-byte aligned.
// log2_row_stride: distance between consecutive rows of the input (default:
// the row length, rows back to back).
// STREAM: outputs stored with the evict-first hint (false: they are read
// again soon, by a later phase of the same kernel).
template <int LB, bool INV, bool CG, int MAXT = 512, bool DISCARD = true, bool STREAM = true, int CMAX = 16>
__device__ __forceinline__ void pass_rows(const float2* __restrict__ in, float2* __restrict__ out, int log2n1,
                                          long long tile, int tid, float2* smem, const float2* __restrict__ tw,
                                          bool live = true, int log2_row_stride = LB)
{
    using P = PassCfg<LB, MAXT, CMAX>;
    constexpr int N2 = 1 << LB;
    const int r = tid / P::T, t = tid % P::T;
    const long long n1len = 1ll << log2n1;
    const long long row0 = tile * P::C;
    const long long rstride = 1ll << log2_row_stride;
    const float2* src = in + (row0 + r) * rstride + t;
    float2 v[P::R];
#pragma unroll
    for (int m = 0; m < P::R; ++m) v[m] = live ? ld_data<CG>(src + m * P::T) : make_float2(0.f, 0.f);
    PaddedView view{smem + r * padded_len(N2)};
    stockham<LB, P::LOG2R, INV, (P::T <= 32)>(v, t, tw, view);
    __syncthreads();
    if (DISCARD && live) {
        // every thread of the tile has consumed its inputs: the intermediate
        // rows are dead, so drop their L2 lines instead of writing them back
        static_assert(N2 % 16 == 0, "rows span whole 128-byte lines");
        const char* row = (const char*)(in + (row0 + r) * rstride);
#pragma unroll
        for (int l = t; l < N2 / 16; l += P::T)
            asm volatile("discard.global.L2 [%0], 128;" ::"l"(row + 128 * l) : "memory");
    }
    // transpose through shared memory so that stores run along rows k1
#pragma unroll
    for (int m = 0; m < P::R; ++m) smem[TileView<P::C>::slot(t + m * P::T, r)] = v[m];
    __syncthreads();
    if (!live) return;
    if constexpr (STREAM && P::C % 2 == 0) {
        if (((uintptr_t)out & 15) == 0) {
            // two adjacent rows per thread, one 16-byte store each: half the
            // store instructions (out 16-byte aligned; row0 and r2 even)
            constexpr int H = P::C / 2, T2 = P::THREADS / H;
            const int r2 = 2 * (tid % H), t2 = tid / H;
            float4* dst4 = reinterpret_cast<float4*>(out + row0 + r2);
#pragma unroll
            for (int m = 0; m < (1 << LB) / T2; ++m) {
                const int k2 = t2 + m * T2;
                const float2 a = smem[TileView<P::C>::slot(k2, r2)], b = smem[TileView<P::C>::slot(k2, r2 + 1)];
                __stcs(dst4 + (long long)k2 * (n1len / 2), make_float4(a.x, a.y, b.x, b.y));
            }
            return;
        }
    }
    const int r2 = tid % P::C, t2 = tid / P::C;
    float2* dst = out + row0 + r2;
#pragma unroll
    for (int m = 0; m < P::R; ++m) {
        const int k2 = t2 + m * P::T;
        if constexpr (STREAM) __stcs(dst + (long long)k2 * n1len, smem[TileView<P::C>::slot(k2, r2)]);
        else dst[(long long)k2 * n1len] = smem[TileView<P::C>::slot(k2, r2)];
    }
}

// Row pass with the output transpose folded into the last stage exchange.
// All stages but the last run on thread (r, t) = (tid / T, tid mod T): row
// r's positions t + mT, coalesced row loads, exchanges inside the row as in
// pass_rows.  The second-to-last stage writes its outputs to the row's
// padded shared-memory image; the last stage then runs on thread
// (r, t) = (tid mod C, tid / C), so the C lanes of one t hold rows row0 ..
// row0 + C - 1 and each output store covers C consecutive bins k1 of one
// k2.  One shared-memory round trip per value fewer than pass_rows
// (exchange inside the row, then a transpose).  Row images are
// padded_len(N2) slots apart, an odd number: the last stage's reads across
// 16 rows fall in distinct 8-byte banks.
// DISCARD / CG / log2_row_stride as in pass_rows; outputs are stored with
// the evict-first hint.
template <int LB, bool INV, bool CG, int MAXT = 512, bool DISCARD = true, int CMAX = 16>
__device__ __forceinline__ void pass_rows_xt(const float2* __restrict__ in, float2* __restrict__ out, int log2n1,
                                             long long tile, int tid, float2* smem, const float2* __restrict__ tw,
                                             int log2_row_stride = LB)
{
    using P = PassCfg<LB, MAXT, CMAX>;
    using S = Sched<LB, P::LOG2R>;
    constexpr int N2 = 1 << LB, R = P::R, T = P::T, LR = P::LOG2R, NST = S::nstages;
    constexpr int RSTRIDE = padded_len(N2);
    static_assert(NST >= 2, "at least two stages");
    static_assert(RSTRIDE % 2 == 1 && P::C * RSTRIDE <= P::SLOTS, "odd row stride inside the tile's memory");
    const long long n1len = 1ll << log2n1;
    const long long row0 = tile * P::C;
    const long long rstride = 1ll << log2_row_stride;
    float2 v[R];
    {
        const int r = tid / T, t = tid % T;
        const float2* src = in + (row0 + r) * rstride + t;
#pragma unroll
        for (int m = 0; m < R; ++m) v[m] = ld_data<CG>(src + m * T);
        PaddedView view{smem + r * RSTRIDE};
        static_for<0, NST - 1>([&](auto sc) {
            constexpr int st = decltype(sc)::value;
            stage_compute<LB, LR, S::lrs(st), S::lns(st), INV>(v, t, tw);
            if constexpr (st + 2 < NST) stage_exchange<LB, LR, S::lrs(st), S::lns(st), (T <= 32)>(v, t, view);
            else stage_write<LB, LR, S::lrs(st), S::lns(st)>(v, t, view);
        });
    }
    __syncthreads();
    if constexpr (DISCARD) {
        // every thread of the tile has consumed its inputs: the intermediate
        // rows are dead, so drop their L2 lines instead of writing them back
        static_assert(N2 % 16 == 0, "rows span whole 128-byte lines");
        constexpr int LINES = N2 / 16;
#pragma unroll
        for (int l = tid; l < P::C * LINES; l += P::THREADS) {
            const char* row = (const char*)(in + (row0 + l / LINES) * rstride);
            asm volatile("discard.global.L2 [%0], 128;" ::"l"(row + 128 * (l % LINES)) : "memory");
        }
    }
    const int r = tid % P::C, t = tid / P::C;
    stage_read<LB, LR>(v, t, PaddedView{smem + r * RSTRIDE});
    constexpr int LRS = S::lrs(NST - 1), LNS = S::lns(NST - 1);
    stage_compute<LB, LR, LRS, LNS, INV>(v, t, tw);
    // v[u + j U] = X[t + u T + j NS] of row row0 + r (the last stage's span
    // NS = N2 / RS; 32-bit offsets: the transform has fewer than 2^31 values)
    constexpr int U = R >> LRS, NS = 1 << LNS;
    float2* dst = out + row0 + r + t * (int)n1len;
#pragma unroll
    for (int u = 0; u < U; ++u) {
#pragma unroll
        for (int j = 0; j < (1 << LRS); ++j) __stcs(dst + (u * T + j * NS) * (int)n1len, v[u + j * U]);
    }
}

// Row pass of a real forward transform with the split fused (half-length
// spectrum of M = N1 N2 values, x2 scaling of the reference): tile u holds
// rows k1 = u C/2 + j and their mirrors N1 - k1 (j < C/2; tile 0 holds row
// N1/2 in place of the mirror of row 0), so both members of every output
// pair (k, M - k) -- k = k1 + N1 k2, M - k = (N1 - k1) + N1 (N2 - 1 - k2) --
// are in one CTA.  After the row DFTs the tile's half-length spectrum stays
// in shared memory and the CTA writes the bins X[k], X[M-k] (M+1 bins per
// transform) directly: no split pass over HBM.  Same algebra as
// split_pair_inplace, with the twiddles factored (see below).
// The third pass of the three-pass transform is the same pass over
// N1 = N1' N2' rows: row k1' + N1' k2' sits at in[k1' N2' N3 + k2' N3] (the
// intermediate of the second pass); log2k1 = log2 N1' selects that address
// form (log2k1 = log2n1: rows back to back).  CG: L2-only loads, as in
// pass_rows.
template <int LB, int MAXT = 512, bool CG = false>
__device__ __forceinline__ void pass_rows_split(const float2* __restrict__ in, float2* __restrict__ out,
                                                int log2n1, long long tile, int tid, float2* smem,
                                                const float2* __restrict__ tw, int log2k1)
{
    using P = PassCfg<LB, MAXT>;
    constexpr int N2 = 1 << LB, H = P::C / 2;
    static_assert(P::C >= 2 && P::C % 2 == 0, "tiles of row pairs");
    const int n1 = 1 << log2n1;
    const long long M = (long long)n1 << LB;
    const float2* twn = tw + 2 * M;
    const int u = (int)tile;
    const int r = tid / P::T, t = tid % P::T;
    // this thread's row
    int k1;
    if (r < H) k1 = u * H + r;
    else k1 = (u == 0 && r == H) ? n1 / 2 : n1 - (u * H + (r - H));
    const float2* rowp = in + ((long long)(k1 & ((1 << log2k1) - 1)) << (log2n1 - log2k1 + LB)) +
                         ((long long)(k1 >> log2k1) << LB);
    float2 v[P::R];
#pragma unroll
    for (int m = 0; m < P::R; ++m) v[m] = ld_data<CG>(rowp + t + m * P::T);
    PaddedView view{smem + r * padded_len(N2)};
    stockham<LB, P::LOG2R, false, (P::T <= 32)>(v, t, tw, view);
    __syncthreads();
    {
        // every thread has consumed its inputs: the intermediate rows are
        // dead, so drop their L2 lines instead of writing them back
        static_assert(N2 % 16 == 0, "rows span whole 128-byte lines");
        const char* row = (const char*)rowp;
#pragma unroll
        for (int l = t; l < N2 / 16; l += P::T)
            asm volatile("discard.global.L2 [%0], 128;" ::"l"(row + 128 * l) : "memory");
    }
#pragma unroll
    for (int m = 0; m < P::R; ++m) view.st(t + m * P::T, v[m]);
    __syncthreads();
    auto z = [&](int slot, int k2) { return smem[slot * padded_len(N2) + PaddedView::pad(k2)]; };
    // H pairs x N2 columns, H consecutive pairs per column; p = tid mod H
    // for every item of a thread.  Twiddles: W_2M^k = W_2N2^k2 * W_2M^A
    // (k = A + N1 k2) -- a factor from the short 2N2 level of the table and
    // one row factor per thread -- and W_2M^(M-k) = -conj(W_2M^k).
    const float2* twc = tw + 2 * N2;                                  // W_2N2^k2
    const int pt = tid % H;
    const bool edge = u == 0 && pt == 0;
    const float2 wrow = __ldg(twn + (edge ? n1 / 2 : u * H + pt));     // row factor
#pragma unroll
    for (int q = 0; q < P::R / 2; ++q) {
        const int i = tid + q * P::THREADS;
        const int k2 = i / H;
        if (edge) {
            // row 0 pairs (k2, N2 - k2) and row N1/2 pairs (j, N2 - 1 - j)
            if (k2 <= N2 / 2) {
                const long long k = (long long)n1 * k2;
                const float2 w = __ldg(twc + k2);                     // row 0: W_2M^(N1 k2)
                const float2 a = z(0, k2), b = z(0, (N2 - k2) & (N2 - 1));
                out[k] = real_split(a, b, w);
                if (k2 != N2 / 2) out[M - k] = real_split(b, a, make_float2(-w.x, w.y));
            }
            const int j = k2 > N2 / 2 ? k2 - N2 / 2 - 1 : (k2 == 0 ? N2 / 2 - 1 : -1);
            if (j >= 0) {
                const long long k = n1 / 2 + (long long)n1 * j;
                const float2 w = cmul(__ldg(twc + j), wrow);          // row N1/2
                const float2 a = z(H, j), b = z(H, N2 - 1 - j);
                out[k] = real_split(a, b, w);
                out[M - k] = real_split(b, a, make_float2(-w.x, w.y));
            }
        } else {
            const long long k = u * H + pt + (long long)n1 * k2;
            const float2 w = cmul(__ldg(twc + k2), wrow);
            const float2 a = z(pt, k2), b = z(H + pt, N2 - 1 - k2);
            out[k] = real_split(a, b, w);
            out[M - k] = real_split(b, a, make_float2(-w.x, w.y));
        }
    }
}

// Real forward split, in place: pair k in [0, M/2] of a natural-order
// half-length spectrum z (room for M+1 values) becomes output bins k and M-k
// (k = 0 gives bins 0 and M; k = M/2 the middle bin).
template <bool CG>
__device__ __forceinline__ void split_pair_inplace(float2* __restrict__ z, long long M, long long k,
                                                   const float2* __restrict__ twn)
{
    if (k == 0) {
        const float2 z0 = ld_data<CG>(z);
        z[0] = real_split(z0, z0, __ldg(twn));
        z[M] = real_split(z0, z0, __ldg(twn + M));
    } else if (k == M / 2) {
        const float2 zk = ld_data<CG>(z + k);
        z[k] = real_split(zk, zk, __ldg(twn + k));
    } else {
        const float2 a = ld_data<CG>(z + k), b = ld_data<CG>(z + (M - k));
        z[k] = real_split(a, b, __ldg(twn + k));
        z[M - k] = real_split(b, a, __ldg(twn + (M - k)));
    }
}

// Real inverse merge of element k < M: y[k] from x[k] and x[M-k].
template <bool CG>
__device__ __forceinline__ void merge_elem(const float2* __restrict__ x, float2* __restrict__ y, long long M,
                                           long long k, const float2* __restrict__ twn)
{
    y[k] = real_merge(ld_data<CG>(x + k), ld_data<CG>(x + (M - k)), __ldg(twn + k));
}

}  // namespace ckg
