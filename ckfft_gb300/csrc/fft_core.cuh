// fft_core.cuh -- device building blocks for the sm_103a FFT kernels.
//
// Replaces the reference's arithmetic layer (src/ckfft/math_util.h:17-33) and
// its radix-4 DIT recursion (src/ckfft/fft_default.cpp:12-266) with a
// register-resident, self-sorting (Stockham) formulation:
//
//   * each thread holds R = 2^r complex values in registers; a length-N
//     sequence is owned by T = N/R threads, thread t holding elements
//     t, t+T, t+2T, ... (so global loads and stores are coalesced over t);
//   * a stage of radix RS with span NS (product of the radices already
//     applied) takes butterfly b's inputs b + j*N/RS, multiplies input j by
//     W_{NS*RS}^{j*(b mod NS)}, runs an in-register DFT_RS and sends output j
//     to (b/NS)*NS*RS + (b mod NS) + j*NS;
//   * stages exchange data through shared memory; after the final stage
//     thread t again holds elements t + m*T, now of the natural-order
//     spectrum, so no bit-reversal pass exists anywhere.
//
// Twiddles come from a device table laid out by level: W_{2^q}^m is at
// tw[2^q + m] for 0 <= m < 2^q.  The table is generated in FP64 on the host
// and rounded once to FP32 (see twiddle.cpp); the inverse uses conjugates.
#pragma once
#include <cuda_runtime.h>
#include <type_traits>
#include <utility>

namespace ckg {

// ------------------------------------------------------------------ helpers

template <int I, int N, class F>
__device__ __forceinline__ void static_for(F&& f)
{
    if constexpr (I < N) {
        f(std::integral_constant<int, I>{});
        static_for<I + 1, N>(f);
    }
}

__host__ __device__ constexpr int ilog2(int x) { return x <= 1 ? 0 : 1 + ilog2(x >> 1); }

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 w)
{
    return make_float2(fmaf(a.x, w.x, -a.y * w.y), fmaf(a.x, w.y, a.y * w.x));
}
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

// cos(2*pi*m/32) for m = 0..8; other angles by symmetry.
__host__ __device__ constexpr double cos32_q(int m)
{
    return m == 0 ? 1.0
         : m == 1 ? 0.98078528040323044912618223613424
         : m == 2 ? 0.92387953251128675612818318939679
         : m == 3 ? 0.83146961230254523707878837761791
         : m == 4 ? 0.70710678118654752440084436210485
         : m == 5 ? 0.55557023301960222474283081394853
         : m == 6 ? 0.38268343236508977172845998403040
         : m == 7 ? 0.19509032201612826784828486847702
         : 0.0;
}
__host__ __device__ constexpr double cos32(int m)
{
    m = ((m % 32) + 32) % 32;
    if (m > 16) m = 32 - m;            // cos(2pi - x) = cos x
    return m > 8 ? -cos32_q(16 - m) : cos32_q(m);
}
__host__ __device__ constexpr double sin32(int m) { return cos32(8 - m); }

// a * W_R^K with W_R = exp(-2 pi i / R) (forward) or exp(+2 pi i / R) (inverse);
// K and R are compile-time, R divides 32.
template <int R, int K, bool INV>
__device__ __forceinline__ float2 rot(float2 a)
{
    constexpr int m = ((K * (32 / R)) % 32 + 32) % 32;
    if constexpr (m == 0) {
        return a;
    } else if constexpr (m == 16) {
        return make_float2(-a.x, -a.y);
    } else if constexpr (m == 8) {          // forward: * -i, inverse: * +i
        return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
    } else if constexpr (m == 24) {         // forward: * +i, inverse: * -i
        return INV ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
    } else if constexpr (m % 8 == 4) {      // odd multiples of 45 degrees
        constexpr float c = (float)cos32(m);
        constexpr float s = INV ? (float)sin32(m) : -(float)sin32(m);
        constexpr float sg = (s > 0.f) == (c > 0.f) ? 1.f : -1.f;    // s = sg * c
        return make_float2(c * (a.x - sg * a.y), c * (sg * a.x + a.y));
    } else {
        constexpr float c = (float)cos32(m);
        constexpr float s = INV ? (float)sin32(m) : -(float)sin32(m);
        return make_float2(fmaf(a.x, c, -a.y * s), fmaf(a.x, s, a.y * c));
    }
}

// ------------------------------------------------------- in-register DFTs

template <int R, bool INV> __device__ __forceinline__ void dft(float2 (&v)[R]);

// Cooley-Tukey split R = P*Q on registers: n = Q*n1 + n2, k = k1 + P*k2.
template <int R, int P, bool INV>
__device__ __forceinline__ void dft_ct(float2 (&v)[R])
{
    constexpr int Q = R / P;
    static_for<0, Q>([&](auto n2c) {
        constexpr int n2 = decltype(n2c)::value;
        float2 t[P];
#pragma unroll
        for (int n1 = 0; n1 < P; ++n1) t[n1] = v[Q * n1 + n2];
        dft<P, INV>(t);
        static_for<0, P>([&](auto k1c) {
            constexpr int k1 = decltype(k1c)::value;
            v[Q * k1 + n2] = rot<R, n2 * k1, INV>(t[k1]);
        });
    });
    float2 o[R];
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) {
        float2 t[Q];
#pragma unroll
        for (int n2 = 0; n2 < Q; ++n2) t[n2] = v[Q * k1 + n2];
        dft<Q, INV>(t);
#pragma unroll
        for (int k2 = 0; k2 < Q; ++k2) o[k1 + P * k2] = t[k2];
    }
#pragma unroll
    for (int k = 0; k < R; ++k) v[k] = o[k];
}

template <int R, bool INV>
__device__ __forceinline__ void dft(float2 (&v)[R])
{
    if constexpr (R == 1) {
        (void)v;
    } else if constexpr (R == 2) {
        float2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    } else if constexpr (R == 4) {
        float2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
        float2 a2 = cadd(v[1], v[3]), a3 = csub(v[1], v[3]);
        v[0] = cadd(a0, a2);
        v[2] = csub(a0, a2);
        if (INV) {
            v[1] = make_float2(a1.x - a3.y, a1.y + a3.x);
            v[3] = make_float2(a1.x + a3.y, a1.y - a3.x);
        } else {
            v[1] = make_float2(a1.x + a3.y, a1.y - a3.x);
            v[3] = make_float2(a1.x - a3.y, a1.y + a3.x);
        }
    } else if constexpr (R == 8) {
        dft_ct<8, 2, INV>(v);
    } else if constexpr (R == 16) {
        dft_ct<16, 4, INV>(v);
    } else if constexpr (R == 32) {
        dft_ct<32, 2, INV>(v);
    } else {
        static_assert(R <= 32, "radix above 32 is not used");
    }
}

// ------------------------------------------------------------ twiddles

template <bool INV>
__device__ __forceinline__ float2 tw_load(const float2* __restrict__ lvl, int idx)
{
    float2 w = __ldg(lvl + idx);
    return INV ? conjf2(w) : w;
}

// ------------------------------------------------------ shared exchange

// Shared-memory views used between stages.  `pos` is a position in the
// natural-order sequence of one transform.
//
// Padded: one transform per contiguous region, one spare slot every 16
// elements so that stride-RS butterfly writes fall in distinct 8-byte banks.
struct PaddedView {
    static constexpr bool kPadded = true;
    float2* base;
    __device__ __forceinline__ static int pad(int pos) { return pos + (pos >> 4); }
    __device__ __forceinline__ void st(int pos, float2 x) const { base[pad(pos)] = x; }
    __device__ __forceinline__ float2 ld(int pos) const { return base[pad(pos)]; }
};
__host__ __device__ constexpr int padded_len(int n) { return n + (n >> 4) + 1; }

// Interleaved: C transforms share rows; element pos of transform c at pos*C + c.
template <int C>
struct InterleavedView {
    float2* base;   // already offset by c
    __device__ __forceinline__ void st(int pos, float2 x) const { base[pos * C] = x; }
    __device__ __forceinline__ float2 ld(int pos) const { return base[pos * C]; }
};

template <class View>
__host__ __device__ constexpr bool is_padded()
{
    if constexpr (std::is_same<View, PaddedView>::value) return true;
    else return false;
}

// Barrier covering every thread that shares the view: the warp, the block,
// or (BAR_ID > 0) the BAR_N threads of a named barrier -- a group of warps
// inside a block whose other warps do other work.
template <bool WARP, int BAR_ID = 0, int BAR_N = 0>
__device__ __forceinline__ void xsync()
{
    if constexpr (WARP) {
        __syncwarp();
    } else if constexpr (BAR_ID > 0) {
        static_assert(BAR_N > 0 && BAR_N % 32 == 0, "a named barrier counts whole warps");
        asm volatile("bar.sync %0, %1;" ::"n"(BAR_ID), "n"(BAR_N) : "memory");
    } else {
        __syncthreads();
    }
}

// ---------------------------------------- programmatic dependent launch
// A kernel launched by launch_pdl() may be scheduled while the kernel before
// it in the stream is still finishing (sm_90+).  Each such kernel calls
// pdl_start() first: it lets the next kernel begin to launch, then waits
// until the previous one has completed and its writes are visible, before
// any memory access.  After a kernel that never signals, the wait returns at
// once: the launch then behaves like a plain one.
__device__ __forceinline__ void pdl_start()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// ------------------------------------------------------- Stockham engine

// Stage s has radix 2^lrs(s) and span 2^lns(s).  The full radix goes first,
// where the span is 1 and no twiddles are needed; a smaller remainder radix
// (log2 N not a multiple of log2 R) is the last stage.
template <int LOG2N, int LOG2R>
struct Sched {
    static_assert(LOG2R >= 1 && LOG2R <= LOG2N, "radix must divide the size");
    static constexpr int rem = LOG2N % LOG2R;
    static constexpr int nstages = LOG2N / LOG2R + (rem ? 1 : 0);
    __host__ __device__ static constexpr int lrs(int s) { return (rem && s == nstages - 1) ? rem : LOG2R; }
    __host__ __device__ static constexpr int lns(int s) { return s * LOG2R; }
};

// One radix-RS stage on the R registers of thread t (R/RS butterflies).
template <int LOG2N, int LOG2R, int LRS, int LNS, bool INV>
__device__ __forceinline__ void stage_compute(float2 (&v)[1 << LOG2R], int t, const float2* __restrict__ tw)
{
    constexpr int R = 1 << LOG2R, RS = 1 << LRS, NS = 1 << LNS;
    constexpr int T = (1 << LOG2N) / R;
    constexpr int U = R / RS;
    static_for<0, U>([&](auto uc) {
        constexpr int u = decltype(uc)::value;
        float2 x[RS];
#pragma unroll
        for (int j = 0; j < RS; ++j) x[j] = v[u + j * U];
        if constexpr (NS > 1) {
            const int k = (t + u * T) & (NS - 1);
            // W^{jk} with W = W_{NS*RS}: the power-of-two multiples W^{2^i k}
            // are element k of the level NS*RS / 2^i (one coalesced load each);
            // the rest are products of at most log2(RS) - 1 of those.
            float2 w[RS];
#pragma unroll
            for (int p = 1; p < RS; p <<= 1) w[p] = tw_load<INV>(tw + NS * RS / p, k);
#pragma unroll
            for (int j = 3; j < RS; ++j) {
                if ((j & (j - 1)) == 0) continue;
                const int hb = 1 << (31 - __clz(j));
                w[j] = cmul(w[hb], w[j - hb]);
            }
#pragma unroll
            for (int j = 1; j < RS; ++j) x[j] = cmul(x[j], w[j]);
        }
        dft<RS, INV>(x);
#pragma unroll
        for (int j = 0; j < RS; ++j) v[u + j * U] = x[j];
    });
}

// The same stage with its table twiddles loaded beforehand: wb[u][i] holds
// W^(2^i k_u) for butterfly u (stage_twiddles); the other powers are products
// as in stage_compute.  For kernels that run the same stage on many tiles,
// where k_u does not change from tile to tile.
template <int LOG2N, int LOG2R, int LRS, int LNS, bool INV>
__device__ __forceinline__ void stage_twiddles(int t, const float2* __restrict__ tw,
                                               float2 (&wb)[(1 << LOG2R) >> LRS][LRS])
{
    constexpr int R = 1 << LOG2R, RS = 1 << LRS, NS = 1 << LNS;
    constexpr int T = (1 << LOG2N) / R;
    constexpr int U = R / RS;
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int k = (t + u * T) & (NS - 1);
#pragma unroll
        for (int i = 0; i < LRS; ++i) wb[u][i] = tw_load<INV>(tw + NS * RS / (1 << i), k);
    }
}

template <int LOG2N, int LOG2R, int LRS, int LNS, bool INV>
__device__ __forceinline__ void stage_compute_pre(float2 (&v)[1 << LOG2R], const float2 (&wb)[(1 << LOG2R) >> LRS][LRS])
{
    constexpr int R = 1 << LOG2R, RS = 1 << LRS;
    constexpr int U = R / RS;
    static_assert((1 << LNS) > 1, "the first stage has no twiddles");
    static_for<0, U>([&](auto uc) {
        constexpr int u = decltype(uc)::value;
        float2 x[RS];
#pragma unroll
        for (int j = 0; j < RS; ++j) x[j] = v[u + j * U];
        float2 w[RS];
#pragma unroll
        for (int i = 0; i < LRS; ++i) w[1 << i] = wb[u][i];
#pragma unroll
        for (int j = 3; j < RS; ++j) {
            if ((j & (j - 1)) == 0) continue;
            const int hb = 1 << (31 - __clz(j));
            w[j] = cmul(w[hb], w[j - hb]);
        }
#pragma unroll
        for (int j = 1; j < RS; ++j) x[j] = cmul(x[j], w[j]);
        dft<RS, INV>(x);
#pragma unroll
        for (int j = 0; j < RS; ++j) v[u + j * U] = x[j];
    });
}

// Writes a stage's outputs to their Stockham positions.
template <int LOG2N, int LOG2R, int LRS, int LNS, class View>
__device__ __forceinline__ void stage_write(const float2 (&v)[1 << LOG2R], int t, const View& view)
{
    constexpr int R = 1 << LOG2R, RS = 1 << LRS, NS = 1 << LNS;
    constexpr int T = (1 << LOG2N) / R;
    constexpr int U = R / RS;
    // With the padded layout, positions base + j*NS map to one base slot plus
    // compile-time offsets when the span is 1 or a multiple of 16.
    constexpr bool kFastWrite = is_padded<View>() && (NS == 1 || NS % 16 == 0);
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int b = t + u * T;
        const int base = ((b >> LNS) << (LNS + LRS)) + (b & (NS - 1));
        if constexpr (kFastWrite) {
            float2* p = view.base + PaddedView::pad(base);
#pragma unroll
            for (int j = 0; j < RS; ++j) {
                const int off = NS == 1 ? (RS >= 16 ? j + (j >> 4) : j) : j * (NS + NS / 16);
                p[off] = v[u + j * U];
            }
        } else {
#pragma unroll
            for (int j = 0; j < RS; ++j) view.st(base + j * NS, v[u + j * U]);
        }
    }
}

// Loads the thread's registers with positions t + m*T.
template <int LOG2N, int LOG2R, class View>
__device__ __forceinline__ void stage_read(float2 (&v)[1 << LOG2R], int t, const View& view)
{
    constexpr int R = 1 << LOG2R;
    constexpr int T = (1 << LOG2N) / R;
    // padded layout: positions t + m*T are one base slot plus compile-time
    // offsets when T is a multiple of 16
    if constexpr (is_padded<View>() && T % 16 == 0) {
        const float2* q = view.base + PaddedView::pad(t);
#pragma unroll
        for (int m = 0; m < R; ++m) v[m] = q[m * (T + T / 16)];
    } else {
#pragma unroll
        for (int m = 0; m < R; ++m) v[m] = view.ld(t + m * T);
    }
}

// Writes a stage's outputs to their Stockham positions, then reloads the
// thread's registers with positions t + m*T.
template <int LOG2N, int LOG2R, int LRS, int LNS, bool WARP, int BAR_ID = 0, int BAR_N = 0, class View>
__device__ __forceinline__ void stage_exchange(float2 (&v)[1 << LOG2R], int t, const View& view)
{
    stage_write<LOG2N, LOG2R, LRS, LNS>(v, t, view);
    xsync<WARP, BAR_ID, BAR_N>();
    stage_read<LOG2N, LOG2R>(v, t, view);
    xsync<WARP, BAR_ID, BAR_N>();
}

// Full transform of one length-2^LOG2N sequence held as v[m] = x[t + m*T].
// On return v[m] = X[t + m*T].  The view must not be in use by other code
// between the call's barriers.
// BAR_ID > 0: the threads sharing the view meet at that named barrier (BAR_N threads).
template <int LOG2N, int LOG2R, bool INV, bool WARP, int BAR_ID = 0, int BAR_N = 0, class View>
__device__ __forceinline__ void stockham(float2 (&v)[1 << LOG2R], int t, const float2* __restrict__ tw, const View& view)
{
    if constexpr (LOG2N == 0) {
        (void)v; (void)t; (void)tw; (void)view;
    } else {
        using S = Sched<LOG2N, LOG2R>;
        static_for<0, S::nstages>([&](auto sc) {
            constexpr int s = decltype(sc)::value;
            constexpr int lrs = S::lrs(s), lns = S::lns(s);
            stage_compute<LOG2N, LOG2R, lrs, lns, INV>(v, t, tw);
            if constexpr (s + 1 < S::nstages)
                stage_exchange<LOG2N, LOG2R, lrs, lns, WARP, BAR_ID, BAR_N>(v, t, view);
        });
    }
}

// ------------------------------------------------- real-transform algebra
// Forward split (real forward, src/ckfft/fft_real_default.cpp:30-58):
//   X[k] = (z0 + conj z1) - i W_n^k (z0 - conj z1),  z0 = Z[k], z1 = Z[m-k] (Z[m] = Z[0]).
__device__ __forceinline__ float2 real_split(float2 z0, float2 z1, float2 w)
{
    const float sx = z0.x + z1.x, sy = z0.y - z1.y;
    const float dx = z0.x - z1.x, dy = z0.y + z1.y;
    // c = (i w) * d = (-w.y + i w.x) * (dx + i dy)
    const float cx = fmaf(-w.y, dx, -w.x * dy);
    const float cy = fmaf(w.x, dx, -w.y * dy);
    return make_float2(sx - cx, sy - cy);
}

// Inverse merge (real inverse, src/ckfft/fft_real_default.cpp:79-107):
//   Y[k] = (z0 + conj z1) + i conj(W_n^k) (z0 - conj z1),  z0 = X[k], z1 = X[m-k].
__device__ __forceinline__ float2 real_merge(float2 z0, float2 z1, float2 w)
{
    const float sx = z0.x + z1.x, sy = z0.y - z1.y;
    const float dx = z0.x - z1.x, dy = z0.y + z1.y;
    // c = (i conj w) * d = (w.y + i w.x) * (dx + i dy)
    const float cx = fmaf(w.y, dx, -w.x * dy);
    const float cy = fmaf(w.x, dx, w.y * dy);
    return make_float2(sx + cx, sy + cy);
}

}  // namespace ckg
