// fft_small_shapes.cuh -- the single-CTA batched kernels in the other launch
// shapes the autotuner measures (variants 4..7 of fft_small.cuh: half or
// twice the values per thread, CTAs of about 512 or 128 threads), for
// complex (half-)lengths 2^6 .. 2^14.  The committed tuning table
// (tuning_table.h) selects one per kind and size; a variant that does not
// exist for a size falls back to the default shape.  Each variant is
// instantiated in its own translation unit (fft_shape_*.cu) so that they
// compile in parallel.
#pragma once
#include "fft_small.cuh"

namespace ckg {

template <int L, int V>
static cudaError_t shape_launch(Kind kind, const void* in, void* out, long long count, long long in_dist,
                                long long out_dist, const float2* tw, cudaStream_t s, bool* done)
{
    using S = ShapeOf<L, V>;
    *done = false;
    if constexpr (S::kValid) {
        *done = true;
        switch (kind) {
        case C2C_FWD: return launch_c2c_L<L, false, S::LR, S::CTH>(in, out, count, in_dist, out_dist, tw, s);
        case C2C_INV: return launch_c2c_L<L, true, S::LR, S::CTH>(in, out, count, in_dist, out_dist, tw, s);
        case R2C: return launch_r2c_L<L, S::LR, S::CTH>(in, out, count, in_dist, out_dist, tw, s);
        default: return launch_c2r_L<L, S::LR, S::CTH>(in, out, count, in_dist, out_dist, tw, s);
        }
    } else {
        return cudaSuccess;
    }
}

// Launches `count` transforms of complex (half-)length 2^log2c in variant V
// (dists as launch_c2c_L / launch_r2c_L / launch_c2r_L take them); *done is
// false when the variant does not exist for this size (nothing launched).
template <int V>
static cudaError_t shape_launch_any(Kind kind, int log2c, const void* in, void* out, long long count,
                                    long long in_dist, long long out_dist, const float2* tw, cudaStream_t s,
                                    bool* done)
{
#define CKG_SHAPE_CASE(L) \
    case L: return shape_launch<L, V>(kind, in, out, count, in_dist, out_dist, tw, s, done);
    switch (log2c) {
        CKG_SHAPE_CASE(6) CKG_SHAPE_CASE(7) CKG_SHAPE_CASE(8) CKG_SHAPE_CASE(9) CKG_SHAPE_CASE(10)
        CKG_SHAPE_CASE(11) CKG_SHAPE_CASE(12) CKG_SHAPE_CASE(13) CKG_SHAPE_CASE(14)
    default:
        *done = false;
        return cudaSuccess;
    }
#undef CKG_SHAPE_CASE
}

template <int L, int V>
static cudaError_t shape_attr()
{
    using S = ShapeOf<L, V>;
    if constexpr (S::kValid) {
        cudaError_t e = attr_c2c_L<L, false, S::LR, S::CTH>();
        if (e == cudaSuccess) e = attr_c2c_L<L, true, S::LR, S::CTH>();
        if (e == cudaSuccess) e = attr_real_L<L, S::LR, S::CTH>();
        return e;
    } else {
        return cudaSuccess;
    }
}

template <int V>
static cudaError_t shape_attr_any()
{
    cudaError_t e = cudaSuccess;
#define CKG_ATTR(L) \
    if (e == cudaSuccess) e = shape_attr<L, V>();
    CKG_ATTR(6) CKG_ATTR(7) CKG_ATTR(8) CKG_ATTR(9) CKG_ATTR(10) CKG_ATTR(11) CKG_ATTR(12) CKG_ATTR(13) CKG_ATTR(14)
#undef CKG_ATTR
    return e;
}

}  // namespace ckg
