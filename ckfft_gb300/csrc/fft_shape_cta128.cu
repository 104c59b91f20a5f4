// fft_shape_cta128.cu -- single-CTA batched kernels with CTAs of about 128 threads
// (variant 7, fft_small_shapes.cuh).
#include "fft_small_shapes.cuh"

namespace ckg {

cudaError_t launch_shape_cta128(Kind kind, int log2c, const void* in, void* out, long long count, long long in_dist,
                            long long out_dist, const float2* tw, cudaStream_t s, bool* done)
{
    return shape_launch_any<7>(kind, log2c, in, out, count, in_dist, out_dist, tw, s, done);
}

cudaError_t prepare_shape_cta128() { return shape_attr_any<7>(); }

}  // namespace ckg
