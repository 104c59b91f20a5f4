// fft_shape_doubler.cu -- single-CTA batched kernels with twice the values per thread
// (variant 5, fft_small_shapes.cuh).
#include "fft_small_shapes.cuh"

namespace ckg {

cudaError_t launch_shape_doubler(Kind kind, int log2c, const void* in, void* out, long long count, long long in_dist,
                            long long out_dist, const float2* tw, cudaStream_t s, bool* done)
{
    return shape_launch_any<5>(kind, log2c, in, out, count, in_dist, out_dist, tw, s, done);
}

cudaError_t prepare_shape_doubler() { return shape_attr_any<5>(); }

}  // namespace ckg
