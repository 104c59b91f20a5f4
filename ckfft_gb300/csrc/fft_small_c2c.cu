// fft_small_c2c.cu -- instantiates the single-CTA complex kernels (2^0 .. 2^14).
#include "fft_small.cuh"

namespace ckg {

cudaError_t launch_small_c2c(bool inv, int log2n, const void* in, void* out, long long count,
                             long long in_dist, long long out_dist, const float2* tw, cudaStream_t s)
{
#define CKG_C2C_CASE(L)                                                                           \
    case L:                                                                                       \
        return inv ? launch_c2c_L<L, true>(in, out, count, in_dist, out_dist, tw, s)              \
                   : launch_c2c_L<L, false>(in, out, count, in_dist, out_dist, tw, s);
    switch (log2n) {
        CKG_C2C_CASE(0) CKG_C2C_CASE(1) CKG_C2C_CASE(2) CKG_C2C_CASE(3) CKG_C2C_CASE(4)
        CKG_C2C_CASE(5) CKG_C2C_CASE(6) CKG_C2C_CASE(7) CKG_C2C_CASE(8) CKG_C2C_CASE(9)
        CKG_C2C_CASE(10) CKG_C2C_CASE(11) CKG_C2C_CASE(12) CKG_C2C_CASE(13) CKG_C2C_CASE(14)
    default:
        return cudaErrorInvalidValue;
    }
#undef CKG_C2C_CASE
}

cudaError_t prepare_small_c2c()
{
    cudaError_t e = cudaSuccess;
#define CKG_ATTR(L)                                                  \
    if (e == cudaSuccess) e = attr_c2c_L<L, false>();                \
    if (e == cudaSuccess) e = attr_c2c_L<L, true>();
    CKG_ATTR(10) CKG_ATTR(11) CKG_ATTR(12) CKG_ATTR(13) CKG_ATTR(14)
#undef CKG_ATTR
    return e;
}

}  // namespace ckg
