// fft_small_c2c.cu -- instantiates the single-CTA complex kernels (2^0 .. 2^14):
// the pipelined persistent kernel for whole frame groups, the plain kernel for
// the rest; the tuned shape variants live in fft_shape_*.cu.
#include "fft_pipe.cuh"

namespace ckg {

template <int L, bool INV>
static cudaError_t launch_c2c_any(const void* in, void* out, long long count, long long in_dist,
                                  long long out_dist, const float2* tw, cudaStream_t s)
{
    long long done = 0;
    cudaError_t e = cudaSuccess;
    if constexpr (L >= kPipeMinLog2) {
        constexpr int K = INV ? C2C_INV : C2C_FWD;
        const int nb = variant_for((Kind)K, L);
        if (nb >= 4) {
            bool shaped = false;
            e = launch_small_shape((Kind)K, nb, L, in, out, count, in_dist, out_dist, tw, s, &shaped);
            if (shaped && e == cudaSuccess) count_launch();
            if (shaped || e != cudaSuccess) return e;
        }
        if (nb == 2) e = launch_pipe<L, K, 2>(in, out, count, in_dist, out_dist, tw, device_error_word(), s, &done);
        else if (nb == 3) e = launch_pipe<L, K, 3>(in, out, count, in_dist, out_dist, tw, device_error_word(), s, &done);
        else if (nb == 8) e = launch_pipe_sx<L, K>(in, out, count, in_dist, out_dist, tw, device_error_word(), s, &done);
        if (e != cudaSuccess) return e;
        if (done) count_launch();
    }
    if (done < count) {
        e = launch_c2c_L<L, INV>((const float2*)in + done * in_dist, (float2*)out + done * out_dist,
                                 count - done, in_dist, out_dist, tw, s);
        if (e == cudaSuccess) count_launch();
    }
    return e;
}

cudaError_t launch_small_c2c(bool inv, int log2n, const void* in, void* out, long long count,
                             long long in_dist, long long out_dist, const float2* tw, cudaStream_t s)
{
#define CKG_C2C_CASE(L)                                                                           \
    case L:                                                                                       \
        return inv ? launch_c2c_any<L, true>(in, out, count, in_dist, out_dist, tw, s)            \
                   : launch_c2c_any<L, false>(in, out, count, in_dist, out_dist, tw, s);
    switch (log2n) {
        CKG_C2C_CASE(0) CKG_C2C_CASE(1) CKG_C2C_CASE(2) CKG_C2C_CASE(3) CKG_C2C_CASE(4)
        CKG_C2C_CASE(5) CKG_C2C_CASE(6) CKG_C2C_CASE(7) CKG_C2C_CASE(8) CKG_C2C_CASE(9)
        CKG_C2C_CASE(10) CKG_C2C_CASE(11) CKG_C2C_CASE(12) CKG_C2C_CASE(13) CKG_C2C_CASE(14)
    default:
        return cudaErrorInvalidValue;
    }
#undef CKG_C2C_CASE
}

template <int L>
static cudaError_t attr_c2c_all()
{
    cudaError_t e = cudaSuccess;
    if (L >= 10 && e == cudaSuccess) e = attr_c2c_L<L, false>();
    if (L >= 10 && e == cudaSuccess) e = attr_c2c_L<L, true>();
    if constexpr (L >= kPipeMinLog2) {
        if (e == cudaSuccess) e = attr_pipe<L, C2C_FWD, 2>();
        if (e == cudaSuccess) e = attr_pipe<L, C2C_INV, 2>();
        if (e == cudaSuccess) e = attr_pipe<L, C2C_FWD, 3>();
        if (e == cudaSuccess) e = attr_pipe<L, C2C_INV, 3>();
        if (e == cudaSuccess) e = attr_pipe_sx<L, C2C_FWD>();
        if (e == cudaSuccess) e = attr_pipe_sx<L, C2C_INV>();
    }
    return e;
}

cudaError_t prepare_small_c2c()
{
    cudaError_t e = cudaSuccess;
#define CKG_ATTR(L) \
    if (e == cudaSuccess) e = attr_c2c_all<L>();
    CKG_ATTR(6) CKG_ATTR(7) CKG_ATTR(8) CKG_ATTR(9) CKG_ATTR(10) CKG_ATTR(11) CKG_ATTR(12) CKG_ATTR(13) CKG_ATTR(14)
#undef CKG_ATTR
    return e;
}

}  // namespace ckg
