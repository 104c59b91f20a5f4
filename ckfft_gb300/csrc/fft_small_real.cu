// fft_small_real.cu -- instantiates the single-CTA real kernels (n = 2^3 .. 2^15)
// and the closed-form kernel for n = 1, 2, 4.
#include "fft_pipe.cuh"

namespace ckg {

template <int LM, bool INV>
static cudaError_t launch_real_any(const void* in, void* out, long long count, long long in_dist,
                                   long long out_dist, const float2* tw, cudaStream_t s)
{
    // in_dist / out_dist in elements of the input / output type (floats on the real side)
    long long done = 0;
    cudaError_t e = cudaSuccess;
    if constexpr (LM >= kPipeMinLog2) {
        constexpr int K = INV ? C2R : R2C;
        const long long di = INV ? in_dist : in_dist / 2, dout = INV ? out_dist / 2 : out_dist;
        const int nb = variant_for((Kind)K, LM);
        if (nb >= 4) {
            bool shaped = false;
            e = launch_small_shape((Kind)K, nb, LM, in, out, count, in_dist, out_dist, tw, s, &shaped);
            if (shaped && e == cudaSuccess) count_launch();
            if (shaped || e != cudaSuccess) return e;
        }
        if (nb == 2) e = launch_pipe<LM, K, 2>(in, out, count, di, dout, tw, device_error_word(), s, &done);
        else if (nb == 3) e = launch_pipe<LM, K, 3>(in, out, count, di, dout, tw, device_error_word(), s, &done);
        else if (nb == 8) e = launch_pipe_sx<LM, K>(in, out, count, di, dout, tw, device_error_word(), s, &done);
        if (e != cudaSuccess) return e;
        if (done) count_launch();
    }
    if (done < count) {
        const void* tin = INV ? (const void*)((const float2*)in + done * in_dist) : (const void*)((const float*)in + done * in_dist);
        void* tout = INV ? (void*)((float*)out + done * out_dist) : (void*)((float2*)out + done * out_dist);
        e = INV ? launch_c2r_L<LM>(tin, tout, count - done, in_dist, out_dist, tw, s)
                : launch_r2c_L<LM>(tin, tout, count - done, in_dist, out_dist, tw, s);
        if (e == cudaSuccess) count_launch();
    }
    return e;
}

cudaError_t launch_small_real(bool inv, int log2n, const void* in, void* out, long long count,
                              long long in_dist, long long out_dist, const float2* tw, cudaStream_t s)
{
    // log2n is the real length; kernels are templated on the complex half-length.
#define CKG_REAL_CASE(LM)                                                                         \
    case LM + 1:                                                                                  \
        return inv ? launch_real_any<LM, true>(in, out, count, in_dist, out_dist, tw, s)          \
                   : launch_real_any<LM, false>(in, out, count, in_dist, out_dist, tw, s);
    switch (log2n) {
        CKG_REAL_CASE(2) CKG_REAL_CASE(3) CKG_REAL_CASE(4) CKG_REAL_CASE(5) CKG_REAL_CASE(6)
        CKG_REAL_CASE(7) CKG_REAL_CASE(8) CKG_REAL_CASE(9) CKG_REAL_CASE(10) CKG_REAL_CASE(11)
        CKG_REAL_CASE(12) CKG_REAL_CASE(13) CKG_REAL_CASE(14)
    default:
        return cudaErrorInvalidValue;
    }
#undef CKG_REAL_CASE
}

template <int LM>
static cudaError_t attr_real_all()
{
    cudaError_t e = cudaSuccess;
    if (LM >= 10) e = attr_real_L<LM>();
    if constexpr (LM >= kPipeMinLog2) {
        if (e == cudaSuccess) e = attr_pipe<LM, R2C, 2>();
        if (e == cudaSuccess) e = attr_pipe<LM, C2R, 2>();
        if (e == cudaSuccess) e = attr_pipe<LM, R2C, 3>();
        if (e == cudaSuccess) e = attr_pipe<LM, C2R, 3>();
        if (e == cudaSuccess) e = attr_pipe_sx<LM, R2C>();
        if (e == cudaSuccess) e = attr_pipe_sx<LM, C2R>();
    }
    return e;
}

cudaError_t prepare_small_real()
{
    cudaError_t e = cudaSuccess;
#define CKG_ATTR(LM) \
    if (e == cudaSuccess) e = attr_real_all<LM>();
    CKG_ATTR(6) CKG_ATTR(7) CKG_ATTR(8) CKG_ATTR(9) CKG_ATTR(10) CKG_ATTR(11) CKG_ATTR(12) CKG_ATTR(13) CKG_ATTR(14)
#undef CKG_ATTR
    return e;
}

// Closed forms of src/ckfft/fft_real.cpp:20-48 (forward, scaled by 2) and
// :69-93 (inverse), one frame per thread.  Only the documented n/2+1 output
// bins are written for the forward n = 4 case.
__global__ void k_real_tiny(int n, bool inv, const float* __restrict__ in, float* __restrict__ out,
                            long long count, long long in_dist, long long out_dist)
{
    const long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= count) return;
    if (!inv) {
        const float* x = in + f * in_dist;          // floats
        float2* y = (float2*)out + f * out_dist;    // complex
        if (n == 1) {
            y[0] = make_float2(x[0] * 2.0f, 0.0f);
        } else if (n == 2) {
            y[0] = make_float2((x[0] + x[1]) * 2.0f, 0.0f);
            y[1] = make_float2((x[0] - x[1]) * 2.0f, 0.0f);
        } else {
            const float s02 = (x[0] + x[2]) * 2.0f, d02 = (x[0] - x[2]) * 2.0f;
            const float s13 = (x[1] + x[3]) * 2.0f, d13 = (x[1] - x[3]) * 2.0f;
            y[0] = make_float2(s02 + s13, 0.0f);
            y[1] = make_float2(d02, -d13);
            y[2] = make_float2(s02 - s13, 0.0f);
        }
    } else {
        const float2* x = (const float2*)in + f * in_dist;   // complex
        float* y = out + f * out_dist;                       // floats
        if (n == 1) {
            y[0] = x[0].x;
        } else if (n == 2) {
            y[0] = x[0].x + x[1].x;
            y[1] = x[0].x - x[1].x;
        } else {
            const float s02 = x[0].x + x[2].x;
            const float s13 = 2.0f * x[1].x;
            const float d02 = x[0].x - x[2].x;
            const float d13 = 2.0f * x[1].y;
            y[0] = s02 + s13;
            y[1] = d02 - d13;
            y[2] = s02 - s13;
            y[3] = d02 + d13;
        }
    }
}

cudaError_t launch_real_tiny(Kind kind, int n, const void* in, void* out, long long count,
                             long long in_dist, long long out_dist, cudaStream_t s)
{
    if (n != 1 && n != 2 && n != 4) return cudaErrorInvalidValue;
    const int threads = 256;
    const unsigned blocks = (unsigned)((count + threads - 1) / threads);
    k_real_tiny<<<blocks, threads, 0, s>>>(n, kind == C2R, (const float*)in, (float*)out, count,
                                           in_dist, out_dist);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ckg
