// fft_groups.cu -- grouped launches of a job run: the transforms of one kind
// and size whose batched kernel beats the job kernel's units run as one
// hardware-scheduled launch that reads each transform's input and output
// pointers from a table (FrameDesc), instead of as units of the persistent
// kernel.  The frame bodies are the batched kernels' (fft_small.cuh); the
// 2^15 / 2^16 complex groups and the real 2^16 / 2^17 groups use the
// cluster two-pass kernel with its table argument (fft_l2pass.cu; real: the
// split / merge fused into its tiles).
#include "fft_small.cuh"
#include "jobs.h"
#include "kernels.h"

namespace ckg {

template <int L, bool INV>
__global__ void __launch_bounds__(SmallCfg<L>::THREADS, SmallCfg<L>::MINB)
k_c2c_table(const FrameDesc* __restrict__ fr, long long count, const float2* __restrict__ tw)
{
    using C = SmallCfg<L>;
    pdl_start();
    extern __shared__ float2 smem[];
    const int g = threadIdx.x / C::T, t = threadIdx.x % C::T;
    const long long f = (long long)blockIdx.x * C::TPB + g;
    const bool live = f < count;
    const FrameDesc d = fr[live ? f : 0];
    frame_c2c<L, INV>(d.in, d.out, live, t, PaddedView{smem + g * C::SLOT}, tw);
}

template <int LM>
__global__ void __launch_bounds__(SmallCfg<LM>::THREADS, SmallCfg<LM>::MINB)
k_r2c_table(const FrameDesc* __restrict__ fr, long long count, const float2* __restrict__ tw)
{
    using C = SmallCfg<LM>;
    pdl_start();
    extern __shared__ float2 smem[];
    const int g = threadIdx.x / C::T, t = threadIdx.x % C::T;
    const long long f = (long long)blockIdx.x * C::TPB + g;
    const bool live = f < count;
    const FrameDesc d = fr[live ? f : 0];
    frame_r2c<LM>(d.in, d.out, live, t, PaddedView{smem + g * C::SLOT}, tw);
}

template <int LM>
__global__ void __launch_bounds__(SmallCfg<LM>::THREADS, SmallCfg<LM>::MINB)
k_c2r_table(const FrameDesc* __restrict__ fr, long long count, const float2* __restrict__ tw)
{
    using C = SmallCfg<LM>;
    pdl_start();
    extern __shared__ float2 smem[];
    const int g = threadIdx.x / C::T, t = threadIdx.x % C::T;
    const long long f = (long long)blockIdx.x * C::TPB + g;
    const bool live = f < count;
    const FrameDesc d = fr[live ? f : 0];
    frame_c2r<LM>(d.in, d.out, live, t, PaddedView{smem + g * C::SLOT}, tw);
}

template <int L, int OP>
static cudaError_t launch_table_L(const FrameDesc* fr, long long count, const float2* tw, cudaStream_t s)
{
    using C = SmallCfg<L>;
    const dim3 grid((unsigned)((count + C::TPB - 1) / C::TPB)), block(C::THREADS);
    if constexpr (OP == U_C2C_FWD) return launch_pdl(k_c2c_table<L, false>, grid, block, C::SMEM, s, fr, count, tw);
    else if constexpr (OP == U_C2C_INV) return launch_pdl(k_c2c_table<L, true>, grid, block, C::SMEM, s, fr, count, tw);
    else if constexpr (OP == U_R2C) return launch_pdl(k_r2c_table<L>, grid, block, C::SMEM, s, fr, count, tw);
    else return launch_pdl(k_c2r_table<L>, grid, block, C::SMEM, s, fr, count, tw);
}

template <int OP>
static cudaError_t launch_table(int l, const FrameDesc* fr, long long count, const float2* tw, cudaStream_t s)
{
    switch (l) {
    case 10: return launch_table_L<10, OP>(fr, count, tw, s);
    case 11: return launch_table_L<11, OP>(fr, count, tw, s);
    case 12: return launch_table_L<12, OP>(fr, count, tw, s);
    case 13: return launch_table_L<13, OP>(fr, count, tw, s);
    case 14: return launch_table_L<14, OP>(fr, count, tw, s);
    default: return cudaErrorInvalidValue;
    }
}

// Sizes the job kernel runs as two phases of pass units (log2a above
// kJobMaxSingleLog2) and a batched kernel runs in one launch: single-CTA up
// to 2^14, the cluster two-pass kernel at 2^15 / 2^16 (complex, and real
// half lengths with the split / merge fused).
bool group_supported(int op, int log2a)
{
    if (log2a <= kJobMaxSingleLog2) return false;
    switch (op) {
    case U_C2C_FWD:
    case U_C2C_INV: return log2a <= 14 || l2pass_supported(log2a);
    case U_R2C: return log2a <= 16;
    case U_C2R: return log2a <= 16;
    default: return false;
    }
}

size_t group_scratch_bytes(int op, int log2a, long long count)
{
    if (log2a <= 14 || !(op == U_C2C_FWD || op == U_C2C_INV || op == U_R2C || op == U_C2R)) return 0;
    const long long per_launch = count < kGroupMaxL2Transforms ? count : kGroupMaxL2Transforms;
    return sizeof(float2) * ((size_t)per_launch << log2a);
}

cudaError_t launch_group(int op, int log2a, const FrameDesc* fr, long long count, const float2* tw,
                         void* scratch, size_t scratch_bytes, cudaStream_t s)
{
    if (count <= 0) return cudaSuccess;
    if (log2a > 14) {
        // the cluster two-pass kernel: complex, or real with the split / merge
        // fused into its tiles (kind 2 / 3)
        const int kind = op == U_C2C_FWD ? 0 : op == U_C2C_INV ? 1 : op == U_R2C ? 2 : op == U_C2R ? 3 : -1;
        if (kind < 0) return cudaErrorInvalidValue;
        return launch_l2pass_table(kind, log2a, fr, count, tw, scratch, scratch_bytes, s);
    }
    cudaError_t e;
    switch (op) {
    case U_C2C_FWD: e = launch_table<U_C2C_FWD>(log2a, fr, count, tw, s); break;
    case U_C2C_INV: e = launch_table<U_C2C_INV>(log2a, fr, count, tw, s); break;
    case U_R2C: e = launch_table<U_R2C>(log2a, fr, count, tw, s); break;
    case U_C2R: e = launch_table<U_C2R>(log2a, fr, count, tw, s); break;
    default: return cudaErrorInvalidValue;
    }
    if (e == cudaSuccess) count_launch();
    return e;
}

template <int L>
static cudaError_t attr_table_L()
{
    const int smem = (int)SmallCfg<L>::SMEM;
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = cudaFuncSetAttribute(k_c2c_table<L, false>, a, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_c2c_table<L, true>, a, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_r2c_table<L>, a, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_c2r_table<L>, a, smem);
    return e;
}

cudaError_t prepare_groups()
{
    cudaError_t e = attr_table_L<10>();
    if (e == cudaSuccess) e = attr_table_L<11>();
    if (e == cudaSuccess) e = attr_table_L<12>();
    if (e == cudaSuccess) e = attr_table_L<13>();
    if (e == cudaSuccess) e = attr_table_L<14>();
    return e;
}

}  // namespace ckg
