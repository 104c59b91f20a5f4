// kernels.h -- host-side launch interface of the CUDA kernels (internal).
//
// Plain C++ (no device code) so that the C-ABI layer can be compiled by the
// host compiler.  Every launcher enqueues work on `stream` and returns the
// launch status; none of them synchronises.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>

struct _CkFftContext;

namespace ckg {

enum Kind : int { C2C_FWD = 0, C2C_INV = 1, R2C = 2, C2R = 3 };

// Largest log2 size whose whole transform runs in one CTA's shared memory.
// For R2C/C2R the size is the real length n (the complex half-length is n/2).
constexpr int kSmallMaxLog2Complex = 14;
constexpr int kSmallMaxLog2Real = 15;

// Single-CTA transforms of 2^log2n points, `count` of them.
//   C2C: in/out are complex, dist in complex elements.
//   R2C: in is float (dist in floats, even), out complex (dist in complex).
//   C2R: in complex (dist in complex), out float (dist in floats, even).
// R2C/C2R need log2n >= 3 (n >= 8); smaller real sizes use launch_real_tiny.
cudaError_t launch_small(Kind kind, int log2n, const void* in, void* out, long long count,
                         long long in_dist, long long out_dist, const float2* tw, cudaStream_t stream);

// Advanced layout of a batch: element p of transform f is read from
// in[f * in_dist + p * in_stride] and written to out[f * out_dist +
// p * out_stride], in elements of each side's type (complex or float).
struct Layout {
    long long in_stride;
    long long in_dist;
    long long out_stride;
    long long out_dist;
};
// Single-CTA sizes the strided kernels cover (complex 2^0..2^14, real 2^3..2^15).
bool strided_supported(Kind kind, int log2n);
cudaError_t launch_strided(Kind kind, int log2n, const void* in, void* out, long long count, const Layout& lay,
                           const float2* tw, cudaStream_t stream);
// Layouts whose consecutive transforms are adjacent (distance 1, stride > 1)
// on the input (cin) and / or output (cout) side: CTAs move whole rows of
// consecutive transforms (fft_inter.cu).  Complex 2^6..2^13 with cin or
// cout; real forward with cin, real inverse with cout, n = 2^7..2^14.
bool inter_applies(Kind kind, int log2n, bool cin, bool cout);
cudaError_t launch_inter(Kind kind, int log2n, const void* in, void* out, long long count, const Layout& lay,
                         bool cin, bool cout, const float2* tw, cudaStream_t stream);
// `count` rows of `len` elements of `esize` bytes (4 or 8) between the
// strided layout (stride, dist) and contiguous rows.
cudaError_t launch_gather(const void* src, long long stride, long long dist, void* dst, long long count,
                          long long len, int esize, cudaStream_t stream);
cudaError_t launch_scatter(const void* src, void* dst, long long stride, long long dist, long long count,
                           long long len, int esize, cudaStream_t stream);
// dst[c dp + r] = src[r sp + c] for r < rows, c < cols, elements of esize 4
// or 8 bytes (pitches in elements); stream_src / stream_dst: evict-first
// loads / stores for a side touched once.
cudaError_t launch_transpose(const void* src, long long sp, void* dst, long long dp, long long rows, long long cols,
                             int esize, bool stream_src, bool stream_dst, cudaStream_t stream);

// Fused steps around the real transforms (single-CTA sizes, 8 <= n <= 2^15):
// windowed frames at a hop -> real forward -> bins x scale; bins x filter x
// scale -> real inverse.  `out` of launch_stft holds n/2+1 bins per frame,
// `out` of launch_filter_inverse n reals per frame (8-byte aligned).
bool fused_supported(int log2n);
cudaError_t launch_stft(int log2n, const float* signal, long long hop, const float* window, long long frame_len,
                        float scale, void* out, long long count, const float2* tw, cudaStream_t stream);
cudaError_t launch_filter_inverse(int log2n, const void* spectra, const void* filter, float scale, float* out,
                                  long long count, const float2* tw, cudaStream_t stream);
// Row passes of the same steps for the other sizes: windowed frames into
// contiguous rows of n reals; bins x filter x scale into contiguous rows;
// `total` complex values scaled in place.
cudaError_t launch_window_rows(const float* signal, long long hop, const float* window, long long frame_len,
                               float* rows, long long count, long long n, cudaStream_t stream);
cudaError_t launch_filter_rows(const void* spectra, const void* filter, float scale, void* rows, long long count,
                               long long bins, cudaStream_t stream);
cudaError_t launch_scale_rows(void* p, long long total, float scale, cudaStream_t stream);

// Real transforms of n = 1, 2 or 4 points (closed forms, src/ckfft/fft_real.cpp:20-93).
cudaError_t launch_real_tiny(Kind kind, int n, const void* in, void* out, long long count,
                             long long in_dist, long long out_dist, cudaStream_t stream);

// Multi-pass complex transforms for sizes above the single-CTA limit.
// scratch must hold count_per_group * 2^log2n complex values; the call splits
// the batch into groups whose scratch fits.  Returns the launch status.
struct LargePlan {
    int log2n;       // total size
    int log2n1;      // column (first-pass) length
    int log2n2;      // row (second-pass) length
};
LargePlan large_plan(int log2n);
cudaError_t launch_large_c2c(bool inverse, int log2n, const void* in, void* out, long long count,
                             long long in_dist, long long out_dist, const float2* tw,
                             void* scratch, size_t scratch_bytes, cudaStream_t stream);

// Real transforms above the single-CTA limit: half-size multi-pass complex
// transform with the split (forward) fused into its last pass, the merge
// (inverse) into its first.
cudaError_t launch_large_r2c(int log2n, const void* in, void* out, long long count,
                             long long in_dist, long long out_dist, const float2* tw,
                             void* scratch, size_t scratch_bytes, cudaStream_t stream);
cudaError_t launch_large_c2r(int log2n, const void* in, void* out, long long count,
                             long long in_dist, long long out_dist, const float2* tw,
                             void* scratch, size_t scratch_bytes, cudaStream_t stream);
// Single-pass complex transforms of 2^14 .. 2^16 on thread-block clusters
// (fft_cluster.cu).  cluster_enabled(): only with CKFFT_CUDA_CLUSTER=1.
bool cluster_supported(int log2n);
bool cluster_enabled();
cudaError_t launch_cluster_c2c(bool inverse, int log2n, const void* in, void* out, long long count,
                               long long in_dist, long long out_dist, const float2* tw, cudaStream_t stream);

// Complex 2^15 and 2^16 with both passes inside one thread-block cluster per
// transform and the intermediate kept in L2 (fft_l2pass.cu); scratch as for
// launch_large_c2c, 128-byte aligned.
// kind: 0 / 1 complex forward / inverse of 2^log2n points, 2 / 3 real
// forward / inverse of 2^(log2n+1) points (split / merge fused; dists in
// complex units).
bool l2pass_supported(int log2n);
cudaError_t launch_l2pass(int kind, int log2n, const void* in, void* out, long long count, long long in_dist,
                          long long out_dist, const float2* tw, void* scratch, size_t scratch_bytes,
                          cudaStream_t stream);

// Complex 2^15 and 2^16 on persistent CTAs, one transform per CTA at a time,
// both passes inside the CTA with bulk-copied tiles and the intermediate in
// L2 (fft_mid.cu).  scratch: mid_scratch_bytes(), 128-byte aligned; in
// 16-byte aligned, in_dist even.  kind 0 / 1: forward / inverse.
// mid_enabled(log2n): only with CKFFT_CUDA_MID=1 (opt-in; the cluster
// two-pass kernel of fft_l2pass.cu measured as fast or faster).
bool mid_supported(int log2n);
bool mid_enabled(int log2n);
size_t mid_scratch_bytes(int log2n, long long count);
cudaError_t launch_mid(int kind, int log2n, const void* in, void* out, long long count, long long in_dist,
                       long long out_dist, const float2* tw, void* scratch, size_t scratch_bytes, cudaStream_t stream);

// Scratch bytes one transform of the given kind and size needs on the large path.
size_t large_scratch_bytes(Kind kind, int log2n);

// Sets per-kernel attributes (dynamic shared memory limits) on the current
// device.  Idempotent; called when a context is created.
cudaError_t prepare_device();

// Launches `kernel` with programmatic stream serialization: it may start
// while the previous kernel in the stream finishes; the kernel must call
// pdl_start() (fft_core.cuh) before touching memory.
template <class... KArgs, class... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// Kernel launches issued so far by this process.
long long launch_count();
void count_launch(int n = 1);

// Read-only view of a context for entry points defined outside ckfft_api.cpp.
struct ContextView {
    int nmax;
    int direction;
    int device;
    const float2* tw;
};
// Validates a context handle and copies its fields (ckfft_api.cpp).
bool context_view(const struct ::_CkFftContext* c, ContextView* out);
// Sets the calling thread's CkFftCudaGetLastError() message.
void set_last_error(const char* msg);

// Smallest log2 (complex) length served by the pipelined persistent kernels.
constexpr int kPipeMinLog2 = 6;
// Kernel variant for a single-CTA size: 0 plain (default shape), 2 / 3
// pipelined with that many bulk-copy buffers, 4 / 5 half / twice the values
// per thread, 6 / 7 CTAs of about 512 / 128 threads, 8 pipelined with one
// bulk-copy buffer and a separate split exchange area (complex kinds).  From the committed
// autotune table (tuning_table.h) unless the CKFFT_CUDA_VARIANT environment
// variable forces one variant (the autotuner uses it to measure each);
// a variant that does not exist for a size runs the plain kernel.
int variant_for(Kind kind, int log2c);
// The batched single-CTA kernels in shape variant v (4..7) for complex
// (half-)length 2^log2c, dists as the plain launchers take them; *done is
// false when that variant does not exist for the size (nothing launched).
cudaError_t launch_small_shape(Kind kind, int v, int log2c, const void* in, void* out, long long count,
                               long long in_dist, long long out_dist, const float2* tw, cudaStream_t stream,
                               bool* done);
// While one of these lives on a thread, variant_for() answers 0 on that
// thread: launches whose input is host memory mapped into the device's
// address space read it with plain loads, never with bulk (TMA) copies.
struct PlainLoadsScope {
    PlainLoadsScope();
    ~PlainLoadsScope();
    int prev;
};
// Device word (in mapped host memory) where kernels record a timed-out wait,
// for the current device; take_device_error() reads and clears it.
unsigned* device_error_word();
unsigned take_device_error();

// Stream-ordered allocation from a library-owned memory pool on the current
// device; the pool keeps freed memory (release threshold: unlimited), so
// repeated calls do not map and unmap device memory.  Free with cudaFreeAsync.
cudaError_t pool_alloc_async(void** p, size_t bytes, cudaStream_t s);
// cudaMalloc through the library's fault-injection point
// (CKFFT_CUDA_FAIL_ALLOC=k fails the k-th allocation of the process).
cudaError_t dev_malloc(void** p, size_t bytes);

}  // namespace ckg
