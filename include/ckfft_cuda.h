/*
 * ckfft_cuda.h -- Cricket FFT's C API on a GB300 (sm_103a), plus batched entry points.
 *
 * Drop-in: the six CkFft* functions and the three types below have the same
 * names, signatures, argument meaning, scaling and return codes as the
 * reference's public header (inc/ckfft/ckfft.h).  A program written against
 * the reference links unchanged against libckfft_cuda.so.  The header compiles
 * as C99 or later and as C++.
 *
 * Pointers given to any entry point may be host memory (pageable or pinned) or
 * device memory (cudaMalloc / cudaMallocManaged) on the context's device; the
 * library moves host data through device-resident staging buffers itself.
 * Every transform runs in hand-written CUDA kernels; there is no CPU path.
 *
 * Scaling (identical to the reference): no scaling in either direction; a
 * complex forward -> inverse round trip multiplies by n; the real forward
 * output is 2 * DFT(x) over n/2+1 bins, and a real forward -> inverse round
 * trip multiplies by 2n.
 */
#ifndef CKFFT_CUDA_H
#define CKFFT_CUDA_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Interleaved complex value, 8 bytes.  Replaces inc/ckfft/ckfft.h:10-15. */
typedef struct
{
    float real;
    float imag;
}
CkFftComplex;

/* Opaque context.  Replaces inc/ckfft/ckfft.h:18.  Holds the device-resident
 * twiddle tables and staging buffers; immutable after CkFftInit apart from a
 * lock-protected pool of staging lanes, so one context may be used from many
 * host threads at once (as inc/ckfft/ckfft.h:39-41 promises). */
typedef struct _CkFftContext CkFftContext;

/* Direction flags.  Replaces inc/ckfft/ckfft.h:21-27. */
typedef enum
{
    kCkFftDirection_Forward = (1 << 0),
    kCkFftDirection_Inverse = (1 << 1),
    kCkFftDirection_Both    = (kCkFftDirection_Forward | kCkFftDirection_Inverse)
}
CkFftDirection;

/* ----------------------------------------------------------------------
 * Reference API (same contracts as inc/ckfft/ckfft.h)
 * ---------------------------------------------------------------------- */

/* Replaces CkFftInit, inc/ckfft/ckfft.h:59 (src/ckfft/ckfft.cpp:14-34,
 * src/ckfft/context.cpp:45-135).  Returns NULL when nMax <= 0, nMax is not a
 * power of two, direction is not one of the three flags, buf != NULL with
 * bufSize == NULL, when *bufSize is given but buf is NULL or *bufSize is too
 * small (the required size is then written to *bufSize), or when the device
 * tables cannot be created (no CUDA device, out of device memory).
 * buf, when given, holds the host-side context object; the twiddle tables
 * live in device memory owned by the library.  The context is bound to the
 * CUDA device that is current when CkFftInit is called. */
CkFftContext* CkFftInit(int nMax, CkFftDirection direction, void* buf, size_t* bufSize);

/* Replaces CkFftRealForward, inc/ckfft/ckfft.h:85 (src/ckfft/ckfft.cpp:36-53).
 * n real inputs -> n/2+1 complex outputs equal to 2 * DFT(input).
 * Returns 0 on: NULL or forward-less context, n not a power of two or
 * n > nMax, NULL input/output, input == output.  Blocks until done. */
int CkFftRealForward(CkFftContext* context, int n, const float* input, CkFftComplex* output);

/* Replaces CkFftRealInverse, inc/ckfft/ckfft.h:108 (src/ckfft/ckfft.cpp:55-76).
 * n/2+1 complex inputs -> n real outputs.  tmpBuf (n/2+1 elements) must be
 * non-NULL, as in the reference (checked first); the kernels keep their
 * intermediate in on-chip memory and use tmpBuf only when it is device memory
 * and n needs a multi-pass transform. */
int CkFftRealInverse(CkFftContext* context, int n, const CkFftComplex* input, float* output, CkFftComplex* tmpBuf);

/* Replaces CkFftComplexForward, inc/ckfft/ckfft.h:129 (src/ckfft/ckfft.cpp:78-95). */
int CkFftComplexForward(CkFftContext* context, int n, const CkFftComplex* input, CkFftComplex* output);

/* Replaces CkFftComplexInverse, inc/ckfft/ckfft.h:150 (src/ckfft/ckfft.cpp:97-114). */
int CkFftComplexInverse(CkFftContext* context, int n, const CkFftComplex* input, CkFftComplex* output);

/* Replaces CkFftShutdown, inc/ckfft/ckfft.h:158 (src/ckfft/ckfft.cpp:116-119).
 * Frees the device tables and staging lanes; frees the context memory only
 * when CkFftInit allocated it.  CkFftShutdown(NULL) does nothing. */
void CkFftShutdown(CkFftContext* context);

/* ----------------------------------------------------------------------
 * Additions (no counterpart in the reference; prefixed CkFftCuda)
 * ---------------------------------------------------------------------- */

/* Message for the calling thread's most recent failed call ("" if none). */
const char* CkFftCudaGetLastError(void);

/* Batched transforms: `count` independent transforms of size n stored back to
 * back (complex: n values per transform; real forward: n floats in, n/2+1
 * complex out; real inverse: n/2+1 complex in, n floats out).  One kernel
 * launch covers the whole batch (two or three for multi-pass sizes).
 *
 * stream: a cudaStream_t passed as void*.  With NULL the call blocks until
 * `out` holds the results.  With a stream and device pointers for both `in`
 * and `out`, the work is only enqueued on that stream (asynchronous).  With a
 * host pointer on either side the call blocks: page-locked host buffers of
 * single-CTA sizes (complex n <= 2^14, real n <= 2^15) are read and written by
 * the kernels in place; other host data is staged through device buffers,
 * pipelining copies against compute.
 * Validation and return codes follow the single-transform calls; count == 0
 * is valid and does nothing; count < 0 returns 0. */
int CkFftCudaComplexForwardBatch(CkFftContext* context, int n, int count,
                                 const CkFftComplex* input, CkFftComplex* output, void* stream);
int CkFftCudaComplexInverseBatch(CkFftContext* context, int n, int count,
                                 const CkFftComplex* input, CkFftComplex* output, void* stream);
int CkFftCudaRealForwardBatch(CkFftContext* context, int n, int count,
                              const float* input, CkFftComplex* output, void* stream);
int CkFftCudaRealInverseBatch(CkFftContext* context, int n, int count,
                              const CkFftComplex* input, float* output, void* stream);

/* Advanced-layout batches: element p of transform f is read from
 * input[f * in_dist + p * in_stride] and written to
 * output[f * out_dist + p * out_stride], in elements of each pointer's type
 * (CkFftComplex or float).  Interleaved channels (stride = channels,
 * dist = 1), columns of a row-major matrix (stride = row length, dist = 1),
 * overlapping frames (stride = 1, dist = hop < n) and padded rows all run
 * without a copy for complex n <= 2^14 and real 8 <= n <= 2^15; other sizes
 * gather into contiguous rows and scatter back on the GPU.
 *
 * Rules: strides >= 1, distances >= 0 (in_dist == 0 transforms one input
 * `count` times); the output transforms must not overlap one another (either
 * out_dist >= (elements - 1) * out_stride + 1, or out_stride >= (count - 1) *
 * out_dist + 1), and the input and output address ranges must not
 * intersect.  Buffers may be device, managed or page-locked host memory
 * (used in place) or pageable host memory (the layout's whole span is staged
 * through device memory, at most 4 GiB per call).  stream: as for the Batch
 * calls (NULL blocks; a stream with device buffers enqueues only).  Other
 * validation and return codes follow the Batch calls. */
int CkFftCudaComplexForwardStrided(CkFftContext* context, int n, long long count,
                                   const CkFftComplex* input, long long in_stride, long long in_dist,
                                   CkFftComplex* output, long long out_stride, long long out_dist,
                                   void* stream);
int CkFftCudaComplexInverseStrided(CkFftContext* context, int n, long long count,
                                   const CkFftComplex* input, long long in_stride, long long in_dist,
                                   CkFftComplex* output, long long out_stride, long long out_dist,
                                   void* stream);
int CkFftCudaRealForwardStrided(CkFftContext* context, int n, long long count,
                                const float* input, long long in_stride, long long in_dist,
                                CkFftComplex* output, long long out_stride, long long out_dist,
                                void* stream);
int CkFftCudaRealInverseStrided(CkFftContext* context, int n, long long count,
                                const CkFftComplex* input, long long in_stride, long long in_dist,
                                float* output, long long out_stride, long long out_dist,
                                void* stream);

/* Short-time Fourier transform: frame f (f < frames) is
 * signal[f * hop + j] * window[j] for j < frame_len and 0 for frame_len <= j
 * < n (window NULL: rectangular); its real forward transform (the scaling of
 * CkFftRealForward) times `scale` is written as n/2+1 bins at
 * output[f * (n/2+1)].  Overlapping frames (hop < n) and zero-padded frames
 * (frame_len < n) read the signal once; window and scale cost no extra pass.
 * signal must hold (frames - 1) * hop + frame_len floats; output 8-byte
 * aligned and disjoint from signal and window.  Needs the forward direction.
 * Buffers and stream as for the Strided calls.  Returns 1 or 0. */
int CkFftCudaStft(CkFftContext* context, int n, long long frames, const float* signal, long long hop,
                  long long frame_len, const float* window, float scale, CkFftComplex* output, void* stream);

/* Spectral multiply + real inverse (FFT convolution / filtering): frame f's
 * n/2+1 bins spectra[f * (n/2+1) + k] times filter[k] (one filter for every
 * frame; NULL: none) times `scale`, real inverse transform (the scaling of
 * CkFftRealInverse: round trip gain 2n), n reals at output[f * n].  Products
 * are rounded one FP32 operation at a time.  output 8-byte aligned and
 * disjoint from spectra and filter.  Needs the inverse direction.  Buffers
 * and stream as for the Strided calls.  Returns 1 or 0. */
int CkFftCudaFilterInverse(CkFftContext* context, int n, long long frames, const CkFftComplex* spectra,
                           const CkFftComplex* filter, float scale, float* output, void* stream);

/* Self-test of the library's failure detection: makes one of its bounded
 * device-side waits run out on purpose -- which = 0: a mixed-run phase unit
 * waiting for a completion counter that nothing increments; which = 1: a wait
 * for a bulk copy that never arrives -- and checks that the kernel reported
 * the timeout through the error word, returned, and left the context able to
 * transform (a 64-point check).  Nothing faults or hangs; each wait is
 * bounded to about a millisecond here.  Returns 1 when all of that held,
 * else 0 with CkFftCudaGetLastError() saying what did not. */
int CkFftCudaSelfTestWait(CkFftContext* context, int which);

/* Number of kernel launches the library has issued in this process (all
 * contexts, all threads).  Lets a caller count launches inside a timed region. */
long long CkFftCudaLaunchCount(void);

/* ----------------------------------------------------------------------
 * Mixed runs: many transforms of different sizes, kinds and directions in
 * one call or one graph replay (no counterpart in the reference): a
 * persistent kernel over a device work queue takes the small transforms,
 * and each (kind, size) that a batched kernel runs in one launch (complex
 * 2^13..2^16, real 2^14..2^17) is one launch over a table of the jobs'
 * pointers.
 * ---------------------------------------------------------------------- */

#define CKFFT_CUDA_COMPLEX_FORWARD 0
#define CKFFT_CUDA_COMPLEX_INVERSE 1
#define CKFFT_CUDA_REAL_FORWARD    2
#define CKFFT_CUDA_REAL_INVERSE    3

/* One job: `count` transforms of size n stored back to back, laid out as in
 * the batch calls.  input / output are device (or managed) memory on the
 * context's device, 8-byte aligned.  Jobs of one run must not write memory
 * that another job of the run reads.  Complex n up to 2^20, real n up to 2^21. */
typedef struct
{
    int kind;             /* CKFFT_CUDA_COMPLEX_FORWARD .. CKFFT_CUDA_REAL_INVERSE */
    int n;
    int count;
    const void* input;
    void* output;
}
CkFftCudaJob;

typedef struct _CkFftCudaPlan CkFftCudaPlan;

/* Validates the jobs (same rules and errors as the single calls), builds the
 * device work queue and pointer tables, allocates the multi-pass
 * intermediates and captures the run into a CUDA graph (the table launches
 * on parallel branches beside the persistent kernel).  Returns NULL on error
 * (see CkFftCudaGetLastError). */
CkFftCudaPlan* CkFftCudaPlanJobs(CkFftContext* context, const CkFftCudaJob* jobs, int njobs);

/* Replays a plan: one graph launch.  stream NULL blocks until done; otherwise
 * the replay is enqueued on that cudaStream_t.  Replays of one plan must not
 * overlap each other (they share the plan's queue and counters). */
int CkFftCudaExecPlan(CkFftCudaPlan* plan, void* stream);

/* Frees a plan (waits for its work). */
void CkFftCudaDestroyPlan(CkFftCudaPlan* plan);

/* Algorithmic HBM bytes of one replay of the plan (each transform read once
 * and written once). */
long long CkFftCudaPlanBytes(const CkFftCudaPlan* plan);

/* One-shot mixed run without a graph: plan, launch, free (stream-ordered).
 * stream NULL blocks until done. */
int CkFftCudaRunJobs(CkFftContext* context, const CkFftCudaJob* jobs, int njobs, void* stream);

/* ----------------------------------------------------------------------
 * Serving: a request server with continuous batching (no counterpart in the
 * reference).  A dispatcher thread keeps up to max_inflight runs of the
 * persistent job kernel on the GPU; requests submitted while runs are in
 * flight are admitted, in arrival order, into the next free run slot while
 * their multi-pass scratch fits the slot's share of scratch_budget_bytes (a
 * larger request runs alone once free HBM covers it).
 * ---------------------------------------------------------------------- */

typedef struct _CkFftCudaServer CkFftCudaServer;

/* A request of a replayed trace: a job and its arrival time in seconds after
 * the replay starts. */
typedef struct
{
    double arrival_s;
    CkFftCudaJob job;
}
CkFftCudaRequest;

/* Latency and throughput of a replay.  Latency runs from a request's
 * scheduled arrival to the moment its results are complete on the device. */
typedef struct
{
    long long requests;
    double seconds;        /* first arrival to last completion */
    double algo_bytes;     /* algorithmic bytes of all requests */
    double p50_s;
    double p99_s;
    double p999_s;
    double max_s;
}
CkFftCudaServeStats;

/* max_inflight: job-kernel runs on the GPU at once (1..16).
 * direct_threshold_bytes: requests whose algorithmic bytes (each transform
 * read once and written once) reach this size skip batching and run through
 * the batched entry points on one of two direct lanes; 0 batches everything. */
CkFftCudaServer* CkFftCudaServerCreate(CkFftContext* context, size_t scratch_budget_bytes, int max_inflight,
                                       long long direct_threshold_bytes);
void CkFftCudaServerDestroy(CkFftCudaServer* server);   /* finishes admitted work first */

/* Queues one request (validated like a job).  Its buffers may be device
 * memory of the context's device or host memory: host-side inputs are copied
 * into the server's resident device staging buffers on the run's stream, and
 * outputs copied back before the request completes (page-locked host memory
 * keeps those copies asynchronous; pageable memory works but makes the
 * dispatcher wait for each copy).  Returns a ticket > 0, or 0 on error.
 * Never blocks on the GPU. */
long long CkFftCudaServerSubmit(CkFftCudaServer* server, const CkFftCudaJob* job);

/* Waits for a ticket (timeout_s < 0: no limit).  1 when its results are
 * complete (latency_s: submission to completion), 0 on timeout or failure. */
int CkFftCudaServerWait(CkFftCudaServer* server, long long ticket, double timeout_s, double* latency_s);

/* Submits a trace at its arrival times from the calling thread, waits for every
 * request, and reports per-request latency (latency_s[n], may be NULL) and
 * statistics.  Returns 1 when every request completed. */
int CkFftCudaServerReplay(CkFftCudaServer* server, const CkFftCudaRequest* requests, int n,
                          double* latency_s, CkFftCudaServeStats* stats);

/* The same trace through the plain path, one batch call per request at its
 * arrival (one launch per request, two or three for multi-pass sizes),
 * blocking: the comparison point for the server. */
int CkFftCudaReplayPerRequest(CkFftContext* context, const CkFftCudaRequest* requests, int n,
                              double* latency_s, CkFftCudaServeStats* stats);

/* Complex batch that allocates no memory.  No counterpart in the reference.
 * For callers that must not allocate while they run: a real-time audio
 * callback cannot wait for cudaMalloc/cudaFree (they can synchronise the whole
 * device), and a host with a fixed memory budget or its own device allocator
 * must not see the library allocate mid-stream.  Same transform and return
 * codes as CkFftCudaComplex{Forward,Inverse}Batch (inverse != 0 selects the
 * inverse), but `input` and `output` must be device (or managed) memory, and
 * n is limited to 2^20: sizes above 2^14 keep their intermediate in one
 * fixed 8 MiB device array compiled into the library, which every GPU that
 * loads the library holds until the process exits.  All calls on a device
 * share that array, so calls that overlap on the GPU race; order them (one
 * stream, or events).  The array's device address is looked up once per
 * device when the first context is created on it (CkFftInit), so the 8 MiB is
 * committed then and this call only reads the cached address; after a
 * cudaDeviceReset, reload the library before using it again.  The first call
 * of each size may still make the CUDA driver load that size's kernel code
 * (lazy module loading; CUDA_MODULE_LOADING=EAGER loads everything up front),
 * so make one call per size you use before the time-critical part and before
 * any stream capture.  stream == NULL blocks until done; otherwise the work
 * is enqueued on that cudaStream_t. */
int CkFftCudaComplexBatchNoAlloc(CkFftContext* context, int n, int count, int inverse,
                                 const CkFftComplex* input, CkFftComplex* output, void* stream);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* CKFFT_CUDA_H */
