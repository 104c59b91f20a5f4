// jobs.h -- work-unit descriptors of the persistent job kernel (host and device).
//
// A run of mixed transforms is flattened into a queue of units that the
// persistent CTAs pop with one atomic add each:
//   * single-CTA units: up to min(256/T, 64) frames of one kind and size,
//     each frame with its own input / output pointer (FrameDesc);
//   * phase units of a multi-pass transform (LargeDesc): a set of column
//     tiles (phase 0; real inverse: with the merge fused) or of row tiles
//     (phase 1; real forward: with the split fused).  A phase unit
//     names how many units of its transform must have finished first; every
//     unit of a transform adds one to that transform's counter when done.
// Phase-p units are queued after every phase-(p-1) unit, so a CTA only ever
// waits for units that CTAs already running have taken.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "ckfft_cuda.h"

namespace ckg {

enum UnitOp : int {
    U_C2C_FWD = 0,     // single-CTA complex forward, log2a = log2 n
    U_C2C_INV = 1,
    U_R2C = 2,         // single-CTA real forward, log2a = log2 (n/2)
    U_C2R = 3,
    U_RTINY_FWD = 4,   // real n = 1, 2, 4 closed forms, log2a = log2 n
    U_RTINY_INV = 5,
    U_COLS_FWD = 6,    // column pass, log2a = column length, log2b = log2 columns
    U_COLS_INV = 7,
    U_ROWS_FWD = 8,    // row pass, log2a = row length, log2b = log2 rows
    U_ROWS_INV = 9,
    U_COLS_MERGE = 10, // real inverse: merge fused into the column pass (pass_cols_merge)
    U_ROWS_SPLIT = 11, // real forward: split fused into the row pass (pass_rows_split)
};

// Buffer selectors of a phase unit.
enum BufSel : int { B_IN = 0, B_OUT = 1, B_SCRATCH = 2 };

struct Unit {
    int op;
    int log2a;
    int log2b;
    int job;       // multi-pass transform index (its counter), -1 for single-CTA units
    int need;      // units of `job` that must have finished before this one
    int first;     // first tile (pass), first element (split / merge)
    int count;     // frames, tiles or elements
    int sel;       // source selector | destination selector << 4 (phase units)
};

struct FrameDesc {
    const float2* in;
    float2* out;
};

// Grouped launches (fft_groups.cu): the transforms of one (op, log2a) of a
// job run in one launch over a FrameDesc table.  op is a single-CTA op
// (U_C2C_FWD .. U_C2R); log2a as for units.
bool group_supported(int op, int log2a);
// Scratch of a group of `count` transforms (cluster two-pass groups: at
// most kGroupMaxL2Transforms transforms per launch).
constexpr long long kGroupMaxL2Transforms = 1024;
size_t group_scratch_bytes(int op, int log2a, long long count);
cudaError_t launch_group(int op, int log2a, const FrameDesc* fr, long long count, const float2* tw,
                         void* scratch, size_t scratch_bytes, cudaStream_t s);
cudaError_t launch_l2pass_table(int kind, int log2n, const FrameDesc* fr, long long count, const float2* tw,
                                void* scratch, size_t scratch_bytes, cudaStream_t s);
cudaError_t prepare_groups();

struct LargeDesc {
    const float2* in;
    float2* out;
    float2* scratch;
    long long pad;
};

// Frame pointers one single-CTA unit carries at most.
constexpr int kRecFrames = 64;

// Everything one unit needs, in one fixed-size record: a CTA copies the next
// unit's record into shared memory (one bulk copy) while it works on the
// current one, so a unit starts without a chain of dependent global loads.
struct UnitRec {
    Unit u;
    LargeDesc big;                  // phase units: the transform's buffers
    FrameDesc frames[kRecFrames];   // single-CTA units: u.count frames
};
static_assert(sizeof(UnitRec) % 16 == 0, "records are bulk-copied in 16-byte units");

struct JobsArgs {
    const UnitRec* recs;
    int nunits;
    int* done;         // one counter per multi-pass transform
    int* head;         // queue head
    const float2* tw;
    unsigned* err;
    int wait_tries;    // bound of a phase unit's counter wait; 0: the default (seconds)
};

// 256 threads per CTA and 64 registers: four CTAs -- four independent unit
// streams -- per SM, which hides the latency of each unit's start (queue
// claim, descriptor, frame pointers) better than two larger CTAs.
constexpr int kJobThreads = 256;
constexpr int kJobCtasPerSm = 4;

// Largest multi-pass size the job kernel handles (sub-lengths up to 2^10).
constexpr int kJobMaxLog2Complex = 20;
// Single-CTA sizes inside the job kernel (complex length); 2^13 and up run
// as column / row passes.
constexpr int kJobMaxSingleLog2 = 12;

struct ContextView;

// Resident buffers of one in-flight run (grown on demand and reused; a slot
// may be refilled only after its previous run has completed).
struct RunSlot {
    void* dev = nullptr;         // units | frames | large | counters, device
    size_t dev_cap = 0;
    char* host = nullptr;        // the same, pinned staging on the host
    size_t host_cap = 0;
    float2* scratch = nullptr;   // multi-pass intermediates
    size_t scratch_cap = 0;
};
void free_run_slot(RunSlot* r);
// Validates, builds and enqueues a mixed run on `s` with the slot's buffers.
// 1 on success, 0 on invalid jobs, -1 on a CUDA failure (message set).
// scratch_override: caller-owned intermediates of scratch_override_bytes
// (a run needing more fails with -1); NULL uses (and grows) the slot's own
// scratch.
int enqueue_run(const ContextView& cv, const CkFftCudaJob* jobs, int njobs, RunSlot* r, cudaStream_t s,
                float2* scratch_override = nullptr, size_t scratch_override_bytes = 0);
bool validate_job(const ContextView& cv, const CkFftCudaJob& j, int index, bool allow_host = false);
long long job_scratch_bytes(const CkFftCudaJob& j);
long long job_algo_bytes(const CkFftCudaJob& j);
// Bytes of a job's whole input / output; whether a buffer is outside the
// context's device (host memory, to be staged).
long long job_in_bytes(const CkFftCudaJob& j);
long long job_out_bytes(const CkFftCudaJob& j);
bool job_host_side(const ContextView& cv, const void* p);

// Launches the job kernel on all resident CTAs of the current device.
cudaError_t launch_jobs(const JobsArgs& a, cudaStream_t s);
// The job kernel on one CTA (self-test of the bounded waits).
cudaError_t launch_jobs_one(const JobsArgs& a, cudaStream_t s);
// Shared memory the job kernel needs (bytes) and resident CTAs per SM.
size_t jobs_smem_bytes();
int jobs_grid();

}  // namespace ckg
