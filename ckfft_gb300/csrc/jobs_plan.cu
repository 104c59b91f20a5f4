// jobs_plan.cu -- host side of mixed runs: CkFftCudaPlanJobs / ExecPlan / RunJobs.
//
// Turns a list of jobs (kind, size, count, device pointers) into the unit
// queue of the persistent job kernel (jobs.h) and the pointer tables of the
// grouped launches (fft_groups.cu), uploads them once, and captures
// "reset counters + grouped launches on side branches + persistent launch"
// into a CUDA graph, so a replay costs one graph launch regardless of how
// many transforms the run holds.
#include <algorithm>
#include <array>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "ckfft_cuda.h"
#include "fft_passes.cuh"
#include "fft_small.cuh"
#include "jobs.h"
#include "kernels.h"

namespace ckg {


// Threads per tile and tiles per pass unit for sub-length 2^LS (PassCfg).
struct PassShape {
    int threads;
    int cols;
};
static PassShape pass_shape(int ls)
{
    switch (ls) {
    case 6: return {PassCfg<6, kJobThreads>::THREADS, PassCfg<6, kJobThreads>::C};
    case 7: return {PassCfg<7, kJobThreads>::THREADS, PassCfg<7, kJobThreads>::C};
    case 8: return {PassCfg<8, kJobThreads>::THREADS, PassCfg<8, kJobThreads>::C};
    case 9: return {PassCfg<9, kJobThreads>::THREADS, PassCfg<9, kJobThreads>::C};
    case 10: return {PassCfg<10, kJobThreads>::THREADS, PassCfg<10, kJobThreads>::C};
    default: return {0, 0};
    }
}

// Threads per frame of a single-CTA size 2^L (SmallCfg<L>::T).
static int single_threads(int l)
{
    switch (l) {
    case 0: return SmallCfg<0>::T;
    case 1: return SmallCfg<1>::T;
    case 2: return SmallCfg<2>::T;
    case 3: return SmallCfg<3>::T;
    case 4: return SmallCfg<4>::T;
    case 5: return SmallCfg<5>::T;
    case 6: return SmallCfg<6>::T;
    case 7: return SmallCfg<7>::T;
    case 8: return SmallCfg<8>::T;
    case 9: return SmallCfg<9>::T;
    case 10: return SmallCfg<10>::T;
    case 11: return SmallCfg<11>::T;
    case 12: return SmallCfg<12>::T;
    case 13: return SmallCfg<13>::T;
    default: return 0;
    }
}


// A grouped launch: `count` transforms of one (op, log2a), their pointers at
// gframes[first ..], scratch at scratch_off (float2 elements) when needed.
struct GroupSpec {
    int op;
    int log2a;
    int first;
    int count;
    long long scratch_off;
    size_t scratch_bytes;
};

struct Built {
    std::vector<Unit> units;
    std::vector<FrameDesc> frames;
    std::vector<LargeDesc> large;   // scratch pointers relative (offset in float2) until placed
    std::vector<long long> scratch_off;
    std::vector<GroupSpec> groups;
    std::vector<FrameDesc> gframes;
    long long scratch_elems = 0;
    long long algo_bytes = 0;
    long long transforms = 0;
    bool empty() const { return units.empty() && groups.empty(); }
};

static int ilog2ll(long long n)
{
    int l = 0;
    while ((1ll << l) < n) ++l;
    return l;
}

static bool on_device(const void* p, int dev)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

// Host memory (page-locked or pageable) as cudaPointerGetAttributes reports it.
static bool on_host(const void* p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return true;
    }
    return a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeUnregistered;
}

// Checks one job against the rules of the single calls plus the job
// kernel's limits; sets the error message (naming job `j`) on failure.
// allow_host: the buffers may also be host memory (the request server stages
// such requests through its own device buffers).
bool validate_job(const ContextView& cv, const CkFftCudaJob& J, int j, bool allow_host)
{
    char msg[200];
    if (J.kind < 0 || J.kind > 3) {
        snprintf(msg, sizeof msg, "job %d: kind must be 0..3", j);
        set_last_error(msg);
        return false;
    }
    const bool inverse = J.kind == 1 || J.kind == 3;
    const bool real = J.kind >= 2;
    if (!(cv.direction & (inverse ? kCkFftDirection_Inverse : kCkFftDirection_Forward))) {
        snprintf(msg, sizeof msg, "job %d: context was created without this direction", j);
        set_last_error(msg);
        return false;
    }
    if (J.n <= 0 || (J.n & (J.n - 1)) || J.n > cv.nmax) {
        snprintf(msg, sizeof msg, "job %d: n must be a power of two no larger than the context's nMax", j);
        set_last_error(msg);
        return false;
    }
    if (J.count < 0) {
        snprintf(msg, sizeof msg, "job %d: count must be >= 0", j);
        set_last_error(msg);
        return false;
    }
    if (J.count == 0) return true;
    if (!J.input || !J.output || J.input == J.output) {
        snprintf(msg, sizeof msg, "job %d: input and output must be distinct non-NULL buffers", j);
        set_last_error(msg);
        return false;
    }
    if (!((on_device(J.input, cv.device) || (allow_host && on_host(J.input))) &&
          (on_device(J.output, cv.device) || (allow_host && on_host(J.output))))) {
        snprintf(msg, sizeof msg, allow_host ? "job %d: buffers must be host memory or device memory of the context's device"
                                             : "job %d: jobs take device (or managed) memory", j);
        set_last_error(msg);
        return false;
    }
    if (((uintptr_t)J.input & 7) || ((uintptr_t)J.output & 7)) {
        snprintf(msg, sizeof msg, "job %d: device buffers must be 8-byte aligned", j);
        set_last_error(msg);
        return false;
    }
    const int lc = ilog2ll(J.n) - (real ? 1 : 0);
    if (lc > kJobMaxLog2Complex) {
        snprintf(msg, sizeof msg, "job %d: n = %d exceeds the job kernel's limit (complex 2^20, real 2^21)", j, J.n);
        set_last_error(msg);
        return false;
    }
    return true;
}

// Validates the jobs and builds the unit queue.  Returns false with an error set.
static bool build_units(const ContextView& cv, const CkFftCudaJob* jobs, int njobs, Built* b)
{
    if (njobs < 0 || (njobs > 0 && !jobs)) {
        set_last_error("jobs must be a non-NULL array when njobs > 0");
        return false;
    }
    std::map<std::pair<int, int>, std::vector<FrameDesc>> buckets;   // (op, log2a) -> frames
    std::map<std::pair<int, int>, std::vector<FrameDesc>> gbuckets;  // grouped launches
    std::vector<std::array<std::vector<Unit>, 2>> phases;           // per multi-pass transform
    for (int j = 0; j < njobs; ++j) {
        const CkFftCudaJob& J = jobs[j];
        if (!validate_job(cv, J, j)) return false;
        if (J.count == 0) continue;
        const bool inverse = J.kind == 1 || J.kind == 3;
        const bool real = J.kind >= 2;
        const int L = ilog2ll(J.n);
        const int lc = real ? L - 1 : L;                     // complex (half-)length
        const long long in_dist = real ? (inverse ? J.n / 2 + 1 : J.n / 2) : J.n;    // float2 units
        const long long out_dist = real ? (inverse ? J.n / 2 : J.n / 2 + 1) : J.n;
        const long long in_stride_bytes = real && !inverse ? 4ll * J.n : 8ll * in_dist;
        const long long out_stride_bytes = real && inverse ? 4ll * J.n : 8ll * out_dist;
        b->algo_bytes += (long long)J.count * (real ? 4ll * J.n + 8ll * (J.n / 2 + 1) : 16ll * J.n);
        b->transforms += J.count;
        for (int f = 0; f < J.count; ++f) {
            const float2* in = (const float2*)((const char*)J.input + (size_t)f * in_stride_bytes);
            float2* out = (float2*)((char*)J.output + (size_t)f * out_stride_bytes);
            const int sop = real ? (inverse ? U_C2R : U_R2C) : (inverse ? U_C2C_INV : U_C2C_FWD);
            if (real && J.n <= 4) {
                buckets[{inverse ? U_RTINY_INV : U_RTINY_FWD, L}].push_back({in, out});
            } else if (group_supported(sop, lc)) {
                gbuckets[{sop, lc}].push_back({in, out});
            } else if (lc <= kJobMaxSingleLog2) {
                const int op = real ? (inverse ? U_C2R : U_R2C) : (inverse ? U_C2C_INV : U_C2C_FWD);
                buckets[{op, lc}].push_back({in, out});
            } else {
                // multi-pass transform: a phase of column tiles, then one of row tiles
                const int job = (int)b->large.size();
                b->large.push_back({in, out, nullptr, 0});
                phases.emplace_back();
                auto& phase = phases.back();
                b->scratch_off.push_back(b->scratch_elems);
                b->scratch_elems += 1ll << lc;
                const int la = lc / 2, lb = lc - la;
                const PassShape pa = pass_shape(la), pb = pass_shape(lb);
                const int sa = kJobThreads / pa.threads, sb = kJobThreads / pb.threads;
                const int tiles_a = (1 << lb) / pa.cols, tiles_b = (1 << la) / pb.cols;
                int done = 0, p = 0, added = 0;   // units of earlier phases, of this phase
                auto add_pass = [&](int op, int ls, int other, int tiles, int per, int src, int dst) {
                    for (int t = 0; t < tiles; t += per, ++added)
                        phase[p].push_back({op, ls, other, job, done, t, per, src | (dst << 4)});
                };
                auto end_phase = [&]() {
                    done += added;
                    added = 0;
                    ++p;
                };
                // real: the merge fused into the column pass (inverse), the
                // split into the row pass (forward) -- two phases, like complex
                add_pass(real && inverse ? U_COLS_MERGE : inverse ? U_COLS_INV : U_COLS_FWD, la, lb, tiles_a, sa,
                         B_IN, B_SCRATCH);
                end_phase();
                add_pass(real && !inverse ? U_ROWS_SPLIT : inverse ? U_ROWS_INV : U_ROWS_FWD, lb, la, tiles_b, sb,
                         B_SCRATCH, B_OUT);
            }
        }
    }
    // Grouped launches: one per (op, log2a), largest first.
    for (auto it = gbuckets.rbegin(); it != gbuckets.rend(); ++it) {
        const std::vector<FrameDesc>& fr = it->second;
        GroupSpec g{it->first.first, it->first.second, (int)b->gframes.size(), (int)fr.size(), 0, 0};
        g.scratch_bytes = group_scratch_bytes(g.op, g.log2a, g.count);
        if (g.scratch_bytes) {
            g.scratch_off = b->scratch_elems;
            b->scratch_elems += (long long)((g.scratch_bytes / sizeof(float2) + 15) / 16 * 16);
        }
        b->groups.push_back(g);
        b->gframes.insert(b->gframes.end(), fr.begin(), fr.end());
    }
    // Single-CTA units, largest frames first.
    std::vector<Unit> singles;
    std::vector<std::pair<std::pair<int, int>, std::vector<FrameDesc>>> order(buckets.begin(), buckets.end());
    std::stable_sort(order.begin(), order.end(), [](const auto& x, const auto& y) { return x.first.second > y.first.second; });
    for (auto& kv : order) {
        const int op = kv.first.first, l2 = kv.first.second;
        const int per = std::min((op == U_RTINY_FWD || op == U_RTINY_INV) ? kJobThreads
                                                                           : kJobThreads / single_threads(l2),
                                 kRecFrames);
        const std::vector<FrameDesc>& fr = kv.second;
        for (size_t i = 0; i < fr.size(); i += per) {
            const int cnt = (int)std::min<size_t>(per, fr.size() - i);
            singles.push_back({op, l2, 0, -1, 0, (int)b->frames.size(), cnt, 0});
            b->frames.insert(b->frames.end(), fr.begin() + i, fr.begin() + i + cnt);
        }
    }
    // Queue order.  The first phase of the multi-pass transforms is spread
    // over the single-CTA units (both grouped by type, see below); each
    // later phase of a transform is placed `window` units after the last unit
    // of its previous phase.  The window (twice the resident CTAs) is long
    // enough that the previous phase has
    // usually finished when the next one is taken (no idle wait), and short
    // enough that the intermediate it wrote is still in L2.  Phase p of a
    // transform always follows all of its phase p-1, so every wait is for
    // units that running CTAs already hold.
    const size_t window = 2 * (size_t)jobs_grid();
    struct Pending {
        size_t ready;
        int job, phase;
    };
    std::vector<Pending> pending;       // kept sorted by `ready`
    auto push_phase = [&](int job, int p) {
        b->units.insert(b->units.end(), phases[job][p].begin(), phases[job][p].end());
        if (p + 1 < 2 && !phases[job][p + 1].empty()) {
            Pending q{b->units.size() + window, job, p + 1};
            auto it = std::upper_bound(pending.begin(), pending.end(), q,
                                       [](const Pending& x, const Pending& y) { return x.ready < y.ready; });
            pending.insert(it, q);
        }
    };
    auto drain_ready = [&]() {
        while (!pending.empty() && pending.front().ready <= b->units.size()) {
            const Pending q = pending.front();
            pending.erase(pending.begin());
            push_phase(q.job, q.phase);
        }
    };
    const size_t nl = phases.size();
    // Multi-pass transforms grouped by unit type (operation, sub-lengths):
    // the kernel holds a device function per operation and size, and a
    // queue that mixes every type at once spills the SMs' instruction cache
    // (the 10000-job run of log2 n 6..16: 24 M instruction-cache misses and
    // 818 us unsorted, 2387-2399 GB/s sorted against 2016).
    std::vector<int> jorder(nl);
    for (size_t j = 0; j < nl; ++j) jorder[j] = (int)j;
    auto jkey = [&](int j) {
        const Unit& u0 = phases[j][0].front();
        const Unit& u1 = phases[j][1].empty() ? u0 : phases[j][1].front();
        return std::make_tuple(u0.op, u0.log2a, u1.op, u1.log2a);
    };
    std::stable_sort(jorder.begin(), jorder.end(), [&](int x, int y) { return jkey(x) < jkey(y); });
    size_t si = 0;
    for (size_t jj = 0; jj < nl; ++jj) {
        push_phase(jorder[jj], 0);
        drain_ready();
        const size_t upto = singles.size() * (jj + 1) / nl;
        for (; si < upto; ++si) {
            b->units.push_back(singles[si]);
            drain_ready();
        }
    }
    for (; si < singles.size(); ++si) {
        b->units.push_back(singles[si]);
        drain_ready();
    }
    while (!pending.empty()) {
        const Pending q = pending.front();
        pending.erase(pending.begin());
        push_phase(q.job, q.phase);
    }
    return true;
}

// Scratch bytes one job needs in a run (multi-pass intermediates; 0 for
// single-CTA sizes).
long long job_scratch_bytes(const CkFftCudaJob& j)
{
    if (j.count <= 0 || j.n <= 0) return 0;
    const bool real = j.kind >= 2;
    const int lc = ilog2ll(j.n) - (real ? 1 : 0);
    if ((real && j.n <= 4) || lc <= kJobMaxSingleLog2) return 0;
    return (long long)j.count * (long long)sizeof(float2) * (1ll << lc);
}

bool job_host_side(const ContextView& cv, const void* p) { return !on_device(p, cv.device); }

long long job_in_bytes(const CkFftCudaJob& j)
{
    const bool real = j.kind >= 2, inverse = j.kind == 1 || j.kind == 3;
    return (long long)j.count * (real ? (inverse ? 8ll * (j.n / 2 + 1) : 4ll * j.n) : 8ll * j.n);
}

long long job_out_bytes(const CkFftCudaJob& j)
{
    const bool real = j.kind >= 2, inverse = j.kind == 1 || j.kind == 3;
    return (long long)j.count * (real ? (inverse ? 4ll * j.n : 8ll * (j.n / 2 + 1)) : 8ll * j.n);
}

long long job_algo_bytes(const CkFftCudaJob& j)
{
    const bool real = j.kind >= 2;
    return (long long)j.count * (real ? 4ll * j.n + 8ll * (j.n / 2 + 1) : 16ll * j.n);
}

// The queue as fixed-size records: each unit with its transform's buffers
// (phase units) or its frame pointers (single-CTA units) inline.
static void make_records(const Built& b, float2* scratch, std::vector<UnitRec>* recs)
{
    recs->assign(b.units.size(), UnitRec{});
    for (size_t i = 0; i < b.units.size(); ++i) {
        UnitRec& r = (*recs)[i];
        r.u = b.units[i];
        if (r.u.job >= 0) {
            r.big = b.large[r.u.job];
            r.big.scratch = scratch + b.scratch_off[r.u.job];
            r.u.need *= kJobThreads / 32;      // completion is counted per warp
        } else {
            for (int f = 0; f < r.u.count; ++f) r.frames[f] = b.frames[r.u.first + f];
            r.u.first = 0;
        }
    }
}

// Device layout of a run: unit records | counters + queue head | the grouped
// launches' frame tables.
struct RunLayout {
    size_t recs, done, gframes, total;
};

static RunLayout run_layout(const Built& b)
{
    RunLayout l{};
    size_t off = 0;
    l.recs = off; off += sizeof(UnitRec) * b.units.size();
    off = (off + 15) / 16 * 16;
    l.done = off; off += sizeof(int) * (b.large.size() + 1);
    off = (off + 15) / 16 * 16;
    l.gframes = off; off += sizeof(FrameDesc) * b.gframes.size();
    l.total = off + 16;
    return l;
}

// The run's grouped launches, in order, on `s` (frame tables on the device).
static cudaError_t launch_groups(const Built& b, const FrameDesc* dframes, float2* scratch, const float2* tw,
                                 cudaStream_t s)
{
    for (const GroupSpec& g : b.groups) {
        cudaError_t e = launch_group(g.op, g.log2a, dframes + g.first, g.count, tw, scratch + g.scratch_off,
                                     g.scratch_bytes, s);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

void free_run_slot(RunSlot* r)
{
    cudaFree(r->dev);
    cudaFreeHost(r->host);
    cudaFree(r->scratch);
    *r = RunSlot{};
}

static cudaError_t grow_dev(void** p, size_t* cap, size_t need)
{
    if (*cap >= need) return cudaSuccess;
    cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    const size_t want = need + need / 4;
    cudaError_t e = dev_malloc(p, want);
    if (e == cudaSuccess) *cap = want;
    return e;
}

int enqueue_run(const ContextView& cv, const CkFftCudaJob* jobs, int njobs, RunSlot* r, cudaStream_t s,
                float2* scratch_override, size_t scratch_override_bytes)
{
    Built b;
    if (!build_units(cv, jobs, njobs, &b)) return 0;
    if (b.empty()) return 1;
    if (scratch_override && sizeof(float2) * (size_t)b.scratch_elems > scratch_override_bytes) {
        set_last_error("the run's intermediates exceed the scratch it was given");
        return -1;
    }
    const RunLayout lay = run_layout(b);
    const size_t o_recs = lay.recs, o_done = lay.done, total = lay.total;
    cudaError_t e = cudaSuccess;
    if (r->host_cap < total) {
        cudaFreeHost(r->host);
        r->host = nullptr;
        r->host_cap = 0;
        e = cudaHostAlloc((void**)&r->host, total + total / 4, cudaHostAllocDefault);
        if (e == cudaSuccess) r->host_cap = total + total / 4;
    }
    if (e == cudaSuccess) e = grow_dev(&r->dev, &r->dev_cap, total);
    if (e == cudaSuccess && b.scratch_elems && !scratch_override)
        e = grow_dev((void**)&r->scratch, &r->scratch_cap, sizeof(float2) * (size_t)b.scratch_elems);
    float2* scratch = scratch_override ? scratch_override : r->scratch;
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        return -1;
    }
    std::vector<UnitRec> recs;
    make_records(b, scratch, &recs);
    memcpy(r->host + o_recs, recs.data(), sizeof(UnitRec) * recs.size());
    memset(r->host + o_done, 0, sizeof(int) * (b.large.size() + 1));
    if (!b.gframes.empty()) memcpy(r->host + lay.gframes, b.gframes.data(), sizeof(FrameDesc) * b.gframes.size());
    char* base = (char*)r->dev;
    JobsArgs a{};
    a.recs = (const UnitRec*)(base + o_recs);
    a.nunits = (int)b.units.size();
    a.done = (int*)(base + o_done);
    a.head = a.done + b.large.size();
    a.tw = cv.tw;
    a.err = device_error_word();
    e = cudaMemcpyAsync(r->dev, r->host, total, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = launch_groups(b, (const FrameDesc*)(base + lay.gframes), scratch, cv.tw, s);
    if (e == cudaSuccess && !b.units.empty()) {
        e = launch_jobs(a, s);
        if (e == cudaSuccess) count_launch();
    }
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        return -1;
    }
    return 1;
}

}  // namespace ckg

using namespace ckg;

struct _CkFftCudaPlan {
    ContextView cv;
    int nunits = 0;
    int nlarge = 0;
    void* dmem = nullptr;        // units | frames | large | done | head
    float2* scratch = nullptr;
    JobsArgs args{};
    size_t counters_bytes = 0;
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool work = false;           // units or grouped launches to run
    int kernels = 0;             // kernel nodes of the graph (launches per replay)
    // graph branches: grouped launches on side streams, concurrent with the
    // persistent kernel and with each other (no launch waits for another's
    // tail); 2 / 4 / 8 branches measured 3112 / 3247 / 3282 GB/s on the
    // 10000-job run
    static constexpr int kBranches = 8;
    cudaStream_t side[kBranches] = {};
    cudaEvent_t fork = nullptr;
    cudaEvent_t join[kBranches] = {};
    long long algo_bytes = 0;
    long long transforms = 0;
};

namespace {

template <class T>
size_t align_up(size_t x) { return (x + alignof(T) - 1) / alignof(T) * alignof(T); }

// Lays out the built queue in one device allocation.  `dmem` receives the
// allocation, `scratch` the multi-pass intermediates.
cudaError_t upload(const Built& b, ContextView cv, void** dmem, float2** scratch, JobsArgs* a, size_t* counters_bytes,
                   const FrameDesc** dframes, cudaStream_t s, bool async_alloc)
{
    const RunLayout lay = run_layout(b);
    const size_t o_recs = lay.recs, o_done = lay.done, total = lay.total;
    cudaError_t e = async_alloc ? pool_alloc_async(dmem, total, s) : dev_malloc(dmem, total);
    if (e != cudaSuccess) return e;
    *scratch = nullptr;
    if (b.scratch_elems) {
        e = async_alloc ? pool_alloc_async((void**)scratch, sizeof(float2) * b.scratch_elems, s)
                        : dev_malloc((void**)scratch, sizeof(float2) * b.scratch_elems);
        if (e != cudaSuccess) return e;
    }
    std::vector<char> host(total, 0);
    std::vector<UnitRec> recs;
    make_records(b, *scratch, &recs);
    memcpy(host.data() + o_recs, recs.data(), sizeof(UnitRec) * recs.size());
    if (!b.gframes.empty()) memcpy(host.data() + lay.gframes, b.gframes.data(), sizeof(FrameDesc) * b.gframes.size());
    // pageable source: the call returns once the data is staged, so `host` may go
    e = cudaMemcpyAsync(*dmem, host.data(), total, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    char* base = (char*)*dmem;
    a->recs = (const UnitRec*)(base + o_recs);
    a->nunits = (int)b.units.size();
    a->done = (int*)(base + o_done);
    a->head = a->done + b.large.size();
    a->tw = cv.tw;
    a->err = device_error_word();
    *counters_bytes = sizeof(int) * (b.large.size() + 1);
    *dframes = (const FrameDesc*)(base + lay.gframes);
    return cudaSuccess;
}

int fail_cuda(const char* where, cudaError_t e)
{
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    set_last_error(m.c_str());
    return 0;
}

struct DevScope {
    int prev = -1;
    bool ok = true;
    explicit DevScope(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) { ok = false; return; }
        if (prev != dev && cudaSetDevice(dev) != cudaSuccess) ok = false;
    }
    ~DevScope() { if (prev >= 0) cudaSetDevice(prev); }
};

}  // namespace

extern "C" {

CkFftCudaPlan* CkFftCudaPlanJobs(CkFftContext* context, const CkFftCudaJob* jobs, int njobs)
{
    ContextView cv;
    if (!context_view(context, &cv)) { set_last_error("NULL or invalid context"); return nullptr; }
    DevScope scope(cv.device);
    if (!scope.ok) { set_last_error("cannot select the context's device"); return nullptr; }
    Built b;
    if (!build_units(cv, jobs, njobs, &b)) return nullptr;
    CkFftCudaPlan* p = new (std::nothrow) _CkFftCudaPlan();
    if (!p) { set_last_error("out of host memory"); return nullptr; }
    p->cv = cv;
    p->nunits = (int)b.units.size();
    p->nlarge = (int)b.large.size();
    p->algo_bytes = b.algo_bytes;
    p->transforms = b.transforms;
    p->work = !b.empty();
    const FrameDesc* dframes = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming);
    for (int i = 0; i < _CkFftCudaPlan::kBranches && e == cudaSuccess; ++i) {
        e = cudaStreamCreateWithFlags(&p->side[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->join[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess)
        e = upload(b, cv, &p->dmem, &p->scratch, &p->args, &p->counters_bytes, &dframes, p->stream, false);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    const long long counted = launch_count();       // launches counted while capturing are not run
    if (e == cudaSuccess && p->work) {
        e = cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            // grouped launches round-robin on the side branches, the
            // persistent kernel over the units on the main one
            cudaError_t e1 = cudaEventRecord(p->fork, p->stream);
            const int nb = (int)std::min<size_t>(b.groups.size(), _CkFftCudaPlan::kBranches);
            for (int i = 0; i < nb && e1 == cudaSuccess; ++i) e1 = cudaStreamWaitEvent(p->side[i], p->fork, 0);
            for (size_t g = 0; g < b.groups.size() && e1 == cudaSuccess; ++g) {
                const GroupSpec& G = b.groups[g];
                e1 = launch_group(G.op, G.log2a, dframes + G.first, G.count, cv.tw, p->scratch + G.scratch_off,
                                  G.scratch_bytes, p->side[g % _CkFftCudaPlan::kBranches]);
            }
            if (e1 == cudaSuccess) e1 = cudaMemsetAsync(p->args.done, 0, p->counters_bytes, p->stream);
            if (e1 == cudaSuccess && p->nunits > 0) e1 = launch_jobs(p->args, p->stream);
            for (int i = 0; i < nb && e1 == cudaSuccess; ++i) {
                e1 = cudaEventRecord(p->join[i], p->side[i]);
                if (e1 == cudaSuccess) e1 = cudaStreamWaitEvent(p->stream, p->join[i], 0);
            }
            cudaError_t e2 = e1;
            e = cudaStreamEndCapture(p->stream, &p->graph);
            if (e == cudaSuccess) e = e2;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&p->exec, p->graph, 0);
        count_launch((int)(counted - launch_count()));
        size_t nn = 0;
        if (e == cudaSuccess) e = cudaGraphGetNodes(p->graph, nullptr, &nn);
        std::vector<cudaGraphNode_t> nodes(nn);
        if (e == cudaSuccess && nn) e = cudaGraphGetNodes(p->graph, nodes.data(), &nn);
        for (size_t i = 0; i < nn && e == cudaSuccess; ++i) {
            cudaGraphNodeType t;
            e = cudaGraphNodeGetType(nodes[i], &t);
            if (e == cudaSuccess && t == cudaGraphNodeTypeKernel) ++p->kernels;
        }
    }
    if (e != cudaSuccess) {
        fail_cuda("planning the job run", e);
        CkFftCudaDestroyPlan(p);
        return nullptr;
    }
    return p;
}

int CkFftCudaExecPlan(CkFftCudaPlan* p, void* stream)
{
    if (!p) { set_last_error("NULL plan"); return 0; }
    if (!p->work) return 1;
    DevScope scope(p->cv.device);
    if (!scope.ok) { set_last_error("cannot select the plan's device"); return 0; }
    cudaStream_t s = stream ? (cudaStream_t)stream : p->stream;
    cudaError_t e = cudaGraphLaunch(p->exec, s);
    if (e != cudaSuccess) return fail_cuda("cudaGraphLaunch", e);
    count_launch(p->kernels);
    if (!stream) {
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return fail_cuda("cudaStreamSynchronize", e);
        if (take_device_error()) { set_last_error("a job kernel wait timed out"); return 0; }
    }
    return 1;
}

void CkFftCudaDestroyPlan(CkFftCudaPlan* p)
{
    if (!p) return;
    DevScope scope(p->cv.device);
    if (p->stream) cudaStreamSynchronize(p->stream);
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    cudaFree(p->dmem);
    cudaFree(p->scratch);
    for (int i = 0; i < _CkFftCudaPlan::kBranches; ++i) {
        if (p->side[i]) cudaStreamDestroy(p->side[i]);
        if (p->join[i]) cudaEventDestroy(p->join[i]);
    }
    if (p->fork) cudaEventDestroy(p->fork);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
}

long long CkFftCudaPlanBytes(const CkFftCudaPlan* p) { return p ? p->algo_bytes : 0; }

int CkFftCudaRunJobs(CkFftContext* context, const CkFftCudaJob* jobs, int njobs, void* stream)
{
    ContextView cv;
    if (!context_view(context, &cv)) { set_last_error("NULL or invalid context"); return 0; }
    DevScope scope(cv.device);
    if (!scope.ok) { set_last_error("cannot select the context's device"); return 0; }
    Built b;
    if (!build_units(cv, jobs, njobs, &b)) return 0;
    if (b.empty()) return 1;
    cudaStream_t s = (cudaStream_t)stream;
    void* dmem = nullptr;
    float2* scratch = nullptr;
    JobsArgs a{};
    size_t cb = 0;
    const FrameDesc* dframes = nullptr;
    cudaError_t e = upload(b, cv, &dmem, &scratch, &a, &cb, &dframes, s, true);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.done, 0, cb, s);
    if (e == cudaSuccess) e = launch_groups(b, dframes, scratch, cv.tw, s);
    if (e == cudaSuccess && !b.units.empty()) {
        e = launch_jobs(a, s);
        if (e == cudaSuccess) count_launch();
    }
    if (dmem) cudaFreeAsync(dmem, s);
    if (scratch) cudaFreeAsync(scratch, s);
    if (e != cudaSuccess) return fail_cuda("job run", e);
    if (!stream) {
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return fail_cuda("cudaStreamSynchronize", e);
        if (take_device_error()) { set_last_error("a job kernel wait timed out"); return 0; }
    }
    return 1;
}

}  // extern "C"
