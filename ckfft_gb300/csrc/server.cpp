// server.cpp -- continuous-batching request server over the persistent job kernel.
//
// Clients submit jobs (device or host buffers) at any time; a dispatcher thread owns
// the GPU side.  It keeps up to `max_inflight` runs on the device at once,
// each on its own stream with resident descriptor buffers, pinned staging and
// a scratch arena.  Whenever a run slot is free and requests are waiting it
// admits them in arrival order -- while their multi-pass scratch fits the
// slot's arena, up to a request cap -- and launches them as one run of the
// job kernel.  A request larger than an arena is admitted alone once free
// HBM (cudaMemGetInfo) covers its scratch, which then comes from the
// library's stream-ordered pool.  Requests that arrive while earlier runs are
// still on the GPU therefore start as soon as a slot frees up and their work
// overlaps the runs already in flight.  Requests whose algorithmic bytes reach
// `direct_threshold_bytes` already fill the GPU on their own: they skip
// batching and go to one of two direct lanes (the batched entry points on a
// lane stream), so a small request never waits behind a large one inside a
// run.  Requests may hold host buffers: their inputs are copied into a
// device staging buffer owned by the run slot (or lane) on that slot's
// stream before the kernels, and their outputs copied back after them, so
// the copies of one run overlap the kernels of the others; the staging
// buffers grow to the largest run seen and then stay resident.  Completion
// is detected by polling each run's or lane's event (recorded after the
// output copies); latency is measured from submission (or scheduled arrival,
// for trace replays) to the dispatcher observing the completion.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "ckfft_cuda.h"
#include "jobs.h"
#include "kernels.h"

namespace {

using Clock = std::chrono::steady_clock;

double seconds_between(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double>(b - a).count();
}

struct Request {
    CkFftCudaJob job;           // as submitted
    bool host_in = false;       // input / output outside the device: staged
    bool host_out = false;
    long long in_bytes = 0;
    long long out_bytes = 0;
    long long ticket;
    Clock::time_point t0;       // submission or scheduled arrival
    long long scratch;          // bytes of multi-pass intermediates
    long long bytes;            // algorithmic bytes
};

struct Result {
    bool done = false;
    bool ok = false;
    double latency = 0.0;
};

// Device staging for the host-side buffers of the requests in one run.
struct Stage {
    void* buf = nullptr;
    size_t cap = 0;
};

struct Slot {
    ckg::RunSlot run;
    Stage stage;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev = nullptr;
    bool busy = false;
    float2* pooled = nullptr;   // oversized scratch for this run, stream-ordered
    std::vector<Request> reqs;
};

// A direct lane runs one large request at a time through the batched entry
// points (one launch, or two or three for multi-pass sizes) on its own stream.
struct Lane {
    Stage stage;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev = nullptr;
    bool busy = false;
    std::vector<Request> reqs;   // zero or one
};

constexpr int kMaxRequestsPerRun = 4096;
constexpr int kDirectLanes = 2;
// Staged (host-side) bytes one run admits; a single larger request runs alone.
constexpr long long kStageBytesPerRun = 1ll << 30;

long long staged_bytes(const Request& r)
{
    auto up = [](long long b) { return (b + 255) / 256 * 256; };
    return (r.host_in ? up(r.in_bytes) : 0) + (r.host_out ? up(r.out_bytes) : 0);
}

// Copies the host-side inputs of `reqs` into the stage on `st` and points the
// jobs at the staged copies (inputs and outputs).  The stage grows when
// needed; the caller's stream is idle then (the slot or lane is free).
cudaError_t stage_inputs(const std::vector<Request>& reqs, std::vector<CkFftCudaJob>& jobs, Stage* stage,
                         cudaStream_t st)
{
    size_t need = 0;
    for (const Request& r : reqs) need += (size_t)staged_bytes(r);
    if (need == 0) return cudaSuccess;
    if (need > stage->cap) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return e;
        cudaFree(stage->buf);
        stage->buf = nullptr;
        stage->cap = 0;
        if ((e = ckg::dev_malloc(&stage->buf, need)) != cudaSuccess) return e;
        stage->cap = need;
    }
    char* p = (char*)stage->buf;
    for (size_t i = 0; i < reqs.size(); ++i) {
        const Request& r = reqs[i];
        if (r.host_in) {
            cudaError_t e = cudaMemcpyAsync(p, r.job.input, (size_t)r.in_bytes, cudaMemcpyHostToDevice, st);
            if (e != cudaSuccess) return e;
            jobs[i].input = p;
            p += (r.in_bytes + 255) / 256 * 256;
        }
        if (r.host_out) {
            jobs[i].output = p;
            p += (r.out_bytes + 255) / 256 * 256;
        }
    }
    return cudaSuccess;
}

// Copies the staged outputs back to the requests' host buffers on `st`.
cudaError_t stage_outputs(const std::vector<Request>& reqs, const std::vector<CkFftCudaJob>& jobs, cudaStream_t st)
{
    for (size_t i = 0; i < reqs.size(); ++i) {
        const Request& r = reqs[i];
        if (!r.host_out) continue;
        cudaError_t e = cudaMemcpyAsync(r.job.output, jobs[i].output, (size_t)r.out_bytes, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace

struct _CkFftCudaServer {
    ckg::ContextView cv{};
    CkFftContext* ctx = nullptr;
    size_t arena = 0;
    long long direct_bytes = 0;     // requests this large skip batching
    std::vector<Slot> slots;
    std::vector<Lane> lanes;
    std::mutex mu;
    std::condition_variable cv_pending;
    std::condition_variable cv_done;
    std::deque<Request> pending;    // batched
    std::deque<Request> direct;     // direct lanes
    std::unordered_map<long long, Result> results;
    std::thread dispatcher;
    std::atomic<bool> stop{false};
    long long next_ticket = 1;
    long long completed = 0;
    double algo_bytes = 0.0;
};

namespace {

struct DevScope {
    int prev = -1;
    explicit DevScope(int dev)
    {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
    }
    ~DevScope() { if (prev >= 0) cudaSetDevice(prev); }
};

void complete(CkFftCudaServer* s, std::vector<Request>& reqs, bool ok)
{
    const Clock::time_point now = Clock::now();
    {
        std::lock_guard<std::mutex> lock(s->mu);
        for (const Request& r : reqs) {
            Result& res = s->results[r.ticket];
            res.done = true;
            res.ok = ok;
            res.latency = seconds_between(r.t0, now);
            s->completed += 1;
            s->algo_bytes += (double)r.bytes;
        }
    }
    reqs.clear();
    s->cv_done.notify_all();
}

// Enqueues a large request through the batched entry points.
bool enqueue_direct(CkFftCudaServer* s, const CkFftCudaJob& j, cudaStream_t st)
{
    switch (j.kind) {
    case CKFFT_CUDA_COMPLEX_FORWARD:
        return CkFftCudaComplexForwardBatch(s->ctx, j.n, j.count, (const CkFftComplex*)j.input, (CkFftComplex*)j.output, st);
    case CKFFT_CUDA_COMPLEX_INVERSE:
        return CkFftCudaComplexInverseBatch(s->ctx, j.n, j.count, (const CkFftComplex*)j.input, (CkFftComplex*)j.output, st);
    case CKFFT_CUDA_REAL_FORWARD:
        return CkFftCudaRealForwardBatch(s->ctx, j.n, j.count, (const float*)j.input, (CkFftComplex*)j.output, st);
    default:
        return CkFftCudaRealInverseBatch(s->ctx, j.n, j.count, (const CkFftComplex*)j.input, (float*)j.output, st);
    }
}

void finish_slot(CkFftCudaServer* s, Slot& sl, bool ok)
{
    const Clock::time_point now = Clock::now();
    if (sl.pooled) {
        cudaFreeAsync(sl.pooled, sl.stream);
        sl.pooled = nullptr;
    }
    {
        std::lock_guard<std::mutex> lock(s->mu);
        for (const Request& r : sl.reqs) {
            Result& res = s->results[r.ticket];
            res.done = true;
            res.ok = ok;
            res.latency = seconds_between(r.t0, now);
            s->completed += 1;
            s->algo_bytes += (double)r.bytes;
        }
    }
    sl.reqs.clear();
    sl.busy = false;
    s->cv_done.notify_all();
}

// Takes the requests the next run admits (lock held).
std::vector<Request> admit(CkFftCudaServer* s, bool* oversized)
{
    std::vector<Request> out;
    *oversized = false;
    long long scratch = 0, staged = 0;
    while (!s->pending.empty() && (int)out.size() < kMaxRequestsPerRun) {
        const Request& r = s->pending.front();
        if (!out.empty() && staged + staged_bytes(r) > kStageBytesPerRun) break;
        if (scratch + r.scratch > (long long)s->arena) {
            if (!out.empty()) break;
            // alone and larger than an arena: admit if free HBM covers it
            size_t free_b = 0, total_b = 0;
            if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess || (size_t)r.scratch + (256ull << 20) > free_b) break;
            *oversized = true;
            out.push_back(r);
            s->pending.pop_front();
            break;
        }
        scratch += r.scratch;
        staged += staged_bytes(r);
        out.push_back(r);
        s->pending.pop_front();
    }
    return out;
}

void dispatch_loop(CkFftCudaServer* s)
{
    DevScope scope(s->cv.device);
    std::vector<CkFftCudaJob> jobs;
    while (true) {
        bool progressed = false;
        int busy = 0;
        // direct lanes: completions, then the next large request
        for (Lane& ln : s->lanes) {
            if (ln.busy) {
                const cudaError_t q = cudaEventQuery(ln.ev);
                if (q == cudaErrorNotReady) {
                    ++busy;
                    continue;
                }
                if (q != cudaSuccess) cudaGetLastError();
                complete(s, ln.reqs, q == cudaSuccess && ckg::take_device_error() == 0);
                ln.busy = false;
                progressed = true;
            }
            Request r;
            {
                std::lock_guard<std::mutex> lock(s->mu);
                if (s->direct.empty()) continue;
                r = s->direct.front();
                s->direct.pop_front();
            }
            ln.reqs.assign(1, r);
            std::vector<CkFftCudaJob> one(1, r.job);
            if (stage_inputs(ln.reqs, one, &ln.stage, ln.stream) == cudaSuccess && enqueue_direct(s, one[0], ln.stream) &&
                stage_outputs(ln.reqs, one, ln.stream) == cudaSuccess && cudaEventRecord(ln.ev, ln.stream) == cudaSuccess) {
                ln.busy = true;
                ++busy;
            } else {
                complete(s, ln.reqs, false);
            }
            progressed = true;
        }
        for (Slot& sl : s->slots) {
            if (!sl.busy) continue;
            const cudaError_t q = cudaEventQuery(sl.ev);
            if (q == cudaSuccess) {
                finish_slot(s, sl, ckg::take_device_error() == 0);
                progressed = true;
            } else if (q != cudaErrorNotReady) {
                cudaGetLastError();
                finish_slot(s, sl, false);
                progressed = true;
            } else {
                ++busy;
            }
        }
        for (Slot& sl : s->slots) {
            if (sl.busy) continue;
            std::vector<Request> batch;
            bool oversized = false;
            {
                std::lock_guard<std::mutex> lock(s->mu);
                batch = admit(s, &oversized);
            }
            if (batch.empty()) break;
            jobs.clear();
            long long scratch = 0;
            for (const Request& r : batch) {
                jobs.push_back(r.job);
                scratch += r.scratch;
            }
            sl.reqs = std::move(batch);
            float2* override_scratch = nullptr;
            size_t override_bytes = 0;
            bool ok = true;
            if (oversized) {
                ok = ckg::pool_alloc_async((void**)&sl.pooled, (size_t)scratch, sl.stream) == cudaSuccess;
                override_scratch = sl.pooled;
                override_bytes = (size_t)scratch;
            } else if (scratch) {
                override_scratch = sl.run.scratch;
                override_bytes = sl.run.scratch_cap;
            }
            ok = ok && stage_inputs(sl.reqs, jobs, &sl.stage, sl.stream) == cudaSuccess;
            const int rc = ok ? ckg::enqueue_run(s->cv, jobs.data(), (int)jobs.size(), &sl.run, sl.stream, override_scratch,
                                                 override_bytes)
                              : -1;
            if (rc == 1 && stage_outputs(sl.reqs, jobs, sl.stream) == cudaSuccess &&
                cudaEventRecord(sl.ev, sl.stream) == cudaSuccess) {
                sl.busy = true;
                ++busy;
            } else {
                finish_slot(s, sl, false);
            }
            progressed = true;
        }
        if (s->stop.load() && busy == 0) {
            std::lock_guard<std::mutex> lock(s->mu);
            if (s->pending.empty() && s->direct.empty()) break;
        }
        if (!progressed) {
            if (busy) {
                std::this_thread::yield();
            } else {
                std::unique_lock<std::mutex> lock(s->mu);
                s->cv_pending.wait_for(lock, std::chrono::milliseconds(1),
                                       [&] { return !s->pending.empty() || !s->direct.empty() || s->stop.load(); });
            }
        }
    }
}

long long submit(CkFftCudaServer* s, const CkFftCudaJob& job, Clock::time_point t0)
{
    if (!ckg::validate_job(s->cv, job, 0, true)) return 0;
    Request r;
    r.job = job;
    if (job.count > 0) {
        r.host_in = ckg::job_host_side(s->cv, job.input);
        r.host_out = ckg::job_host_side(s->cv, job.output);
        r.in_bytes = ckg::job_in_bytes(job);
        r.out_bytes = ckg::job_out_bytes(job);
    }
    r.t0 = t0;
    r.scratch = ckg::job_scratch_bytes(job);
    r.bytes = ckg::job_algo_bytes(job);
    {
        std::lock_guard<std::mutex> lock(s->mu);
        r.ticket = s->next_ticket++;
        s->results[r.ticket] = Result{};
        if (s->direct_bytes > 0 && r.bytes >= s->direct_bytes) s->direct.push_back(r);
        else s->pending.push_back(r);
    }
    s->cv_pending.notify_one();
    return r.ticket;
}

bool wait_ticket(CkFftCudaServer* s, long long ticket, double timeout_s, Result* out)
{
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->results.find(ticket);
    if (it == s->results.end()) return false;
    auto ready = [&] { return s->results[ticket].done; };
    if (timeout_s < 0) {
        s->cv_done.wait(lock, ready);
    } else if (!s->cv_done.wait_for(lock, std::chrono::duration<double>(timeout_s), ready)) {
        return false;
    }
    *out = s->results[ticket];
    s->results.erase(ticket);
    return true;
}

void fill_stats(const std::vector<double>& lat, double seconds, double bytes, CkFftCudaServeStats* st)
{
    if (!st) return;
    std::vector<double> v(lat);
    std::sort(v.begin(), v.end());
    auto pct = [&](double p) {
        if (v.empty()) return 0.0;
        size_t i = (size_t)(p * (double)(v.size() - 1) + 0.5);
        return v[std::min(i, v.size() - 1)];
    };
    st->requests = (long long)v.size();
    st->seconds = seconds;
    st->algo_bytes = bytes;
    st->p50_s = pct(0.50);
    st->p99_s = pct(0.99);
    st->p999_s = pct(0.999);
    st->max_s = v.empty() ? 0.0 : v.back();
}

void spin_until(Clock::time_point t)
{
    while (Clock::now() < t) {
    }
}

}  // namespace

extern "C" {

CkFftCudaServer* CkFftCudaServerCreate(CkFftContext* context, size_t scratch_budget_bytes, int max_inflight,
                                       long long direct_threshold_bytes)
{
    ckg::ContextView cv;
    if (!ckg::context_view(context, &cv)) { ckg::set_last_error("NULL or invalid context"); return nullptr; }
    if (max_inflight < 1 || max_inflight > 16) { ckg::set_last_error("max_inflight must be 1..16"); return nullptr; }
    DevScope scope(cv.device);
    CkFftCudaServer* s = new (std::nothrow) _CkFftCudaServer();
    if (!s) { ckg::set_last_error("out of host memory"); return nullptr; }
    s->cv = cv;
    s->ctx = context;
    s->arena = scratch_budget_bytes / (size_t)max_inflight / 16 * 16;
    s->direct_bytes = direct_threshold_bytes;
    s->slots.resize(max_inflight);
    s->lanes.resize(direct_threshold_bytes > 0 ? kDirectLanes : 0);
    cudaError_t e = cudaSuccess;
    for (Lane& ln : s->lanes) {
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ln.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ln.ev, cudaEventDisableTiming);
    }
    for (Slot& sl : s->slots) {
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming);
        // resident buffers: scratch arena, and descriptor space for large runs
        if (e == cudaSuccess && s->arena) {
            e = ckg::dev_malloc((void**)&sl.run.scratch, s->arena);
            if (e == cudaSuccess) sl.run.scratch_cap = s->arena;
        }
        if (e == cudaSuccess) {
            const size_t desc = 8u << 20;
            e = ckg::dev_malloc(&sl.run.dev, desc);
            if (e == cudaSuccess) sl.run.dev_cap = desc;
            if (e == cudaSuccess) e = cudaHostAlloc((void**)&sl.run.host, desc, cudaHostAllocDefault);
            if (e == cudaSuccess) sl.run.host_cap = desc;
        }
    }
    if (e != cudaSuccess) {
        ckg::set_last_error(cudaGetErrorString(e));
        for (Lane& ln : s->lanes) {
            if (ln.ev) cudaEventDestroy(ln.ev);
            if (ln.stream) cudaStreamDestroy(ln.stream);
        }
        for (Slot& sl : s->slots) {
            ckg::free_run_slot(&sl.run);
            if (sl.ev) cudaEventDestroy(sl.ev);
            if (sl.stream) cudaStreamDestroy(sl.stream);
        }
        delete s;
        return nullptr;
    }
    s->dispatcher = std::thread(dispatch_loop, s);
    return s;
}

void CkFftCudaServerDestroy(CkFftCudaServer* s)
{
    if (!s) return;
    s->stop.store(true);
    s->cv_pending.notify_all();
    if (s->dispatcher.joinable()) s->dispatcher.join();
    DevScope scope(s->cv.device);
    for (Slot& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        ckg::free_run_slot(&sl.run);
        cudaFree(sl.stage.buf);
        if (sl.ev) cudaEventDestroy(sl.ev);
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    for (Lane& ln : s->lanes) {
        if (ln.stream) cudaStreamSynchronize(ln.stream);
        cudaFree(ln.stage.buf);
        if (ln.ev) cudaEventDestroy(ln.ev);
        if (ln.stream) cudaStreamDestroy(ln.stream);
    }
    delete s;
}

long long CkFftCudaServerSubmit(CkFftCudaServer* s, const CkFftCudaJob* job)
{
    if (!s || !job) { ckg::set_last_error("NULL server or job"); return 0; }
    return submit(s, *job, Clock::now());
}

int CkFftCudaServerWait(CkFftCudaServer* s, long long ticket, double timeout_s, double* latency_s)
{
    if (!s) { ckg::set_last_error("NULL server"); return 0; }
    Result r;
    if (!wait_ticket(s, ticket, timeout_s, &r)) { ckg::set_last_error("unknown ticket or timeout"); return 0; }
    if (latency_s) *latency_s = r.latency;
    if (!r.ok) { ckg::set_last_error("the run holding this request failed"); return 0; }
    return 1;
}

int CkFftCudaServerReplay(CkFftCudaServer* s, const CkFftCudaRequest* reqs, int n, double* latency_s,
                          CkFftCudaServeStats* stats)
{
    if (!s || n < 0 || (n > 0 && !reqs)) { ckg::set_last_error("invalid replay arguments"); return 0; }
    std::vector<long long> tickets(n);
    const Clock::time_point start = Clock::now() + std::chrono::milliseconds(2);
    double bytes = 0.0;
    for (int i = 0; i < n; ++i) {
        const Clock::time_point t = start + std::chrono::duration_cast<Clock::duration>(
                                                std::chrono::duration<double>(reqs[i].arrival_s));
        spin_until(t);
        tickets[i] = submit(s, reqs[i].job, t);
        if (!tickets[i]) return 0;
        bytes += (double)ckg::job_algo_bytes(reqs[i].job);
    }
    std::vector<double> lat(n);
    bool ok = true;
    for (int i = 0; i < n; ++i) {
        Result r;
        if (!wait_ticket(s, tickets[i], -1.0, &r) || !r.ok) ok = false;
        lat[i] = r.latency;
        if (latency_s) latency_s[i] = r.latency;
    }
    const double secs = seconds_between(start, Clock::now());
    fill_stats(lat, secs, bytes, stats);
    if (!ok) { ckg::set_last_error("a run failed during the replay"); return 0; }
    return 1;
}

int CkFftCudaReplayPerRequest(CkFftContext* context, const CkFftCudaRequest* reqs, int n, double* latency_s,
                              CkFftCudaServeStats* stats)
{
    ckg::ContextView cv;
    if (!ckg::context_view(context, &cv)) { ckg::set_last_error("NULL or invalid context"); return 0; }
    if (n < 0 || (n > 0 && !reqs)) { ckg::set_last_error("invalid replay arguments"); return 0; }
    DevScope scope(cv.device);
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
        ckg::set_last_error("cannot create a stream");
        return 0;
    }
    std::vector<double> lat(n);
    const Clock::time_point start = Clock::now() + std::chrono::milliseconds(2);
    double bytes = 0.0;
    int ok = 1;
    for (int i = 0; i < n && ok; ++i) {
        const Clock::time_point t = start + std::chrono::duration_cast<Clock::duration>(
                                                std::chrono::duration<double>(reqs[i].arrival_s));
        spin_until(t);
        const CkFftCudaJob& j = reqs[i].job;
        switch (j.kind) {
        case CKFFT_CUDA_COMPLEX_FORWARD:
            ok = CkFftCudaComplexForwardBatch(context, j.n, j.count, (const CkFftComplex*)j.input, (CkFftComplex*)j.output, st);
            break;
        case CKFFT_CUDA_COMPLEX_INVERSE:
            ok = CkFftCudaComplexInverseBatch(context, j.n, j.count, (const CkFftComplex*)j.input, (CkFftComplex*)j.output, st);
            break;
        case CKFFT_CUDA_REAL_FORWARD:
            ok = CkFftCudaRealForwardBatch(context, j.n, j.count, (const float*)j.input, (CkFftComplex*)j.output, st);
            break;
        default:
            ok = CkFftCudaRealInverseBatch(context, j.n, j.count, (const CkFftComplex*)j.input, (float*)j.output, st);
            break;
        }
        if (ok && cudaStreamSynchronize(st) != cudaSuccess) ok = 0;
        lat[i] = seconds_between(t, Clock::now());
        if (latency_s) latency_s[i] = lat[i];
        bytes += (double)ckg::job_algo_bytes(j);
    }
    const double secs = seconds_between(start, Clock::now());
    cudaStreamDestroy(st);
    fill_stats(lat, secs, bytes, stats);
    return ok;
}

}  // extern "C"
