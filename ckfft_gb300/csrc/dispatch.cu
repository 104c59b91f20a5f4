// dispatch.cu -- routes a launch request to the kernel family for its size.
#include <atomic>
#include <cstdlib>
#include <mutex>
#include "kernels.h"
#include "tuning_table.h"

namespace ckg {

cudaError_t launch_small_c2c(bool inv, int log2n, const void* in, void* out, long long count,
                             long long in_dist, long long out_dist, const float2* tw, cudaStream_t s);
cudaError_t launch_small_real(bool inv, int log2n, const void* in, void* out, long long count,
                              long long in_dist, long long out_dist, const float2* tw, cudaStream_t s);
cudaError_t prepare_small_c2c();
cudaError_t prepare_small_real();
cudaError_t prepare_large();
cudaError_t prepare_jobs();
cudaError_t prepare_cluster();
cudaError_t prepare_strided();
cudaError_t prepare_fused();
cudaError_t prepare_inter();
cudaError_t prepare_l2pass();
cudaError_t prepare_groups();
cudaError_t prepare_shape_halfr();
cudaError_t prepare_shape_doubler();
cudaError_t prepare_shape_cta512();
cudaError_t prepare_shape_cta128();
#define CKG_SHAPE_DECL(name)                                                                                     \
    cudaError_t launch_shape_##name(Kind kind, int log2c, const void* in, void* out, long long count,          \
                                    long long in_dist, long long out_dist, const float2* tw, cudaStream_t s,   \
                                    bool* done);
CKG_SHAPE_DECL(halfr)
CKG_SHAPE_DECL(doubler)
CKG_SHAPE_DECL(cta512)
CKG_SHAPE_DECL(cta128)
#undef CKG_SHAPE_DECL
cudaError_t prepare_noalloc();
cudaError_t prepare_mid();

// Opt-in (CKFFT_CUDA_CLUSTER=1): measured slower than the default paths on
// GB300 (2^14: 2366 vs 3669 GB/s single CTA; 2^15 / 2^16: 1936 / 1516 vs about
// 2810 GB/s in two passes), because the cluster exchanges cost more than the
// HBM pass they save.
bool cluster_enabled()
{
    static const bool on = [] {
        const char* v = std::getenv("CKFFT_CUDA_CLUSTER");
        return v && v[0] == '1';
    }();
    return on;
}

// Opt-in (CKFFT_CUDA_MID=1): the persistent kernel of fft_mid.cu for complex
// 2^15 / 2^16.  Measured on GB300 (batches of 1 GiB, GB/s) against the
// cluster two-pass kernel of fft_l2pass.cu that runs these sizes by default:
// 2^15 3201 vs 3313, 2^16 3189 vs 3491 (earlier builds of it measured up to
// 3529 / 3429); both are bound by the two passes' instructions, and the
// persistent form, holding a whole SM per CTA, also keeps other kernels of a
// mixed run off its SMs (the uneven batch fell from 3217 to 2983 GB/s with
// its grouped 2^15 launches on it).
bool mid_enabled(int log2n)
{
    static const bool on = [] {
        const char* v = std::getenv("CKFFT_CUDA_MID");
        return v && v[0] == '1';
    }();
    return on && mid_supported(log2n);
}

static std::atomic<long long> g_launches{0};

long long launch_count() { return g_launches.load(std::memory_order_relaxed); }
void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

cudaError_t launch_small(Kind kind, int log2n, const void* in, void* out, long long count,
                         long long in_dist, long long out_dist, const float2* tw, cudaStream_t s)
{
    if (count <= 0) return cudaSuccess;
    cudaError_t e;
    switch (kind) {
    case C2C_FWD: e = launch_small_c2c(false, log2n, in, out, count, in_dist, out_dist, tw, s); break;
    case C2C_INV: e = launch_small_c2c(true, log2n, in, out, count, in_dist, out_dist, tw, s); break;
    case R2C: e = launch_small_real(false, log2n, in, out, count, in_dist, out_dist, tw, s); break;
    case C2R: e = launch_small_real(true, log2n, in, out, count, in_dist, out_dist, tw, s); break;
    default: e = cudaErrorInvalidValue;
    }
    return e;
}

cudaError_t launch_small_shape(Kind kind, int v, int log2c, const void* in, void* out, long long count,
                               long long in_dist, long long out_dist, const float2* tw, cudaStream_t s, bool* done)
{
    switch (v) {
    case 4: return launch_shape_halfr(kind, log2c, in, out, count, in_dist, out_dist, tw, s, done);
    case 5: return launch_shape_doubler(kind, log2c, in, out, count, in_dist, out_dist, tw, s, done);
    case 6: return launch_shape_cta512(kind, log2c, in, out, count, in_dist, out_dist, tw, s, done);
    case 7: return launch_shape_cta128(kind, log2c, in, out, count, in_dist, out_dist, tw, s, done);
    default: *done = false; return cudaSuccess;
    }
}

static thread_local int t_plain_loads = 0;

PlainLoadsScope::PlainLoadsScope() : prev(t_plain_loads) { t_plain_loads = 1; }
PlainLoadsScope::~PlainLoadsScope() { t_plain_loads = prev; }

int variant_for(Kind kind, int log2c)
{
    if (t_plain_loads) return 0;
    static const int forced = [] {
        const char* v = std::getenv("CKFFT_CUDA_VARIANT");
        if (!v || !*v) return -1;
        const int x = std::atoi(v);
        return (x == 0 || (x >= 2 && x <= 8)) ? x : -1;
    }();
    if (forced >= 0) return forced;
    if (kind < 0 || kind > 3 || log2c < 0 || log2c > 14) return 0;
    return kTunedVariant[kind][log2c];
}

static std::mutex g_err_mu;
static unsigned* g_err_host[64] = {};
static unsigned* g_err_dev[64] = {};

unsigned* device_error_word()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    return g_err_dev[dev];
}

unsigned take_device_error()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64 || !g_err_host[dev]) return 0;
    volatile unsigned* h = g_err_host[dev];
    const unsigned v = *h;
    if (v) *h = 0;
    return v;
}

static cudaMemPool_t g_pool[64] = {};

static cudaError_t prepare_pool(int dev)
{
    std::lock_guard<std::mutex> lock(g_err_mu);
    if (dev < 0 || dev >= 64 || g_pool[dev]) return cudaSuccess;
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool;
    cudaError_t e = cudaMemPoolCreate(&pool, &props);
    if (e != cudaSuccess) return e;
    unsigned long long keep = ~0ull;
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    if (e != cudaSuccess) {
        cudaMemPoolDestroy(pool);
        return e;
    }
    g_pool[dev] = pool;
    return cudaSuccess;
}

// CKFFT_CUDA_FAIL_ALLOC=k: the k-th device allocation the library requests
// (counting from 1 over every allocation site) fails with
// cudaErrorMemoryAllocation -- one injected failure per process, for tests of
// the failure paths.  Unset or 0: off.
bool injected_alloc_failure()
{
    static const long long target = [] {
        const char* v = std::getenv("CKFFT_CUDA_FAIL_ALLOC");
        return v ? std::atoll(v) : 0ll;
    }();
    if (target <= 0) return false;
    static std::atomic<long long> seen{0};
    return seen.fetch_add(1, std::memory_order_relaxed) + 1 == target;
}

cudaError_t dev_malloc(void** p, size_t bytes)
{
    if (injected_alloc_failure()) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes);
}

cudaError_t pool_alloc_async(void** p, size_t bytes, cudaStream_t s)
{
    if (injected_alloc_failure()) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64 || !g_pool[dev]) return cudaMallocAsync(p, bytes, s);
    return cudaMallocFromPoolAsync(p, bytes, g_pool[dev], s);
}

static cudaError_t prepare_error_word(int dev)
{
    std::lock_guard<std::mutex> lock(g_err_mu);
    if (dev < 0 || dev >= 64 || g_err_host[dev]) return cudaSuccess;
    void* h = nullptr;
    void* d = nullptr;
    cudaError_t e = cudaHostAlloc(&h, 64, cudaHostAllocMapped);
    if (e != cudaSuccess) return e;
    e = cudaHostGetDevicePointer(&d, h, 0);
    if (e != cudaSuccess) {
        cudaFreeHost(h);
        return e;
    }
    *(volatile unsigned*)h = 0;
    g_err_host[dev] = (unsigned*)h;
    g_err_dev[dev] = (unsigned*)d;
    return cudaSuccess;
}

cudaError_t prepare_device()
{
    static std::mutex mu;
    static unsigned long long done = 0;     // bit per device ordinal (< 64)
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 64 && (done >> dev) & 1ull) return cudaSuccess;
    if ((e = prepare_error_word(dev)) != cudaSuccess) return e;
    if ((e = prepare_pool(dev)) != cudaSuccess) return e;
    if ((e = prepare_small_c2c()) != cudaSuccess) return e;
    if ((e = prepare_small_real()) != cudaSuccess) return e;
    if ((e = prepare_large()) != cudaSuccess) return e;
    if ((e = prepare_jobs()) != cudaSuccess) return e;
    if ((e = prepare_cluster()) != cudaSuccess) return e;
    if ((e = prepare_strided()) != cudaSuccess) return e;
    if ((e = prepare_fused()) != cudaSuccess) return e;
    if ((e = prepare_inter()) != cudaSuccess) return e;
    if ((e = prepare_l2pass()) != cudaSuccess) return e;
    if ((e = prepare_groups()) != cudaSuccess) return e;
    if ((e = prepare_shape_halfr()) != cudaSuccess) return e;
    if ((e = prepare_shape_doubler()) != cudaSuccess) return e;
    if ((e = prepare_shape_cta512()) != cudaSuccess) return e;
    if ((e = prepare_shape_cta128()) != cudaSuccess) return e;
    if ((e = prepare_noalloc()) != cudaSuccess) return e;
    if ((e = prepare_mid()) != cudaSuccess) return e;
    if (dev < 64) done |= 1ull << dev;
    return cudaSuccess;
}

}  // namespace ckg
