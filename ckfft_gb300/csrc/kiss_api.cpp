// kiss_api.cpp -- kiss_fft's C interface (include/kiss_fft_cuda.h) on the
// C ABI of this library.
//
// kiss_fft 1.3.0 (ext/kiss_fft130/kiss_fft.c:339-408, tools/kiss_fftr.c:
// 27-159 of the reference tree) computes unscaled DFTs; in the scaling of
// the ckfft calls that is: complex forward / inverse unchanged, real forward
// = CkFftRealForward / 2 (the reference harness multiplies kiss by 2 to
// compare, src/test/test.cpp:368-372), real inverse = CkFftRealInverse.  The
// halving runs inside the transform kernel (CkFftCudaStft with scale 0.5,
// exact in binary floating point).
#include "kiss_fft_cuda.h"

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>

#include "ckfft_cuda.h"
#include "kernels.h"

struct kiss_fft_state {
    uint32_t magic;
    int nfft;
    int inverse;
    int own;
    CkFftContext* ctx;
};

struct kiss_fftr_state {
    kiss_fft_state s;
};

namespace {

constexpr uint32_t kComplexMagic = 0x4b495343u;   // "KISC"
constexpr uint32_t kRealMagic = 0x4b495352u;      // "KISR"

bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// The alloc protocol of kiss_fft.c:339-360 (mem / lenmem), then a context
// with the one direction the cfg runs.
kiss_fft_state* alloc_state(size_t need, int nfft, int inverse, void* mem, size_t* lenmem, uint32_t magic,
                            int min_n)
{
    kiss_fft_state* st = nullptr;
    int own = 0;
    if (!lenmem) {
        st = (kiss_fft_state*)std::malloc(need);
        own = 1;
    } else {
        if (mem && *lenmem >= need) st = (kiss_fft_state*)mem;
        *lenmem = need;
    }
    if (!st) return nullptr;
    if (!pow2(nfft) || nfft < min_n) {
        ckg::set_last_error(min_n > 1 ? "kiss_fftr_alloc: nfft must be a power of two >= 2"
                                      : "kiss_fft_alloc: nfft must be a power of two");
        if (own) std::free(st);
        return nullptr;
    }
    CkFftContext* ctx =
        CkFftInit(nfft, inverse ? kCkFftDirection_Inverse : kCkFftDirection_Forward, nullptr, nullptr);
    if (!ctx) {
        if (own) std::free(st);
        return nullptr;
    }
    st->magic = magic;
    st->nfft = nfft;
    st->inverse = inverse ? 1 : 0;
    st->own = own;
    st->ctx = ctx;
    return st;
}

void free_state(kiss_fft_state* st, uint32_t magic)
{
    if (!st || st->magic != magic) return;
    CkFftShutdown(st->ctx);
    st->ctx = nullptr;
    st->magic = 0;
    if (st->own) std::free(st);
}

bool is_device(const void* p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// A private buffer in the same kind of memory as `like` (host or device).
struct Temp {
    void* p = nullptr;
    bool dev = false;
    bool make(const void* like, size_t bytes)
    {
        dev = is_device(like);
        if (dev) {
            if (cudaMalloc(&p, bytes) != cudaSuccess) {
                cudaGetLastError();
                p = nullptr;
            }
        } else {
            p = std::malloc(bytes);
        }
        if (!p) ckg::set_last_error("kiss: cannot allocate a temporary buffer");
        return p != nullptr;
    }
    bool copy_from(const void* src, size_t bytes)
    {
        if (dev) return cudaMemcpy(p, src, bytes, cudaMemcpyDefault) == cudaSuccess;
        std::memcpy(p, src, bytes);
        return true;
    }
    bool copy_to(void* dst, size_t bytes) const
    {
        if (dev) return cudaMemcpy(dst, p, bytes, cudaMemcpyDefault) == cudaSuccess;
        std::memcpy(dst, p, bytes);
        return true;
    }
    ~Temp()
    {
        if (dev) cudaFree(p);
        else std::free(p);
    }
};

bool meet(const void* a, size_t na, const void* b, size_t nb)
{
    const uintptr_t a0 = (uintptr_t)a, b0 = (uintptr_t)b;
    return a0 < b0 + nb && b0 < a0 + na;
}

// Input that overlaps the output is read from a copy (kiss_fft allows
// fin == fout, kiss_fft.c:373-379).
const void* distinct_input(const void* in, size_t in_bytes, const void* out, size_t out_bytes, Temp* t)
{
    if (!meet(in, in_bytes, out, out_bytes)) return in;
    if (!t->make(in, in_bytes) || !t->copy_from(in, in_bytes)) return nullptr;
    return t->p;
}

bool check(const kiss_fft_state* st, uint32_t magic, const void* in, const void* out)
{
    if (!st || st->magic != magic) {
        ckg::set_last_error("kiss: NULL or invalid cfg");
        return false;
    }
    if (!in || !out) {
        ckg::set_last_error("kiss: NULL buffer");
        return false;
    }
    return true;
}

}  // namespace

extern "C" {

kiss_fft_cfg kiss_fft_alloc(int nfft, int inverse_fft, void* mem, size_t* lenmem)
{
    return alloc_state(sizeof(kiss_fft_state), nfft, inverse_fft, mem, lenmem, kComplexMagic, 1);
}

void kiss_fft_stride(kiss_fft_cfg cfg, const kiss_fft_cpx* fin, kiss_fft_cpx* fout, int fin_stride)
{
    if (!check(cfg, kComplexMagic, fin, fout)) return;
    if (fin_stride < 1) {
        ckg::set_last_error("kiss_fft_stride: fin_stride must be >= 1");
        return;
    }
    const long long n = cfg->nfft;
    const size_t in_bytes = (size_t)((n - 1) * fin_stride + 1) * sizeof(kiss_fft_cpx);
    const size_t out_bytes = (size_t)n * sizeof(kiss_fft_cpx);
    Temp t;
    const void* src = distinct_input(fin, in_bytes, fout, out_bytes, &t);
    if (!src) return;
    const CkFftComplex* in = (const CkFftComplex*)src;
    CkFftComplex* out = (CkFftComplex*)fout;
    if (fin_stride == 1) {
        if (cfg->inverse) CkFftComplexInverse(cfg->ctx, cfg->nfft, in, out);
        else CkFftComplexForward(cfg->ctx, cfg->nfft, in, out);
    } else if (cfg->inverse) {
        CkFftCudaComplexInverseStrided(cfg->ctx, cfg->nfft, 1, in, fin_stride, 0, out, 1, n, nullptr);
    } else {
        CkFftCudaComplexForwardStrided(cfg->ctx, cfg->nfft, 1, in, fin_stride, 0, out, 1, n, nullptr);
    }
}

void kiss_fft(kiss_fft_cfg cfg, const kiss_fft_cpx* fin, kiss_fft_cpx* fout) { kiss_fft_stride(cfg, fin, fout, 1); }

void kiss_fft_free(kiss_fft_cfg cfg) { free_state(cfg, kComplexMagic); }

void kiss_fft_cleanup(void) {}

int kiss_fft_next_fast_size(int n)
{
    int p = 1;
    while (p < n && p < (1 << 30)) p <<= 1;
    return p;
}

kiss_fftr_cfg kiss_fftr_alloc(int nfft, int inverse_fft, void* mem, size_t* lenmem)
{
    return (kiss_fftr_cfg)alloc_state(sizeof(kiss_fftr_state), nfft, inverse_fft, mem, lenmem, kRealMagic, 2);
}

void kiss_fftr(kiss_fftr_cfg cfg, const kiss_fft_scalar* timedata, kiss_fft_cpx* freqdata)
{
    kiss_fft_state* st = cfg ? &cfg->s : nullptr;
    if (!check(st, kRealMagic, timedata, freqdata)) return;
    if (st->inverse) {
        ckg::set_last_error("kiss_fftr: the cfg was allocated for the inverse");
        return;
    }
    const int n = st->nfft;
    const size_t in_bytes = (size_t)n * sizeof(float), out_bytes = (size_t)(n / 2 + 1) * sizeof(kiss_fft_cpx);
    Temp ti, to;
    const float* src = (const float*)distinct_input(timedata, in_bytes, freqdata, out_bytes, &ti);
    if (!src) return;
    // the kernels store bins as 8-byte pairs
    CkFftComplex* dst = (CkFftComplex*)freqdata;
    const bool bounce = ((uintptr_t)freqdata & 7) != 0;
    if (bounce) {
        if (!to.make(freqdata, out_bytes)) return;
        dst = (CkFftComplex*)to.p;
    }
    if (CkFftCudaStft(st->ctx, n, 1, src, n, n, nullptr, 0.5f, dst, nullptr) && bounce) to.copy_to(freqdata, out_bytes);
}

void kiss_fftri(kiss_fftr_cfg cfg, const kiss_fft_cpx* freqdata, kiss_fft_scalar* timedata)
{
    kiss_fft_state* st = cfg ? &cfg->s : nullptr;
    if (!check(st, kRealMagic, freqdata, timedata)) return;
    if (!st->inverse) {
        ckg::set_last_error("kiss_fftri: the cfg was allocated for the forward transform");
        return;
    }
    const int n = st->nfft;
    const size_t in_bytes = (size_t)(n / 2 + 1) * sizeof(kiss_fft_cpx), out_bytes = (size_t)n * sizeof(float);
    Temp ti, to;
    const CkFftComplex* src = (const CkFftComplex*)distinct_input(freqdata, in_bytes, timedata, out_bytes, &ti);
    if (!src) return;
    float* dst = timedata;
    const bool bounce = ((uintptr_t)timedata & 7) != 0;
    if (bounce) {
        if (!to.make(timedata, out_bytes)) return;
        dst = (float*)to.p;
    }
    if (CkFftCudaFilterInverse(st->ctx, n, 1, src, nullptr, 1.0f, dst, nullptr) && bounce)
        to.copy_to(timedata, out_bytes);
}

void kiss_fftr_free(kiss_fftr_cfg cfg) { free_state(cfg ? &cfg->s : nullptr, kRealMagic); }

}  // extern "C"
