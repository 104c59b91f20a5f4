// ckfft_timing.cpp -- the reference's timing test (src/test/test.cpp:610-721)
// for Linux, on this library.
//
// For n = 4096, 2048, ..., 256 it times the four tests of the reference,
// fft_<n>, fft_inv_<n>, fft_real_<n>, fft_inv_real_<n> (the inverse tests
// take the forward test's output as input, as the reference does), 500 runs
// per tester, and records the median milliseconds per transform in
// results_linux_<machine>.xml in the reference's layout:
//
//   <ckfft_test><fft_4096><ckfft time="..." /><ckfft_kiss_api time="..." />...</fft_4096>...</ckfft_test>
//
// Testers (one transform per call unless noted):
//   ckfft         the reference-named calls on host (pageable) buffers, the
//                 reference harness's usage (src/test/test.cpp:269-297);
//   ckfft_device  the same calls on device buffers;
//   ckfft_kiss_api the kiss_fft-compatible calls of this library on host
//                 buffers (the reference harness's second tester,
//                 src/test/test.cpp:315-395);
//   ckfft_batch   CkFftCuda*Batch of 4096 transforms on device buffers,
//                 time per transform.
// The console table has the reference's columns (median, min, max, norm to
// ckfft, change against a previous results file given with --prev).
//
//   ckfft_timing [--out DIR] [--input FILE] [--prev FILE] [--reps N]
//
// --input reads "real imag" pairs (the reference's input.txt format,
// src/test/test.cpp:90-107); without it the input is 4096 seeded values
// uniform in [-1, 1).
#include <cuda_runtime.h>
#include <sys/utsname.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <random>
#include <string>
#include <vector>

#include "ckfft_cuda.h"
#include "kiss_fft_cuda.h"

namespace {

struct Stats {
    std::vector<float> v;
    void sample(float x) { v.push_back(x); }
    float median()
    {
        std::sort(v.begin(), v.end());
        const size_t n = v.size();
        return n % 2 ? v[n / 2] : 0.5f * (v[n / 2] + v[n / 2 - 1]);
    }
    float min() const { return *std::min_element(v.begin(), v.end()); }
    float max() const { return *std::max_element(v.begin(), v.end()); }
};

[[noreturn]] void die(const char* what)
{
    std::fprintf(stderr, "ckfft_timing: %s: %s\n", what, CkFftCudaGetLastError());
    std::exit(1);
}

void check(int ok, const char* what)
{
    if (!ok) die(what);
}

void cuda_check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) {
        std::fprintf(stderr, "ckfft_timing: %s: %s\n", what, cudaGetErrorString(e));
        std::exit(1);
    }
}

// One tester: set up for (n, inverse, real), run once per call, tear down.
// Input and output are n complex values (real tests use the first n floats
// / n/2+1 bins, as the reference harness does).
struct Tester {
    virtual ~Tester() {}
    virtual const char* name() const = 0;
    virtual void init(const CkFftComplex* in, CkFftComplex* out, int n, bool inverse, bool real) = 0;
    virtual void run() = 0;
    virtual void shutdown() = 0;
    // transforms one run covers
    virtual int per_run() const { return 1; }
};

struct HostCkfft : Tester {
    CkFftContext* ctx = nullptr;
    const CkFftComplex* in = nullptr;
    CkFftComplex* out = nullptr;
    std::vector<CkFftComplex> tmp;
    int n = 0;
    bool inv = false, real = false;
    const char* name() const override { return "ckfft"; }
    void init(const CkFftComplex* i, CkFftComplex* o, int count, bool inverse, bool r) override
    {
        in = i, out = o, n = count, inv = inverse, real = r;
        ctx = CkFftInit(n, inv ? kCkFftDirection_Inverse : kCkFftDirection_Forward, nullptr, nullptr);
        if (!ctx) die("CkFftInit");
        tmp.resize(n / 2 + 1);
    }
    void run() override
    {
        if (real) {
            if (inv) check(CkFftRealInverse(ctx, n, in, (float*)out, tmp.data()), "CkFftRealInverse");
            else check(CkFftRealForward(ctx, n, (const float*)in, out), "CkFftRealForward");
        } else if (inv) {
            check(CkFftComplexInverse(ctx, n, in, out), "CkFftComplexInverse");
        } else {
            check(CkFftComplexForward(ctx, n, in, out), "CkFftComplexForward");
        }
    }
    void shutdown() override { CkFftShutdown(ctx); }
};

struct DeviceCkfft : Tester {
    CkFftContext* ctx = nullptr;
    CkFftComplex *din = nullptr, *dout = nullptr, *dtmp = nullptr;
    CkFftComplex* out = nullptr;
    int n = 0, batch = 1;
    bool inv = false, real = false;
    explicit DeviceCkfft(int b) : batch(b) {}
    const char* name() const override { return batch == 1 ? "ckfft_device" : "ckfft_batch"; }
    int per_run() const override { return batch; }
    void init(const CkFftComplex* i, CkFftComplex* o, int count, bool inverse, bool r) override
    {
        out = o, n = count, inv = inverse, real = r;
        ctx = CkFftInit(n, inv ? kCkFftDirection_Inverse : kCkFftDirection_Forward, nullptr, nullptr);
        if (!ctx) die("CkFftInit");
        // transforms back to back in the batch calls' layout: n complex,
        // n floats (real forward) or n/2+1 bins (real inverse) per input
        const size_t in_bytes = !real ? sizeof(CkFftComplex) * (size_t)n
                                      : (inv ? sizeof(CkFftComplex) * (size_t)(n / 2 + 1) : sizeof(float) * (size_t)n);
        const size_t slot = sizeof(CkFftComplex) * (size_t)(n + 2);
        cuda_check(cudaMalloc(&din, slot * batch), "cudaMalloc");
        cuda_check(cudaMalloc(&dout, slot * batch), "cudaMalloc");
        cuda_check(cudaMalloc(&dtmp, slot), "cudaMalloc");
        for (int b = 0; b < batch; ++b)
            cuda_check(cudaMemcpy((char*)din + in_bytes * b, i, in_bytes, cudaMemcpyHostToDevice), "cudaMemcpy");
    }
    void run() override
    {
        if (batch == 1) {
            if (real) {
                if (inv) check(CkFftRealInverse(ctx, n, din, (float*)dout, dtmp), "CkFftRealInverse");
                else check(CkFftRealForward(ctx, n, (const float*)din, dout), "CkFftRealForward");
            } else if (inv) {
                check(CkFftComplexInverse(ctx, n, din, dout), "CkFftComplexInverse");
            } else {
                check(CkFftComplexForward(ctx, n, din, dout), "CkFftComplexForward");
            }
            return;
        }
        if (real) {
            if (inv) check(CkFftCudaRealInverseBatch(ctx, n, batch, din, (float*)dout, nullptr), "RealInverseBatch");
            else check(CkFftCudaRealForwardBatch(ctx, n, batch, (const float*)din, dout, nullptr), "RealForwardBatch");
        } else if (inv) {
            check(CkFftCudaComplexInverseBatch(ctx, n, batch, din, dout, nullptr), "ComplexInverseBatch");
        } else {
            check(CkFftCudaComplexForwardBatch(ctx, n, batch, din, dout, nullptr), "ComplexForwardBatch");
        }
    }
    void shutdown() override
    {
        const size_t out_bytes = real && !inv ? sizeof(CkFftComplex) * (size_t)(n / 2 + 1)
                                              : (real ? sizeof(float) * (size_t)n : sizeof(CkFftComplex) * (size_t)n);
        cuda_check(cudaMemcpy(out, dout, out_bytes, cudaMemcpyDeviceToHost), "cudaMemcpy");
        cudaFree(din);
        cudaFree(dout);
        cudaFree(dtmp);
        CkFftShutdown(ctx);
    }
};

struct Kiss : Tester {
    kiss_fft_cfg cfg = nullptr;
    kiss_fftr_cfg rcfg = nullptr;
    std::vector<kiss_fft_cpx> kin, kout;
    CkFftComplex* out = nullptr;
    int n = 0;
    bool inv = false, real = false;
    const char* name() const override { return "ckfft_kiss_api"; }
    void init(const CkFftComplex* i, CkFftComplex* o, int count, bool inverse, bool r) override
    {
        out = o, n = count, inv = inverse, real = r;
        kin.resize(n);
        kout.resize(n);
        for (int k = 0; k < n; ++k) kin[k] = kiss_fft_cpx{i[k].real, i[k].imag};
        if (real) rcfg = kiss_fftr_alloc(n, inv, nullptr, nullptr);
        else cfg = kiss_fft_alloc(n, inv, nullptr, nullptr);
        if (!cfg && !rcfg) die("kiss alloc");
    }
    void run() override
    {
        if (real) {
            if (inv) kiss_fftri(rcfg, kin.data(), (float*)kout.data());
            else kiss_fftr(rcfg, (const float*)kin.data(), kout.data());
        } else {
            kiss_fft(cfg, kin.data(), kout.data());
        }
    }
    void shutdown() override
    {
        // kiss's real forward is half of ckfft's (src/test/test.cpp:368-372)
        const float scale = real && !inv ? 2.0f : 1.0f;
        for (int k = 0; k < n; ++k) out[k] = CkFftComplex{kout[k].r * scale, kout[k].i * scale};
        if (rcfg) kiss_fftr_free(rcfg);
        if (cfg) kiss_fft_free(cfg);
        rcfg = nullptr;
        cfg = nullptr;
    }
};

std::string results_name()
{
    struct utsname u;
    std::string m = uname(&u) == 0 ? u.machine : "unknown";
    std::replace(m.begin(), m.end(), ',', '_');
    return "results_linux_" + m + ".xml";
}

// previous times: test -> tester -> ms, from a results file of this layout
std::map<std::string, std::map<std::string, float>> read_prev(const std::string& path)
{
    std::map<std::string, std::map<std::string, float>> r;
    std::ifstream f(path);
    if (!f) return r;
    std::string line, test;
    while (std::getline(f, line)) {
        const size_t a = line.find('<');
        if (a == std::string::npos || line.compare(a, 2, "</") == 0) continue;
        const size_t b = line.find_first_of(" />", a + 1);
        const std::string tag = line.substr(a + 1, b - a - 1);
        const size_t t = line.find("time=\"");
        if (t == std::string::npos) {
            if (tag != "ckfft_test") test = tag;
            continue;
        }
        r[test][tag] = std::strtof(line.c_str() + t + 6, nullptr);
    }
    return r;
}

}  // namespace

int main(int argc, char** argv)
{
    std::string out_dir = ".", input_path, prev_path;
    int reps = 500;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "--out" && i + 1 < argc) out_dir = argv[++i];
        else if (a == "--input" && i + 1 < argc) input_path = argv[++i];
        else if (a == "--prev" && i + 1 < argc) prev_path = argv[++i];
        else if (a == "--reps" && i + 1 < argc) reps = std::atoi(argv[++i]);
        else {
            std::fprintf(stderr, "usage: %s [--out DIR] [--input FILE] [--prev FILE] [--reps N]\n", argv[0]);
            return 2;
        }
    }
    if (reps < 1) reps = 1;
    std::vector<CkFftComplex> input;
    if (!input_path.empty()) {
        std::ifstream f(input_path);
        CkFftComplex v;
        while (f >> v.real >> v.imag) input.push_back(v);
    } else {
        std::mt19937 g(20261204);
        std::uniform_real_distribution<float> u(-1.f, 1.f);
        for (int k = 0; k < 4096; ++k) input.push_back(CkFftComplex{u(g), u(g)});
    }
    int count = 1;
    while (count * 2 <= (int)input.size()) count *= 2;
    if (count < 256) {
        std::fprintf(stderr, "ckfft_timing: the input holds %zu values; the tests need at least 256\n", input.size());
        return 2;
    }
    input.resize(count);
    std::vector<CkFftComplex> output(count), inv_output(count);
    const auto prev = read_prev(prev_path);

    HostCkfft host;
    DeviceCkfft dev(1), batch(4096);
    Kiss kiss;
    std::vector<Tester*> testers = {&host, &dev, &kiss, &batch};

    std::string xml = "<ckfft_test>\n";
    std::printf("\n%d iterations\n", reps);
    auto timing_test = [&](const std::string& test, const std::vector<CkFftComplex>& in,
                           std::vector<CkFftComplex>& out, bool inverse, bool real) {
        std::printf("\n%s:\n", test.c_str());
        std::printf("        name    median       min       max      norm    change\n");
        std::printf("--------------------------------------------------------------------\n");
        xml += "    <" + test + ">\n";
        float base = 0.f;
        for (size_t k = 0; k < testers.size(); ++k) {
            Tester* t = testers[k];
            t->init(in.data(), out.data(), (int)in.size(), inverse, real);
            t->run();                                          // first call sets up lanes and caches
            cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
            Stats st;
            for (int r = 0; r < reps; ++r) {
                const auto t0 = std::chrono::steady_clock::now();
                t->run();
                if (t->per_run() > 1) cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
                const auto t1 = std::chrono::steady_clock::now();
                st.sample(std::chrono::duration<float, std::milli>(t1 - t0).count() / t->per_run());
            }
            t->shutdown();
            const float time = st.median();
            if (k == 0) base = time;
            float was = time;
            auto a = prev.find(test);
            if (a != prev.end()) {
                auto b = a->second.find(t->name());
                if (b != a->second.end()) was = b->second;
            }
            std::printf("%12s: %f  %f  %f  %f  %7.2f%%\n", t->name(), time, st.min(), st.max(), time / base,
                        100.0f * (time - was) / was);
            char line[160];
            std::snprintf(line, sizeof(line), "        <%s time=\"%g\" />\n", t->name(), time);
            xml += line;
        }
        xml += "    </" + test + ">\n";
    };
    std::vector<CkFftComplex> in = input;
    for (int n = count; n > 128; n /= 2) {
        in.resize(n);
        output.resize(n);
        inv_output.resize(n);
        timing_test("fft_" + std::to_string(n), in, output, false, false);
        timing_test("fft_inv_" + std::to_string(n), output, inv_output, true, false);
        timing_test("fft_real_" + std::to_string(n), in, output, false, true);
        timing_test("fft_inv_real_" + std::to_string(n), output, inv_output, true, true);
    }
    xml += "</ckfft_test>\n";
    const std::string path = out_dir + "/" + results_name();
    std::ofstream f(path);
    if (!f) {
        std::fprintf(stderr, "ckfft_timing: cannot write %s\n", path.c_str());
        return 1;
    }
    f << xml;
    std::printf("\nwrote results to %s\n", path.c_str());
    return 0;
}
