// twiddle.cpp -- device twiddle table generation (host side).
//
// Replaces the reference's FP32 table (src/ckfft/context.cpp:111-126, which
// evaluates cosf/sinf of a float angle) with values computed in FP64 and
// rounded once to FP32.  The angle is reduced exactly in integer arithmetic
// to a quadrant and a remainder in [0, pi/4] before any trigonometry, so the
// table is exactly symmetric: W^{N/4} = -i, W^{N/2} = -1, W^{N/8} has equal
// components, and W^{N/4 - m} mirrors W^m bit for bit.
//
// Layout (all levels in one allocation of 2*N entries): W_{2^q}^m at index
// 2^q + m for 0 <= q <= log2 N and 0 <= m < 2^q; index 0 is unused.  Lower
// levels are exact subsamples of the top level.
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>
#include <vector>

namespace ckg {

// exp(-2 pi i m / n) for a power-of-two n, m in [0, n).
static void w_exact(uint64_t m, uint64_t n, double& c, double& s)
{
    if (n < 4) {                        // n = 1: m = 0; n = 2: m in {0, 1}
        c = (m == 0) ? 1.0 : -1.0;
        s = 0.0;
        return;
    }
    const uint64_t q4 = n / 4;
    const uint64_t quad = m / q4;       // quadrant 0..3 of the angle 2 pi m / n
    const uint64_t r = m % q4;          // remainder, angle 2 pi r / n in [0, pi/2)
    double cr, sr;                      // cos, sin of the remainder angle
    const double two_pi = 6.283185307179586476925286766559;
    if (2 * r <= q4) {
        const double a = two_pi * (double)r / (double)n;
        cr = std::cos(a);
        sr = std::sin(a);
    } else {                            // use the complement pi/2 - a for accuracy and symmetry
        const double a = two_pi * (double)(q4 - r) / (double)n;
        cr = std::sin(a);
        sr = std::cos(a);
    }
    double cc, ss;                      // cos, sin of the full angle
    switch (quad) {
    case 0: cc = cr; ss = sr; break;
    case 1: cc = 0.0 - sr; ss = cr; break;
    case 2: cc = 0.0 - cr; ss = 0.0 - sr; break;
    default: cc = sr; ss = 0.0 - cr; break;
    }
    c = cc;
    s = 0.0 - ss;                       // forward twiddle: exp(-i angle)
}

void build_twiddles(int log2n, std::vector<float2>& tab)
{
    const uint64_t n = 1ull << log2n;
    tab.assign(2 * n, make_float2(1.0f, 0.0f));
    float2* top = tab.data() + n;
    for (uint64_t m = 0; m < n; ++m) {
        double c, s;
        w_exact(m, n, c, s);
        top[m] = make_float2((float)c, (float)s);
    }
    for (int q = log2n - 1; q >= 0; --q) {
        const uint64_t len = 1ull << q;
        float2* lvl = tab.data() + len;
        const uint64_t step = n >> q;
        for (uint64_t m = 0; m < len; ++m) lvl[m] = top[m * step];
    }
}

}  // namespace ckg
