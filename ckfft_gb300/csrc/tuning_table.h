// tuning_table.h -- generated by ckfft_gb300/autotune.py; do not edit by hand.
// Measured on NVIDIA GB300, 2026-12-03.  kTunedVariant[kind][L]: kernel variant for
// kind (0 complex forward, 1 complex inverse, 2 real forward, 3 real inverse)
// and complex (half-)length 2^L: 0 plain, 2 / 3 pipelined with 2 / 3 buffers.
#pragma once
namespace ckg {
constexpr signed char kTunedVariant[4][15] = {
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},   // cfwd
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},   // cinv
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},   // rfwd
    {0, 0, 2, 0, 0, 0, 2, 0, 0, 2, 2, 2, 0, 0, 0},   // rinv
};
}  // namespace ckg
