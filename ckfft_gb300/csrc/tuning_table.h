// tuning_table.h -- generated by ckfft_gb300/autotune.py; do not edit by hand.
// Measured on NVIDIA GB300, 2026-12-04.
// kTunedLog2R[L]: values per thread (log2) of every single-CTA kernel family
// (batched, pipelined, strided, fused, grouped, job kernel) for complex
// (half-)length 2^L, so that all of them compute a size with the same radices.
// kTunedVariant[kind][L]: batched kernel variant for kind (0 complex forward,
// 1 complex inverse, 2 real forward, 3 real inverse): 0 plain, 2 / 3 pipelined
// with 2 / 3 bulk-copy buffers, 6 / 7 CTAs of about 512 / 128 threads, 8
// pipelined with one buffer and a split exchange area (the same arithmetic
// as plain).
#pragma once
namespace ckg {
constexpr signed char kTunedLog2R[15] = {0, 1, 2, 3, 4, 4, 3, 3, 4, 4, 4, 4, 4, 5, 5};
constexpr signed char kTunedVariant[4][15] = {
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 7, 7, 0, 8, 8},   // cfwd
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 7, 7, 0, 0, 8},   // cinv
    {0, 0, 0, 0, 0, 0, 0, 7, 0, 7, 7, 7, 0, 0, 8},   // rfwd
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 2, 2, 2, 0, 8, 8},   // rinv
};
}  // namespace ckg
