/* kiss_fft_cuda.h -- kiss_fft's C interface on the CUDA transforms of
 * libckfft_cuda (power-of-two sizes).
 *
 * Replaces ext/kiss_fft130/kiss_fft.h:51-118 and tools/kiss_fftr.h:18-41 of
 * the reference tree (kiss_fft 1.3.0, the comparison library of the
 * reference's test harness, src/test/test.cpp:315-395): same type names,
 * function names, arguments, scaling (unscaled forward and inverse; the real
 * forward is half of CkFftRealForward, the real inverse equals
 * CkFftRealInverse) and the same mem / lenmem protocol of the alloc calls.
 * A program switches by including this header instead of kiss_fft.h /
 * kiss_fftr.h and linking libckfft_cuda instead of kiss_fft.c / kiss_fftr.c.
 *
 * Differences:
 *   - nfft must be a power of two (real: at least 2); other sizes make the
 *     alloc calls return NULL (kiss_fft also factors 3, 5 and others);
 *   - kiss_fft_free / kiss_fftr_free are functions, not `free`: a cfg holds
 *     GPU resources, so release it with them (they free the cfg memory only
 *     when the alloc call allocated it);
 *   - buffers may be host (pageable or page-locked) or device memory of the
 *     cfg's GPU; fin == fout is allowed, as in kiss_fft;
 *   - failures (a NULL or wrong cfg, a CUDA error) leave the output
 *     untouched and set CkFftCudaGetLastError() (kiss_fft has no error path);
 *   - kiss_fft_next_fast_size(n) is the smallest power of two >= n.
 * Needs C99 or later (the same as ckfft_cuda.h). */
#ifndef KISS_FFT_CUDA_H
#define KISS_FFT_CUDA_H

/* The original headers' guards: a later #include of kiss_fft.h or
 * kiss_fftr.h becomes a no-op instead of a second set of definitions. */
#define KISS_FFT_H
#define KISS_FTR_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define kiss_fft_scalar float

typedef struct {
    kiss_fft_scalar r;
    kiss_fft_scalar i;
} kiss_fft_cpx;

typedef struct kiss_fft_state* kiss_fft_cfg;
typedef struct kiss_fftr_state* kiss_fftr_cfg;

/* Complex transform of nfft points, forward or (inverse_fft != 0) inverse.
 * lenmem == NULL: the cfg is allocated; mem != NULL and *lenmem large
 * enough: the cfg is placed in mem and *lenmem set to the size used;
 * otherwise NULL is returned and *lenmem set to the size needed. */
kiss_fft_cfg kiss_fft_alloc(int nfft, int inverse_fft, void* mem, size_t* lenmem);
void kiss_fft(kiss_fft_cfg cfg, const kiss_fft_cpx* fin, kiss_fft_cpx* fout);
/* Input read from every fin_stride-th element (fin_stride >= 1). */
void kiss_fft_stride(kiss_fft_cfg cfg, const kiss_fft_cpx* fin, kiss_fft_cpx* fout, int fin_stride);
void kiss_fft_free(kiss_fft_cfg cfg);
void kiss_fft_cleanup(void);
int kiss_fft_next_fast_size(int n);

#define kiss_fftr_next_fast_size_real(n) (kiss_fft_next_fast_size(((n) + 1) >> 1) << 1)

/* Real transforms: kiss_fftr maps nfft reals to nfft/2+1 bins, kiss_fftri
 * nfft/2+1 bins to nfft reals (unscaled). */
kiss_fftr_cfg kiss_fftr_alloc(int nfft, int inverse_fft, void* mem, size_t* lenmem);
void kiss_fftr(kiss_fftr_cfg cfg, const kiss_fft_scalar* timedata, kiss_fft_cpx* freqdata);
void kiss_fftri(kiss_fftr_cfg cfg, const kiss_fft_cpx* freqdata, kiss_fft_scalar* timedata);
void kiss_fftr_free(kiss_fftr_cfg cfg);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* KISS_FFT_CUDA_H */
