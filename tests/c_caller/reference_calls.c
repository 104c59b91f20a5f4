/* reference_calls.c -- a plain C99 caller of the six reference-named calls.
 *
 * Uses nothing but CkFftInit / CkFftShutdown / CkFftRealForward /
 * CkFftRealInverse / CkFftComplexForward / CkFftComplexInverse from
 * include/ckfft_cuda.h, on ordinary malloc'd host buffers, the way a program
 * written against the reference's inc/ckfft/ckfft.h calls them (the
 * reference's example program, src/example/main.cpp:44-85, runs a real
 * forward then inverse of 1024 values and expects the input back scaled by
 * 2 * 1024).  Built by the tests with gcc -std=c99 against the header and
 * linked to libckfft_cuda.so, with no other change.
 *
 *   reference_calls IN.f32 OUT.bin
 *
 * IN.f32: n float32 values (n a power of two).  OUT.bin receives, in order,
 * the real forward spectrum (n/2+1 complex), the real round trip (n floats,
 * unscaled), the complex forward of the values read as n/2 complex pairs
 * and that spectrum's complex inverse (n/2 complex each).  Prints the
 * squared error of both round trips after removing their gains.
 */
#include <stdio.h>
#include <stdlib.h>

#include "ckfft_cuda.h"

static long file_floats(FILE* f)
{
    long bytes;
    if (fseek(f, 0, SEEK_END) != 0) return -1;
    bytes = ftell(f);
    if (fseek(f, 0, SEEK_SET) != 0) return -1;
    return bytes < 0 ? -1 : bytes / (long)sizeof(float);
}

int main(int argc, char** argv)
{
    FILE* fin;
    FILE* fout;
    long n;
    int i, m, ok;
    float* input;
    float* back;
    float err_real = 0.0f, err_complex = 0.0f;
    CkFftComplex* spectrum;
    CkFftComplex* tmp;
    CkFftComplex* cspec;
    CkFftComplex* cback;
    CkFftContext* context;

    if (argc != 3) {
        fprintf(stderr, "usage: %s IN.f32 OUT.bin\n", argv[0]);
        return 2;
    }
    fin = fopen(argv[1], "rb");
    if (!fin) { perror(argv[1]); return 2; }
    n = file_floats(fin);
    if (n < 8 || (n & (n - 1)) != 0) { fprintf(stderr, "need a power-of-two count >= 8 of floats\n"); return 2; }
    m = (int)n / 2;
    input = (float*)malloc(sizeof(float) * (size_t)n);
    back = (float*)malloc(sizeof(float) * (size_t)n);
    spectrum = (CkFftComplex*)malloc(sizeof(CkFftComplex) * (size_t)(m + 1));
    tmp = (CkFftComplex*)malloc(sizeof(CkFftComplex) * (size_t)(m + 1));
    cspec = (CkFftComplex*)malloc(sizeof(CkFftComplex) * (size_t)m);
    cback = (CkFftComplex*)malloc(sizeof(CkFftComplex) * (size_t)m);
    if (!input || !back || !spectrum || !tmp || !cspec || !cback) { fprintf(stderr, "out of memory\n"); return 2; }
    if (fread(input, sizeof(float), (size_t)n, fin) != (size_t)n) { fprintf(stderr, "short read\n"); return 2; }
    fclose(fin);

    /* the context: nMax = n, both directions, memory allocated by the library */
    context = CkFftInit((int)n, kCkFftDirection_Both, NULL, NULL);
    if (!context) { fprintf(stderr, "CkFftInit failed\n"); return 1; }

    ok = CkFftRealForward(context, (int)n, input, spectrum);
    ok = ok && CkFftRealInverse(context, (int)n, spectrum, back, tmp);
    /* the same values as n/2 complex numbers, forward then inverse */
    ok = ok && CkFftComplexForward(context, m, (const CkFftComplex*)input, cspec);
    ok = ok && CkFftComplexInverse(context, m, cspec, cback);
    if (!ok) { fprintf(stderr, "a transform returned 0\n"); CkFftShutdown(context); return 1; }

    for (i = 0; i < (int)n; ++i) {
        const float d = back[i] / (2.0f * (float)n) - input[i];
        err_real += d * d;
    }
    for (i = 0; i < m; ++i) {
        const float dr = cback[i].real / (float)m - input[2 * i];
        const float di = cback[i].imag / (float)m - input[2 * i + 1];
        err_complex += dr * dr + di * di;
    }
    printf("real round trip error: %g\ncomplex round trip error: %g\n", err_real, err_complex);

    fout = fopen(argv[2], "wb");
    if (!fout) { perror(argv[2]); CkFftShutdown(context); return 2; }
    fwrite(spectrum, sizeof(CkFftComplex), (size_t)(m + 1), fout);
    fwrite(back, sizeof(float), (size_t)n, fout);
    fwrite(cspec, sizeof(CkFftComplex), (size_t)m, fout);
    fwrite(cback, sizeof(CkFftComplex), (size_t)m, fout);
    fclose(fout);

    CkFftShutdown(context);
    free(input); free(back); free(spectrum); free(tmp); free(cspec); free(cback);
    return 0;
}
