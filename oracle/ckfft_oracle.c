/*
 * ckfft_oracle.c -- CPU restatement of Cricket FFT's scalar path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle and the timed
 * CPU baseline.  It is never linked into, loaded by, or called from the product
 * library (ckfft_gb300/libckfft_cuda.so); only tests/, __graft_entry__.smoke()
 * and bench.py's CPU legs use it.
 *
 * It restates, operation for operation, the arithmetic of the reference's
 * portable path so that its output is bit-identical to the reference built with
 * the same compiler flags (checked by tests/test_oracle.py against oracle/_ref,
 * a build of the reference's own sources):
 *   - twiddle table          src/ckfft/context.cpp:111-126  (FP32 cosf/sinf)
 *   - argument validation    src/ckfft/ckfft.cpp:14-114
 *   - complex dispatch       src/ckfft/fft.cpp:13-46        (n=1 copy, n=2 add/sub)
 *   - radix-4 DIT recursion  src/ckfft/fft_default.cpp:12-266 (leaves n=4, n=8)
 *   - real dispatch          src/ckfft/fft_real.cpp:13-105  (n=1,2,4 closed forms)
 *   - real split / merge     src/ckfft/fft_real_default.cpp:13-114
 *   - complex arithmetic     src/ckfft/math_util.h:17-33    (4 mul + 2 add, no FMA)
 * Bit-identity needs the same operation order and no FMA contraction, so this
 * file is compiled with -ffp-contract=off for parity work.
 *
 * The traversal is written independently (one recursive node function with a
 * separate radix-4 combine), but the per-element arithmetic, the twiddle indices
 * and the leaf structure follow the reference because bit-identity requires it.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

typedef struct { float re, im; } ocx;

typedef struct {
    int nmax;
    ocx* fwd;   /* NULL when the context was made without the forward direction */
    ocx* inv;   /* NULL when the context was made without the inverse direction */
} ock_ctx;

enum { OCK_FWD = 1, OCK_INV = 2, OCK_BOTH = 3 };

static int is_pow2(unsigned int x) { return x != 0 && (x & (x - 1)) == 0; }

/* math_util.h:17-33: complex ops exactly as the reference writes them */
static inline ocx c_add(ocx a, ocx b) { ocx r; r.re = a.re + b.re; r.im = a.im + b.im; return r; }
static inline ocx c_sub(ocx a, ocx b) { ocx r; r.re = a.re - b.re; r.im = a.im - b.im; return r; }
static inline ocx c_mul(ocx a, ocx b)
{
    ocx r;
    r.re = a.re * b.re - a.im * b.im;
    r.im = a.im * b.re + a.re * b.im;
    return r;
}

/* ---------------------------------------------------------------- context */

/* context.cpp:111-126 -- theta evaluated in float: ((-2f * (float)pi) * i) / nmax */
static void fill_tables(int nmax, ocx* fwd, ocx* inv)
{
    for (int i = 0; i < nmax; ++i) {
        float theta = -2.0f * (float)M_PI * i / nmax;
        float c = cosf(theta);
        float s = sinf(theta);
        if (fwd) { fwd[i].re = c; fwd[i].im = s; }
        if (inv) { inv[i].re = c; inv[i].im = -s; }
    }
}

/* ckfft.cpp:14-34 validation, then an owned allocation (the oracle has no
   user-buffer mode; the product library's buf/bufSize handling is tested
   against the reference's rules directly). */
ock_ctx* ock_init(int nmax, int direction)
{
    if (nmax <= 0) return NULL;
    if (!is_pow2((unsigned)nmax)) return NULL;
    if (direction != OCK_FWD && direction != OCK_INV && direction != OCK_BOTH) return NULL;
    ock_ctx* c = (ock_ctx*)calloc(1, sizeof(ock_ctx));
    if (!c) return NULL;
    c->nmax = nmax;
    if (direction & OCK_FWD) c->fwd = (ocx*)malloc(sizeof(ocx) * (size_t)nmax);
    if (direction & OCK_INV) c->inv = (ocx*)malloc(sizeof(ocx) * (size_t)nmax);
    if (((direction & OCK_FWD) && !c->fwd) || ((direction & OCK_INV) && !c->inv)) {
        free(c->fwd); free(c->inv); free(c);
        return NULL;
    }
    fill_tables(nmax, c->fwd, c->inv);
    return c;
}

void ock_free(ock_ctx* c)
{
    if (!c) return;
    free(c->fwd);
    free(c->inv);
    free(c);
}

/* Copies the forward/inverse table out (for checking against the reference's). */
int ock_table(const ock_ctx* c, int inverse, ocx* dst)
{
    const ocx* t = inverse ? c->inv : c->fwd;
    if (!t) return 0;
    memcpy(dst, t, sizeof(ocx) * (size_t)c->nmax);
    return 1;
}

/* ------------------------------------------------------- radix-4 DIT core */

/* Radix-4 butterfly on already-twiddled inputs (fft_default.cpp:226-256).
   X0 = s02 + s13, X2 = s02 - s13, X1/X3 = d02 -/+ i*d13 (forward),
   with the sign of i flipped for the inverse. */
static inline void combine4(ocx f0, ocx f1w, ocx f2w2, ocx f3w3, int inverse,
                            ocx* x0, ocx* x1, ocx* x2, ocx* x3)
{
    ocx s02 = c_add(f0, f2w2), d02 = c_sub(f0, f2w2);
    ocx s13 = c_add(f1w, f3w3), d13 = c_sub(f1w, f3w3);
    *x0 = c_add(s02, s13);
    *x2 = c_sub(s02, s13);
    if (inverse) {
        x1->re = d02.re - d13.im; x1->im = d02.im + d13.re;
        x3->re = d02.re + d13.im; x3->im = d02.im - d13.re;
    } else {
        x1->re = d02.re + d13.im; x1->im = d02.im - d13.re;
        x3->re = d02.re - d13.im; x3->im = d02.im + d13.re;
    }
}

/* DFT of the n samples in[0], in[s], in[2s], ... into out[0..n) (natural order).
   tab/tstride: twiddle table and the step giving W_(n*s)... i.e. W_top^1 at
   tab[tstride]; at this node the combine twiddle for index i is tab[i*s*tstride].
   Mirrors fft_default.cpp:12-266. */
static void dit(const ocx* in, ocx* out, int n, int inverse, int s, const ocx* tab, int tstride)
{
    if (n == 4) {
        /* leaf n=4 (fft_default.cpp:22-67): gather, then an untwiddled combine */
        ocx a = in[0], b = in[s], c = in[2 * s], d = in[3 * s];
        out[0] = a; out[1] = b; out[2] = c; out[3] = d;
        combine4(out[0], out[1], out[2], out[3], inverse, &out[0], &out[1], &out[2], &out[3]);
        return;
    }
    if (n == 8) {
        /* leaf n=8 (fft_default.cpp:68-167): four radix-2 DFTs of (x_r, x_r+4),
           then the r=0 column untwiddled and the r=1 column twiddled */
        for (int r = 0; r < 4; ++r) {
            ocx p = in[r * s], q = in[(r + 4) * s];
            out[2 * r] = c_add(p, q);
            out[2 * r + 1] = c_sub(p, q);
        }
        combine4(out[0], out[2], out[4], out[6], inverse, &out[0], &out[2], &out[4], &out[6]);
        int step = s * tstride;
        ocx w1 = tab[step], w2 = tab[2 * step], w3 = tab[3 * step];
        ocx f1 = c_mul(out[3], w1), f2 = c_mul(out[5], w2), f3 = c_mul(out[7], w3);
        combine4(out[1], f1, f2, f3, inverse, &out[1], &out[3], &out[5], &out[7]);
        return;
    }
    /* general node (fft_default.cpp:168-266): 4 sub-DFTs on stride 4s, then combine */
    int q = n / 4;
    for (int r = 0; r < 4; ++r)
        dit(in + r * s, out + r * q, q, inverse, 4 * s, tab, tstride);
    int step = s * tstride;
    for (int i = 0; i < q; ++i) {
        ocx f1 = c_mul(out[q + i], tab[i * step]);
        ocx f2 = c_mul(out[2 * q + i], tab[2 * i * step]);
        ocx f3 = c_mul(out[3 * q + i], tab[3 * i * step]);
        combine4(out[i], f1, f2, f3, inverse, &out[i], &out[q + i], &out[2 * q + i], &out[3 * q + i]);
    }
}

/* fft.cpp:13-46 */
static void complex_dispatch(const ock_ctx* c, const ocx* in, ocx* out, int n, int inverse)
{
    if (n == 1) {
        out[0] = in[0];
    } else if (n == 2) {
        out[0] = c_add(in[0], in[1]);
        out[1] = c_sub(in[0], in[1]);
    } else {
        dit(in, out, n, inverse, 1, inverse ? c->inv : c->fwd, c->nmax / n);
    }
}

/* -------------------------------------------------------------- real FFT */

/* fft_real_default.cpp:13-63: pack as n/2 complex, half-size DFT, split.
   out[k] = S_k - (i W^k) D_k with S_k = (z_k + conj z_{m-k}), D_k = (z_k - conj z_{m-k})
   (in the reference's component form), output is 2 * DFT(x). */
static void real_forward_split(const ock_ctx* c, const float* input, ocx* out, int n)
{
    int m = n / 2;
    dit((const ocx*)input, out, m, 0, 1, c->fwd, c->nmax / m);
    out[m] = out[0];
    int ts = c->nmax / n;
    for (int i = 0; i < n / 4; ++i) {
        ocx z0 = out[i], z1 = out[m - i];
        ocx w0 = c->fwd[i * ts], w1 = c->fwd[(m - i) * ts];
        ocx sum, diff, f, t;
        sum.re = z0.re + z1.re;  sum.im = z0.im - z1.im;
        diff.re = z0.re - z1.re; diff.im = z0.im + z1.im;
        f.re = -w0.im; f.im = w0.re;
        t = c_mul(f, diff);
        out[i] = c_sub(sum, t);
        diff.re = -diff.re; sum.im = -sum.im;
        f.re = -w1.im; f.im = w1.re;
        t = c_mul(f, diff);
        out[m - i] = c_sub(sum, t);
    }
    out[n / 4].re = out[n / 4].re * 2.0f;
    out[n / 4].im = -out[n / 4].im * 2.0f;
}

/* fft_real_default.cpp:65-114: merge into tmp (S + i W~^k D), half-size inverse */
static void real_inverse_merge(const ock_ctx* c, const ocx* in, float* output, int n, ocx* tmp)
{
    int m = n / 2;
    int ts = c->nmax / n;
    for (int i = 0; i < n / 4; ++i) {
        ocx z0 = in[i], z1 = in[m - i];
        ocx w0 = c->inv[i * ts], w1 = c->inv[(m - i) * ts];
        ocx sum, diff, f, t;
        sum.re = z0.re + z1.re;  sum.im = z0.im - z1.im;
        diff.re = z0.re - z1.re; diff.im = z0.im + z1.im;
        f.re = -w0.im; f.im = w0.re;
        t = c_mul(f, diff);
        tmp[i] = c_add(sum, t);
        diff.re = -diff.re; sum.im = -sum.im;
        f.re = -w1.im; f.im = w1.re;
        t = c_mul(f, diff);
        tmp[m - i] = c_add(sum, t);
    }
    tmp[n / 4].re = in[n / 4].re * 2.0f;
    tmp[n / 4].im = -in[n / 4].im * 2.0f;
    dit(tmp, (ocx*)output, m, 1, 1, c->inv, c->nmax / m);
}

/* fft_real.cpp:13-60 (closed forms for n <= 4 are scaled by 2 like the split path) */
static void real_forward_dispatch(const ock_ctx* c, const float* in, ocx* out, int n)
{
    if (n == 1) {
        out[0].re = in[0] * 2.0f; out[0].im = 0.0f;
    } else if (n == 2) {
        out[0].re = (in[0] + in[1]) * 2.0f; out[0].im = 0.0f;
        out[1].re = (in[0] - in[1]) * 2.0f; out[1].im = 0.0f;
    } else if (n == 4) {
        float s02 = (in[0] + in[2]) * 2.0f, d02 = (in[0] - in[2]) * 2.0f;
        float s13 = (in[1] + in[3]) * 2.0f, d13 = (in[1] - in[3]) * 2.0f;
        out[0].re = s02 + s13; out[0].im = 0.0f;
        out[1].re = d02;       out[1].im = -d13;
        out[2].re = s02 - s13; out[2].im = 0.0f;
        /* The reference also stores bin 3 = conj(bin 1) here (fft_real.cpp:46-47),
           one element past the documented n/2+1 output; that write is left out. */
    } else {
        real_forward_split(c, in, out, n);
    }
}

/* fft_real.cpp:62-105 */
static void real_inverse_dispatch(const ock_ctx* c, const ocx* in, float* out, int n, ocx* tmp)
{
    if (n == 1) {
        out[0] = in[0].re;
    } else if (n == 2) {
        out[0] = in[0].re + in[1].re;
        out[1] = in[0].re - in[1].re;
    } else if (n == 4) {
        float s02 = in[0].re + in[2].re;
        float s13 = 2.0f * in[1].re;
        ocx d02 = c_sub(in[0], in[2]);
        float d13i = 2.0f * in[1].im;
        out[0] = s02 + s13;
        out[1] = d02.re - d13i;
        out[2] = s02 - s13;
        out[3] = d02.re + d13i;
    } else {
        real_inverse_merge(c, in, out, n, tmp);
    }
}

/* ------------------------------------------------- public entry points
   Return codes and check order follow ckfft.cpp:36-114. */

static int check_n(const ock_ctx* c, int n)
{
    return is_pow2((unsigned)n) && n <= c->nmax;
}

int ock_complex(const ock_ctx* c, int n, const ocx* in, ocx* out, int inverse)
{
    if (!c || !(inverse ? c->inv : c->fwd)) return 0;
    if (!check_n(c, n)) return 0;
    if (!in || !out || in == out) return 0;
    complex_dispatch(c, in, out, n, inverse);
    return 1;
}

int ock_real_forward(const ock_ctx* c, int n, const float* in, ocx* out)
{
    if (!c || !c->fwd) return 0;
    if (!check_n(c, n)) return 0;
    if (!in || !out || (const void*)in == (const void*)out) return 0;
    real_forward_dispatch(c, in, out, n);
    return 1;
}

int ock_real_inverse(const ock_ctx* c, int n, const ocx* in, float* out, ocx* tmp)
{
    if (!tmp) return 0;
    if (!c || !c->inv) return 0;
    if (!check_n(c, n)) return 0;
    if (!in || !out || (const void*)in == (const void*)out) return 0;
    real_inverse_dispatch(c, in, out, n, tmp);
    return 1;
}

/* ------------------------------------------------------ batch runner
   Runs `count` independent transforms of one kind over contiguous frames,
   split across `threads` POSIX threads that share one context (contexts are
   read-only after init, as the reference's header allows).  Used for the
   multi-core CPU baseline and to produce oracle outputs for large batches.
   kind: 0 = complex forward, 1 = complex inverse, 2 = real forward, 3 = real inverse.
   Frame sizes: complex n -> n complex; real forward n floats -> n/2+1 complex;
   real inverse n/2+1 complex -> n floats. */

typedef struct {
    const ock_ctx* c;
    int kind, n;
    long long first, last;
    const char* in;
    char* out;
    size_t in_bytes, out_bytes;
    int ok;
} batch_job;

static void* batch_worker(void* arg)
{
    batch_job* j = (batch_job*)arg;
    ocx* tmp = NULL;
    if (j->kind == 3) {
        tmp = (ocx*)malloc(sizeof(ocx) * (size_t)(j->n / 2 + 1));
        if (!tmp) { j->ok = 0; return NULL; }
    }
    j->ok = 1;
    for (long long f = j->first; f < j->last; ++f) {
        const char* src = j->in + (size_t)f * j->in_bytes;
        char* dst = j->out + (size_t)f * j->out_bytes;
        int r = 0;
        switch (j->kind) {
        case 0: r = ock_complex(j->c, j->n, (const ocx*)src, (ocx*)dst, 0); break;
        case 1: r = ock_complex(j->c, j->n, (const ocx*)src, (ocx*)dst, 1); break;
        case 2: r = ock_real_forward(j->c, j->n, (const float*)src, (ocx*)dst); break;
        case 3: r = ock_real_inverse(j->c, j->n, (const ocx*)src, (float*)dst, tmp); break;
        }
        if (!r) { j->ok = 0; break; }
    }
    free(tmp);
    return NULL;
}

int ock_batch(const ock_ctx* c, int kind, int n, long long count, const void* in, void* out, int threads)
{
    if (!c || count < 0 || threads < 1 || kind < 0 || kind > 3) return 0;
    size_t ib, ob;
    if (kind <= 1) { ib = ob = sizeof(ocx) * (size_t)n; }
    else if (kind == 2) { ib = sizeof(float) * (size_t)n; ob = sizeof(ocx) * (size_t)(n / 2 + 1); }
    else { ib = sizeof(ocx) * (size_t)(n / 2 + 1); ob = sizeof(float) * (size_t)n; }
    if (threads > count) threads = count > 0 ? (int)count : 1;
    batch_job* jobs = (batch_job*)calloc((size_t)threads, sizeof(batch_job));
    pthread_t* tid = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    if (!jobs || !tid) { free(jobs); free(tid); return 0; }
    for (int t = 0; t < threads; ++t) {
        jobs[t].c = c; jobs[t].kind = kind; jobs[t].n = n;
        jobs[t].first = count * t / threads;
        jobs[t].last = count * (t + 1) / threads;
        jobs[t].in = (const char*)in; jobs[t].out = (char*)out;
        jobs[t].in_bytes = ib; jobs[t].out_bytes = ob;
    }
    int started = 0;
    for (int t = 1; t < threads; ++t) {
        if (pthread_create(&tid[t], NULL, batch_worker, &jobs[t]) != 0) break;
        started = t;
    }
    batch_worker(&jobs[0]);
    int ok = jobs[0].ok;
    for (int t = 1; t <= started; ++t) {
        pthread_join(tid[t], NULL);
        ok &= jobs[t].ok;
    }
    if (started != threads - 1) ok = 0;
    free(jobs);
    free(tid);
    return ok;
}
