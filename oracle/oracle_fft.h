/*
 * oracle_fft.h -- TEST INFRASTRUCTURE ONLY.  FP64 complex helpers and the
 * iterative radix-2 FFT shared by the CPU oracles (oracle.c: the chi(2) crystal
 * pass; gnlse_oracle.c: the chi(3) fibre).  Unnormalised, sign -1 forward, +1
 * inverse.  Every definition is static, so each oracle file has its own copy.
 */
#ifndef OFX_ORACLE_FFT_H
#define OFX_ORACLE_FFT_H

#include <math.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double re, im; } cplx;

/* point loops of one schedule go parallel from this many points, when the
 * calling thread runs a lone schedule with an explicit thread count (t_inner)
 * and no outer (per-schedule) parallel region is active */
#define OFX_PAR_MIN 4096
#ifdef _OPENMP
static _Thread_local int t_inner = 0;
static inline int par_ok(size_t count) { return t_inner && count >= OFX_PAR_MIN && !omp_in_parallel(); }
#else
static inline int par_ok(size_t count) { (void)count; return 0; }
#endif

static inline cplx cmk(double r, double i) { cplx z = {r, i}; return z; }
static inline cplx cadd(cplx a, cplx b) { return cmk(a.re + b.re, a.im + b.im); }
static inline cplx csub(cplx a, cplx b) { return cmk(a.re - b.re, a.im - b.im); }
static inline cplx cmul(cplx a, cplx b) {
    return cmk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
static inline cplx cscale(cplx a, double s) { return cmk(a.re * s, a.im * s); }
static inline cplx cconj(cplx a) { return cmk(a.re, -a.im); }
static inline double cabs2(cplx a) { return hypot(a.re, a.im); }
static inline cplx cexpi(double phi) { return cmk(cos(phi), sin(phi)); }

/* ------------------------------------------------------------------------ */
/* FFT: iterative radix-2, in place, unnormalised, sign -1 forward.          */
/* ------------------------------------------------------------------------ */
typedef struct {
    int n, log2n;
    cplx* tw;       /* exp(-2 pi i e / n), e in [0, n/2) */
    cplx* tws;      /* the same values per stage, contiguous: stage len holds tw[j n / len], j < len / 2 */
    int* rev;       /* bit reversal permutation */
} fft_plan;

static int ilog2(int n) { int l = 0; while ((1 << l) < n) ++l; return l; }

static int fft_plan_init(fft_plan* p, int n) {
    p->tw = p->tws = NULL;
    p->rev = NULL;                      /* a failed init leaves nothing to free */
    p->n = n; p->log2n = ilog2(n);
    if ((1 << p->log2n) != n) return -1;
    p->tw = (cplx*)malloc(sizeof(cplx) * (size_t)(n / 2 + 1));
    p->tws = (cplx*)malloc(sizeof(cplx) * (size_t)n);
    p->rev = (int*)malloc(sizeof(int) * (size_t)n);
    if (!p->tw || !p->tws || !p->rev) return -2;
    for (int e = 0; e < n / 2; ++e) {
        /* angle in turns computed exactly, then to radians */
        double a = -2.0 * M_PI * (double)e / (double)n;
        p->tw[e] = cmk(cos(a), sin(a));
    }
    size_t off = 0;
    for (int len = 2; len <= n; len <<= 1) {
        for (int j = 0; j < len / 2; ++j) p->tws[off + j] = p->tw[j * (n / len)];
        off += (size_t)(len / 2);
    }
    for (int i = 0; i < n; ++i) {
        int r = 0;
        for (int b = 0; b < p->log2n; ++b) if (i & (1 << b)) r |= 1 << (p->log2n - 1 - b);
        p->rev[i] = r;
    }
    return 0;
}

static void fft_plan_free(fft_plan* p) { free(p->tw); free(p->tws); free(p->rev); }

static void fft_exec(const fft_plan* p, cplx* x, int inverse) {
    const int n = p->n;
    if (!par_ok((size_t)n)) {
        /* one thread: the same butterflies in the same order, block by block */
        for (int i = 0; i < n; ++i) {
            int r = p->rev[i];
            if (r > i) { cplx t = x[i]; x[i] = x[r]; x[r] = t; }
        }
        const cplx* tw = p->tws;
        for (int len = 2; len <= n; len <<= 1) {
            const int half = len >> 1;
            for (int b = 0; b < n; b += len) {
                cplx* xa = x + b;
                cplx* xb = x + b + half;
                for (int j = 0; j < half; ++j) {
                    cplx w = tw[j];
                    if (inverse) w = cconj(w);
                    cplx u = xa[j], v = cmul(xb[j], w);
                    xa[j] = cadd(u, v);
                    xb[j] = csub(u, v);
                }
            }
            tw += half;
        }
        return;
    }
#pragma omp parallel
    {
#pragma omp for schedule(static)
        for (int i = 0; i < n; ++i) {
            int r = p->rev[i];
            if (r > i) { cplx t = x[i]; x[i] = x[r]; x[r] = t; }
        }
        /* stage by stage (the implicit barrier of each loop), butterfly q of n/2:
         * block (q / half) of length len, offset j = q mod half */
        for (int len = 2; len <= n; len <<= 1) {
            const int half = len >> 1, step = n / len;
#pragma omp for schedule(static)
            for (int q = 0; q < n / 2; ++q) {
                const int j = q & (half - 1);
                const int b = (q - j) << 1;
                cplx w = p->tw[j * step];
                if (inverse) w = cconj(w);
                cplx u = x[b + j], v = cmul(x[b + j + half], w);
                x[b + j] = cadd(u, v);
                x[b + j + half] = csub(u, v);
            }
        }
    }
}

#ifdef _OPENMP
/* The butterfly stages of fft_exec spread over a team of T threads (T a power of
 * two, n / T at least 2), called by every thread of an enclosing parallel region
 * with its own tid.  Thread tid owns points [tid n/T, (tid+1) n/T) and must itself
 * have written its own points of x in bit-reversed order (a gather
 * x[i] = src[rev[i]], which reads only and keeps each thread's writes in its own
 * cache lines).  Stages whose blocks fit in one thread's span run without
 * synchronisation; a barrier, then the last log2 T stages split their butterflies
 * evenly, each followed by a barrier.  Each element sees the same butterflies,
 * with the same twiddles, as in fft_exec, so the result is bit-identical.  On
 * return x is complete. */
static void fft_team_stages(const fft_plan* p, cplx* x, int inverse, int tid, int T) {
    const int n = p->n, span = n / T, lo = tid * span, hi = lo + span;
    const cplx* tw = p->tws;
    int len = 2;
    for (; len <= span; len <<= 1) {
        const int half = len >> 1;
        for (int b = lo; b < hi; b += len) {
            cplx* xa = x + b;
            cplx* xb = x + b + half;
            for (int j = 0; j < half; ++j) {
                cplx w = tw[j];
                if (inverse) w = cconj(w);
                cplx u = xa[j], v = cmul(xb[j], w);
                xa[j] = cadd(u, v);
                xb[j] = csub(u, v);
            }
        }
        tw += half;
    }
#pragma omp barrier
    const int q0 = tid * (n / 2 / T), q1 = q0 + n / 2 / T;
    for (; len <= n; len <<= 1) {
        const int half = len >> 1;
        for (int q = q0; q < q1; ++q) {
            const int j = q & (half - 1);
            const int b = (q - j) << 1;
            cplx w = tw[j];
            if (inverse) w = cconj(w);
            cplx u = x[b + j], v = cmul(x[b + j + half], w);
            x[b + j] = cadd(u, v);
            x[b + j + half] = csub(u, v);
        }
        tw += half;
#pragma omp barrier
    }
}
#endif

#endif
