/*
 * gnlse_oracle.c -- FP64 C restatement of the chi(3) fibre GNLSE solver.
 *
 * TEST INFRASTRUCTURE ONLY: a second oracle for optifax_gb300's gnlse_kernel
 * (csrc/ofx_gnlse.cu), beside oracle/gnlse_oracle.py, and the timed CPU baseline
 * of the fibre workload.  Only tests/ and bench.py's cpu_baseline leg load it.
 *
 * The equation, grids and operators are gnlsefib.m:22-66
 * (toolbox/lib/internal/main/gnlsefib.m): the interaction-picture spectral field
 * AW obeys dAW/dz = i gamma W ifft(AT ((1 - fR)|AT|^2 + RS)) e^{-Lz} with
 * AT = fft(AW e^{Lz}), RS = dT fR fft(ifft(|AT|^2) RW) and L = i B - alpha/2, in
 * MATLAB's (and NumPy's) fft/ifft conventions, from AW(0) = ifft(A).
 * gnlsefib.m:70-80 integrates it with MATLAB's ode45 (a closed binary) and outputs at
 * linspace(0, length, n_saves).  This file follows the step control that
 * oracle/gnlse_oracle.py and the GPU kernel share, restated from ode45's published
 * algorithm (Shampine & Reichelt, "The MATLAB ODE Suite", 1997): the Dormand-Prince
 * 5(4) pair (FSAL), NormControl error norm err = ||h sum_i e_i k_i|| /
 * max(||y||, ||y_new||, AbsTol/RelTol), accepted when err <= RelTol; initial step
 * min(hmax, 0.8 RelTol^(1/5) max(||y0||, threshold) / ||f0||); hmax = length / 10;
 * a step stretched to the end when 1.1 h reaches it; after a failure h scales by
 * max(0.1, 0.8 (RelTol/err)^(1/5)) the first time and halves after that; after an
 * accepted step with no failure h /= 1.25 (err/RelTol)^(1/5) (h *= 5 when that
 * divisor is <= 0.2), after one that failed first h is kept.  Steps do not stop at
 * the save points: a save point inside an accepted step is output from a separate
 * Dormand-Prince step of exactly that length from the step's start.  Positions are
 * integers in units of length / 2^40.  Outputs as gnlsefib.m:82-89.  Independent
 * pulses run in parallel (OpenMP).
 *
 * Parity with MATLAB's own ode45 output is unpinned; this restatement is checked
 * against the NumPy one (tests/test_gnlse_oracle.py) and the known answers there.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "gnlse_oracle.h"
#include "oracle_fft.h"

#define Z_BITS 40
#define MAX_ATTEMPTS 10000000

/* Dormand-Prince 5(4) tableau (Dormand & Prince 1980); row 6 = the 5th-order
 * weights (FSAL), DP_E = b - b_hat */
static const double DP_C[7] = {0.0, 1.0 / 5, 3.0 / 10, 4.0 / 5, 8.0 / 9, 1.0, 1.0};
static const double DP_A[7][6] = {
    {0.0},
    {1.0 / 5},
    {3.0 / 40, 9.0 / 40},
    {44.0 / 45, -56.0 / 15, 32.0 / 9},
    {19372.0 / 6561, -25360.0 / 2187, 64448.0 / 6561, -212.0 / 729},
    {9017.0 / 3168, -355.0 / 33, 46732.0 / 5247, 49.0 / 176, -5103.0 / 18656},
    {35.0 / 384, 0.0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84}};
static const double DP_E[7] = {71.0 / 57600, 0.0, -71.0 / 16695, 71.0 / 1920, -17253.0 / 339200, 22.0 / 525,
                               -1.0 / 40};

typedef struct {
    int n;
    fft_plan plan;
    cplx* buf[7];               /* stage derivatives; buf[f] is the FSAL k_1 */
    cplx *y, *ys, *ynew, *acc, *e, *at, *t;
    double* it;
} gwork;

static void gwork_free(gwork* w) {
    fft_plan_free(&w->plan);
    for (int i = 0; i < 7; ++i) free(w->buf[i]);
    free(w->y); free(w->ys); free(w->ynew); free(w->acc); free(w->e); free(w->at); free(w->t); free(w->it);
}

static int gwork_init(gwork* w, int n) {
    memset(w, 0, sizeof(*w));
    w->n = n;
    if (fft_plan_init(&w->plan, n)) return -1;
    const size_t cb = sizeof(cplx) * (size_t)n;
    for (int i = 0; i < 7; ++i) if (!(w->buf[i] = (cplx*)malloc(cb))) return -2;
    w->y = (cplx*)malloc(cb); w->ys = (cplx*)malloc(cb); w->ynew = (cplx*)malloc(cb);
    w->acc = (cplx*)malloc(cb); w->e = (cplx*)malloc(cb); w->at = (cplx*)malloc(cb); w->t = (cplx*)malloc(cb);
    w->it = (double*)malloc(sizeof(double) * (size_t)n);
    if (!w->y || !w->ys || !w->ynew || !w->acc || !w->e || !w->at || !w->t || !w->it) return -2;
    return 0;
}

/* a / b by Smith's method */
static inline cplx cdiv(cplx a, cplx b) {
    if (fabs(b.re) >= fabs(b.im)) {
        double r = b.im / b.re, s = 1.0 / (b.re + b.im * r);
        return cmk((a.re + a.im * r) * s, (a.im - a.re * r) * s);
    }
    double r = b.re / b.im, s = 1.0 / (b.im + b.re * r);
    return cmk((a.re * r + a.im) * s, (a.im * r - a.re) * s);
}

/* e = e^{Lz} = e^{-alpha z / 2} e^{i B z} */
static void lz(const ofx_gnlse_params* p, const double* B, double z, cplx* e) {
    const double att = exp(-0.5 * p->alpha * z);
    for (int i = 0; i < p->n; ++i) e[i] = cscale(cexpi(B[i] * z), att);
}

static double norm(const cplx* x, int n) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += x[i].re * x[i].re + x[i].im * x[i].im;
    return sqrt(s);
}

/* out = dAW/dz at (z, AW) (gnlsefib.m:54-66) */
static void rhs(const ofx_gnlse_params* p, const double* B, const double* W, const cplx* RW, gwork* w,
                double z, const cplx* AW, cplx* out) {
    const int n = p->n;
    const double inv_n = 1.0 / (double)n;
    lz(p, B, z, w->e);
    for (int i = 0; i < n; ++i) w->at[i] = cmul(AW[i], w->e[i]);
    fft_exec(&w->plan, w->at, 0);                                     /* AT = fft(AW e^{Lz}) */
    for (int i = 0; i < n; ++i) {
        const double m = hypot(w->at[i].re, w->at[i].im);
        w->it[i] = m * m;                                             /* |AT|^2 */
    }
    if (!RW) {
        for (int i = 0; i < n; ++i) w->t[i] = cscale(w->at[i], w->it[i]);
    } else {
        for (int i = 0; i < n; ++i) w->t[i] = cmk(w->it[i], 0.0);
        fft_exec(&w->plan, w->t, 1);                                  /* ifft(|AT|^2) n */
        for (int i = 0; i < n; ++i) w->t[i] = cmul(cscale(w->t[i], inv_n), RW[i]);
        fft_exec(&w->plan, w->t, 0);                                  /* fft(ifft(|AT|^2) RW) */
        const double dtfr = p->dT * p->fr;
        for (int i = 0; i < n; ++i) {
            const cplx rs = cscale(w->t[i], dtfr);
            const cplx g = cmk((1.0 - p->fr) * w->it[i] + rs.re, rs.im);
            w->t[i] = cmul(w->at[i], g);
        }
    }
    fft_exec(&w->plan, w->t, 1);                                      /* ifft(Q) n */
    for (int i = 0; i < n; ++i) {
        const cplx m = cscale(w->t[i], inv_n);
        const double g = p->gamma * W[i];
        out[i] = cdiv(cmk(-g * m.im, g * m.re), w->e[i]);             /* i gamma W M / e^{Lz} */
    }
}

/* save i at position zc (units): AT = fft(AW e^{Lz}), AW e^{Lz} fftshifted x dT n */
static void save(const ofx_gnlse_params* p, const double* B, gwork* w, const cplx* y, int i, long long zc,
                 double unit, double* AT_out, double* AW_out) {
    const int n = p->n;
    cplx* at = (cplx*)AT_out + (size_t)i * n;
    cplx* aw = (cplx*)AW_out + (size_t)i * n;
    lz(p, B, (double)zc * unit, w->e);
    for (int k = 0; k < n; ++k) at[k] = cmul(y[k], w->e[k]);
    for (int k = 0; k < n; ++k) aw[k] = cscale(cscale(at[(k + n / 2) % n], p->dT), (double)n);
    fft_exec(&w->plan, at, 0);
}

/* save point i: i total / (n_saves - 1), rounded half up */
static long long save_point(int i, long long total, long long nm1) { return ((long long)i * total + nm1 / 2) / nm1; }

/* stages 2..last+1 of a Dormand-Prince step of hc units from (zc, y) with k[0] = k1
 * given, into k[1..last]; out = the 5th-order value y + h sum a_7j k_j (its k_7 is
 * computed only when last == 6) */
static void dp_stages(const ofx_gnlse_params* p, const double* B, const double* W, const cplx* RW, gwork* w,
                      cplx* const* k, long long zc, long long hc, double unit, int last, cplx* out) {
    const int n = p->n;
    const double hz = (double)hc * unit;
    for (int s = 1; s <= last; ++s) {
        for (int i = 0; i < n; ++i) {
            cplx a = cmk(0.0, 0.0);
            for (int j = 0; j < s; ++j)
                if (DP_A[s][j] != 0.0) a = cadd(a, cscale(k[j][i], DP_A[s][j]));
            w->ys[i] = cadd(w->y[i], cscale(a, hz));
        }
        const long long zs = zc + (long long)nearbyint(DP_C[s] * (double)hc);
        rhs(p, B, W, RW, w, (double)zs * unit, w->ys, k[s]);
    }
    for (int i = 0; i < n; ++i) {
        cplx a = cmk(0.0, 0.0);
        for (int j = 0; j < 6; ++j)
            if (DP_A[6][j] != 0.0) a = cadd(a, cscale(k[j][i], DP_A[6][j]));
        out[i] = cadd(w->y[i], cscale(a, hz));
    }
}

static int run_one(const ofx_gnlse_params* p, const cplx* A, const double* B, const double* W, const cplx* RW,
                   double* AT_out, double* AW_out, long long* trace, int trace_cap, const long long* forced,
                   int n_forced, int* attempts_out, int* accepted_out) {
    const int n = p->n;
    gwork w;
    int rc = gwork_init(&w, n);
    if (rc) { gwork_free(&w); return rc; }
    const long long total = 1LL << Z_BITS, hmax = total / 10;
    const double unit = p->length / (double)total, thr = p->atol / p->rtol;
    const long long nm1 = p->n_saves - 1;

    memcpy(w.y, A, sizeof(cplx) * (size_t)n);                        /* y = ifft(A) */
    fft_exec(&w.plan, w.y, 1);
    for (int i = 0; i < n; ++i) w.y[i] = cscale(w.y[i], 1.0 / (double)n);
    long long zc = 0;
    save(p, B, &w, w.y, 0, 0, unit, AT_out, AW_out);
    int si = 1;
    int f = 0;
    rhs(p, B, W, RW, &w, 0.0, w.y, w.buf[f]);
    double ny = norm(w.y, n);
    const double nf = norm(w.buf[f], n);
    long long h;
    if (nf == 0.0) h = hmax;
    else {
        const double hh = (0.8 * pow(p->rtol, 0.2)) * fmax(ny, thr) / nf / unit;
        h = !(hh < (double)hmax) ? hmax : (hh < 1.0 ? 1 : (long long)hh);   /* NaN: hmax */
    }
    int att = 0, acc = 0, fi = 0;
    while (zc < total && rc == 0) {
        h = h > hmax ? hmax : (h < 1 ? 1 : h);
        long long hc = h;
        if (1.1 * (double)hc >= (double)(total - zc)) hc = total - zc;    /* stretch to the end */
        int nofailed = 1;
        double err = 0.0, nyn = 0.0;
        cplx* k[7];
        for (int s_ = 0; s_ < 7; ++s_) k[s_] = w.buf[(f + s_) % 7];
        for (;;) {
            if (forced) {
                if (fi >= n_forced) { rc = -3; break; }
                hc = forced[2 * fi];
            }
            dp_stages(p, B, W, RW, &w, k, zc, hc, unit, 6, w.ynew);
            const double hz = (double)hc * unit;
            for (int i = 0; i < n; ++i) {
                cplx e = cmk(0.0, 0.0);
                for (int j = 0; j < 7; ++j)
                    if (DP_E[j] != 0.0) e = cadd(e, cscale(k[j][i], DP_E[j]));
                w.acc[i] = cscale(e, hz);
            }
            nyn = norm(w.ynew, n);
            err = norm(w.acc, n) / fmax(fmax(ny, nyn), thr);
            if (!isfinite(err) || att >= MAX_ATTEMPTS) { rc = isfinite(err) ? -5 : -4; break; }
            int ok = err <= p->rtol;
            if (forced) { ok = forced[2 * fi + 1] != 0; ++fi; }
            if (trace && att < trace_cap) { trace[2 * att] = hc; trace[2 * att + 1] = ok; }
            ++att;
            if (ok) break;
            if (nofailed) {
                nofailed = 0;
                const long long hi = (long long)((double)hc * fmax(0.1, 0.8 * pow(p->rtol / err, 0.2)));
                hc = hi < 1 ? 1 : hi;
            } else {
                hc = hc / 2 < 1 ? 1 : hc / 2;
            }
        }
        if (rc) break;
        ++acc;
        /* save points inside the step: a separate step of exactly that length from zc
           (stages k2..k6 overwrite the accepted step's, which are not needed again) */
        while (si < p->n_saves && save_point(si, total, nm1) < zc + hc) {
            const long long sp = save_point(si, total, nm1);
            dp_stages(p, B, W, RW, &w, k, zc, sp - zc, unit, 5, w.ys);
            save(p, B, &w, w.ys, si, sp, unit, AT_out, AW_out);
            ++si;
        }
        zc += hc;
        cplx* t = w.y; w.y = w.ynew; w.ynew = t;
        f = (f + 6) % 7;                                                /* FSAL: k_7 is the next k_1 */
        ny = nyn;
        if (si < p->n_saves && save_point(si, total, nm1) == zc) {
            save(p, B, &w, w.y, si, zc, unit, AT_out, AW_out);
            ++si;
        }
        if (nofailed) {
            const double temp = 1.25 * pow(err / p->rtol, 0.2);
            h = temp > 0.2 ? (long long)((double)hc / temp) : 5 * hc;
        } else {
            h = hc;
        }
    }
    *attempts_out = att;
    *accepted_out = acc;
    gwork_free(&w);
    return rc;
}

int ofx_gnlse_oracle_run(const ofx_gnlse_params* p, int n_pulses, const double* A, const double* B,
                         const double* W, const double* RW, double* AT_out, double* AW_out,
                         long long* trace, int trace_cap, const long long* forced, int n_forced,
                         int* attempts, int* accepted, int nthreads) {
    if (!p || !A || !B || !W || !AT_out || !AW_out || !attempts || !accepted || n_pulses < 1) return -1;
    if (p->n < 4 || (p->n & (p->n - 1)) || p->n_saves < 2 || !(p->length > 0.0) || !(p->rtol > 0.0) ||
        !(p->atol > 0.0) || (trace && trace_cap < 0) || (forced && n_forced < 0))
        return -1;
    const size_t per = (size_t)p->n_saves * (size_t)p->n * 2;
    int rc_all = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) reduction(min : rc_all) if (n_pulses > 1)
#endif
    for (int b = 0; b < n_pulses; ++b) {
        const int rc = run_one(p, (const cplx*)A + (size_t)b * p->n, B, W, (const cplx*)RW, AT_out + b * per,
                               AW_out + b * per, trace ? trace + (size_t)b * 2 * trace_cap : NULL, trace_cap,
                               forced ? forced + (size_t)b * 2 * n_forced : NULL, n_forced, attempts + b,
                               accepted + b);
        if (rc < rc_all) rc_all = rc;
    }
    (void)nthreads;
    return rc_all;
}
