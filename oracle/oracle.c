/*
 * oracle.c -- FP64 CPU restatement of OptiFax's chi(2) crystal-pass solver.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle for the GPU propagator
 * in optifax_gb300/csrc/.  Only tests/, __graft_entry__.smoke() and bench.py
 * (its cpu_baseline leg and its --impl reference arm) may load it.  The
 * product path never calls it.
 *
 * Parity status: PINNED to the reference's own CUDA kernels.  The reference
 * ships no golden vectors, fixtures or tests for this path, and its MATLAB
 * code cannot run here; its MEX kernels (OPO_CUDA_BATCH_XTAL.cu, _BATCH_OP.cu,
 * _NO_BC.cu, _HARD_BC.cu, ode23/OPO_CUDA_ODE23.cu) are compiled unmodified into
 * cubins and driven with cuFFT by oracle/ref_mex.cpp.
 * tests/test_reference_kernels_gpu.py checks this restatement against them on
 * the GPU: identical step schedules (Heun), and fields within the drift of
 * cuFFT's FP32 round trips; tests/test_golden_cpu.py does the same on the CPU
 * against their outputs saved in tests/golden/.  Known-answer tests
 * (pure dispersion, FFT, convergence order, replay, the reject rules) are in
 * tests/test_oracle.py.  The NEE_CPU.m schedule (MATLAB only) stays unpinned.
 *
 * Three schedules are restated, each in double precision, with every input
 * value taken exactly as the reference receives it (w0, h, G, beta, alpha are
 * FP32 values in the reference; they arrive here already rounded):
 *
 *   OFX_ORACLE_HEUN_MEX  toolbox/lib/MEXlib/src/OPO_CUDA_BATCH_XTAL.cu:373-525
 *                        (host driver), kernels :142-305.  Variants:
 *                        OPO_CUDA_BATCH_OP.cu (shared poling G[k], :221),
 *                        OPO_CUDA_NO_BC.cu (unshifted time :172, no absorber
 *                        :399-402, truncated chunk count, no k<Nsteps guard),
 *                        OPO_CUDA_HARD_BC.cu (hard absorber :118-129).
 *   OFX_ORACLE_RK23_MEX  toolbox/lib/MEXlib/src/ode23/OPO_CUDA_ODE23.cu:375-557
 *                        (Bogacki-Shampine 3(2) with FSAL taken before the
 *                        dispersion sub-step, step doubling).
 *   OFX_ORACLE_HEUN_NEE  toolbox/lib/internal/main/NEE_CPU.m:1-122 (the
 *                        MATLAB CPU solver, plotting removed).
 *
 * The FFT is a plain radix-2 FP64 transform of our own (FFTW, which MATLAB
 * uses, and cuFFT, which the MEX uses, are closed binaries and neither is
 * available here); any transform exact to FP64 rounding is equivalent.
 *
 * Threads: independent schedules (pulses) run in parallel.  A call with one
 * schedule of 4096 points or more and an explicit thread count (nthreads > 1)
 * spreads the pass over those threads instead; with nthreads = 0 a pass stays
 * on one thread.  Each schedule of one pulse runs as one parallel region per
 * pass (run_heun_mex_team, run_rk23_mex_team, run_heun_nee_team): each thread
 * owns a span of points, updates the stages of its span with a halo of two (Heun)
 * or three (RK23) points, and runs the FFT stages that fit its span without
 * synchronisation, so a rejected Heun attempt costs one barrier and an accepted
 * one 2 log2(T) + 4.  A batch sharing one schedule spreads each point loop and
 * FFT stage separately instead.  Each point's arithmetic is the same whichever thread
 * does it and the only reductions (a max and an OR) are exact, so the results do
 * not depend on the thread count.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle.h"

#include "oracle_fft.h"

int ofx_oracle_fft(const double* in, double* out, int n, int inverse) {
    fft_plan p;
    if (fft_plan_init(&p, n)) { fft_plan_free(&p); return OFX_ORACLE_EINVAL; }
    memcpy(out, in, sizeof(double) * 2 * (size_t)n);
    fft_exec(&p, (cplx*)out, inverse);
    fft_plan_free(&p);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Physics pieces shared by the schedules                                    */
/* ------------------------------------------------------------------------ */

/* Sample time used by the nonlinear drive for array index i.
 *   shifted:   OPO_CUDA_BATCH_XTAL.cu:173-180  t = (i +- N/2) dt
 *   unshifted: OPO_CUDA_NO_BC.cu:172, OPO_CUDA_ODE23.cu:176  t = i dt
 *   nee:       NEE_CPU.m:12,53  t = fftshift((-N/2:N/2-1) dt)            */
static double sample_time(int mode, int i, int n, double dt) {
    if (mode == OFX_TIME_SHIFTED) {
        if (i > n / 2) return dt * (double)(i - n / 2);
        return dt * (double)(i + n / 2);
    } else if (mode == OFX_TIME_UNSHIFTED) {
        return dt * (double)i;
    } else {
        return (i < n / 2) ? dt * (double)i : dt * (double)(i - n);
    }
}

/* NL = A^2 e^{i phi} + 2 |A|^2 e^{-i phi},  phi = w0 t_i - bdwz
 * (OPO_CUDA_BATCH_XTAL.cu:182-187; NEE_CPU.m:98-101). */
static inline cplx nl_point(cplx a, cplx cw, cplx ez) {
    cplx e = cmul(cw, ez);
    const double m2 = a.re * a.re + a.im * a.im;          /* |A|^2 */
    cplx a2 = cmul(a, a);
    return cadd(cmul(a2, e), cscale(cconj(e), 2.0 * m2));
}

static void nl_eval(const cplx* A, cplx* NL, int n, const cplx* cw0, double bdwz) {
    const cplx ez = cexpi(-bdwz);                /* exp(i phi) = exp(i w0 t_i) exp(-i bdwz) */
#pragma omp parallel for schedule(static) if (par_ok((size_t)n))
    for (int i = 0; i < n; ++i) NL[i] = nl_point(A[i], cw0[i], ez);
}

/* K = -i h G (NL - i/(2 dt w0) (NL[i+1] - NL[i-1])), periodic neighbours
 * (OPO_CUDA_BATCH_XTAL.cu:221-249; NEE_CPU.m:103-105). */
static inline cplx k_point(cplx nlp, cplx nlm, cplx nl, double hmod, double g, double c_shock) {
    cplx d = csub(nlp, nlm);
    /* i * c_shock * d */
    cplx id = cmk(-c_shock * d.im, c_shock * d.re);
    cplx in = csub(nl, id);
    /* -i * hG * in */
    double hg = hmod * g;
    return cmk(hg * in.im, -hg * in.re);
}

static void k_eval(const cplx* NL, cplx* K, int n, double hmod, double g, double c_shock) {
#pragma omp parallel for schedule(static) if (par_ok((size_t)n))
    for (int i = 0; i < n; ++i) {
        int ip = (i + 1 == n) ? 0 : i + 1;
        int im = (i == 0) ? n - 1 : i - 1;
        K[i] = k_point(NL[ip], NL[im], NL[i], hmod, g, c_shock);
    }
}

/* Absorbing boundary factor for array index i (OPO_CUDA_BATCH_XTAL.cu:105-137,
 * window gi1 = 6(N/16), gi2 = 10(N/16) at :412-413; HARD_BC: factor 0 with
 * a=2; NO_BC: gi1 = gi2 = 0, i.e. no points). */
static double abc_factor_mex(int mode, int i, int n) {
    if (mode == OFX_ABC_NONE) return 1.0;
    int gi1 = 6 * (n / 16), gi2 = 10 * (n / 16);
    if (!(i > gi1 && i < gi2)) return 1.0;
    if (mode == OFX_ABC_HARD) return 0.0;
    double pos = (24.0 * 2.0 / (double)n) * fabs((double)i - (double)n / 2.0);
    double g = cosh(pos);
    return 1.0 - 1.0 / (g * g);
}

/* NEE_CPU.m:114-121: t_idx = range(t) - |2t| < b range(t), factor
 * 1 - sech(a (1 - |2t|/range(t)))^2, a = 24, b = 0.25, t = fftshift(t). */
static double abc_factor_nee(int i, int n, double dt) {
    double t = sample_time(OFX_TIME_NEE, i, n, dt);
    double range = (double)(n - 1) * dt;
    double a2t = fabs(2.0 * t);
    if (!(range - a2t < 0.25 * range)) return 1.0;
    double s = 1.0 / cosh(24.0 * (1.0 - a2t / range));
    return 1.0 - s * s;
}

/* ------------------------------------------------------------------------ */
/* Schedules                                                                 */
/* ------------------------------------------------------------------------ */

typedef struct {
    const ofx_oracle_params* p;
    int b0, nb;                 /* pulses in this schedule */
    const cplx* E_in;
    const double* alpha;
    const double* G;
    const double* beta;
    cplx* A_out;
    cplx* Ap; long long ap_len;
    double* stepmods;
    int* trace; int trace_cap; int* n_attempts;
    const int* forced; int n_forced;
    ofx_oracle_stats* stats;
} sched_ctx;

#define OFX_DISP_SLOTS 8

typedef struct {
    int n;
    fft_plan plan;
    cplx *A0, *A1, *E, *NL, *K1, *K2, *K3, *K4;
    cplx* cw0;          /* carrier exp(i w0 t_i), tabulated once */
    double* abc;        /* absorber factor per point, tabulated once */
    cplx* disp;         /* OFX_DISP_SLOTS tables of alpha^s exp(-i beta s); slot disp_slot(s) */
    double disp_s[OFX_DISP_SLOTS];      /* the step size each slot holds, -1 for none */
} work;

/* Step sizes are whole numbers of z-samples; a pass moves among a few of them, so
 * a small direct-mapped cache of dispersion tables (keyed by s mod 8) saves the
 * n exponentials and powers of a table rebuild at most changes of step size. */
static int disp_slot(double s) { return (int)((long long)s & (OFX_DISP_SLOTS - 1)); }

static int work_init(work* w, int n, int nb, int time_mode, int nee, int abc_mode, double w0, double dt) {
    memset(w, 0, sizeof(*w));
    w->n = n;
    if (fft_plan_init(&w->plan, n)) return -1;
    size_t sz = sizeof(cplx) * (size_t)n * (size_t)nb;
    w->A0 = (cplx*)malloc(sz); w->A1 = (cplx*)malloc(sz); w->E = (cplx*)malloc(sz);
    w->NL = (cplx*)malloc(sizeof(cplx) * (size_t)n);
    w->K1 = (cplx*)malloc(sz); w->K2 = (cplx*)malloc(sz);
    w->K3 = (cplx*)malloc(sz); w->K4 = (cplx*)malloc(sz);
    w->cw0 = (cplx*)malloc(sizeof(cplx) * (size_t)n);
    w->abc = (double*)malloc(sizeof(double) * (size_t)n);
    w->disp = (cplx*)malloc(sizeof(cplx) * (size_t)n * OFX_DISP_SLOTS);
    for (int j = 0; j < OFX_DISP_SLOTS; ++j) w->disp_s[j] = -1.0;
    if (!w->A0 || !w->A1 || !w->E || !w->NL || !w->K1 || !w->K2 || !w->K3 || !w->K4 || !w->cw0 || !w->abc ||
        !w->disp)
        return -2;
    for (int i = 0; i < n; ++i) {
        w->cw0[i] = cexpi(w0 * sample_time(time_mode, i, n, dt));
        w->abc[i] = nee ? abc_factor_nee(i, n, dt) : abc_factor_mex(abc_mode, i, n);
    }
    return 0;
}

/* alpha^s exp(-i beta s) per mode (OPO_CUDA_BATCH_XTAL.cu:255-305), recomputed only
 * when the step size changes */
static const cplx* disp_factor(work* w, const double* beta, const double* alpha, double s) {
    const int slot = disp_slot(s);
    cplx* f = w->disp + (size_t)slot * (size_t)w->n;
    if (w->disp_s[slot] != s) {
        const int n = w->n;
#pragma omp parallel for schedule(static) if (par_ok((size_t)n))
        for (int i = 0; i < n; ++i) f[i] = cscale(cexpi(-beta[i] * s), pow(alpha[i], s));
        w->disp_s[slot] = s;
    }
    return f;
}

static void work_free(work* w) {
    fft_plan_free(&w->plan);
    free(w->A0); free(w->A1); free(w->E); free(w->NL);
    free(w->K1); free(w->K2); free(w->K3); free(w->K4); free(w->cw0); free(w->abc); free(w->disp);
}

static double g_at(const sched_ctx* c, int k, int b) {
    const ofx_oracle_params* p = c->p;
    if (k < 0) k = 0;
    if (k >= p->S) k = p->S - 1;
    return p->g_per_pulse ? c->G[(size_t)k + (size_t)(c->b0 + b) * (size_t)p->S] : c->G[k];
}

/* one NL+K stage for every pulse of the schedule: K = f(X) */
static void stage(const sched_ctx* c, work* w, const cplx* X, cplx* K, double pos,
                  double hmod, int kidx) {
    const ofx_oracle_params* p = c->p;
    const int n = p->N;
    double bdwz = p->bdiffw0 * pos * p->h;
    double c_shock = 1.0 / (2.0 * p->dt * p->w0);
    for (int b = 0; b < c->nb; ++b) {
        nl_eval(X + (size_t)b * n, w->NL, n, w->cw0, bdwz);
        k_eval(w->NL, K + (size_t)b * n, n, hmod, g_at(c, kidx, b), c_shock);
    }
}

/* error classification over all pulses of the schedule:
 * OPO_CUDA_BATCH_XTAL.cu:325-349 (pct = 100 |E-A1|/(|E|+1), >= maxErr sets
 * flag0, else >= minErr sets flag1, points with |E| == 0 skipped);
 * ODE23 uses 4*100*0.5*|E-A1| (OPO_CUDA_ODE23.cu:332-335). */
static inline int classify_point(const ofx_oracle_params* p, cplx e, cplx a1, double scale, double* pm) {
    int flags = 0;
    double ae = cabs2(e);
    if (ae > 0) {
        double pct = scale * cabs2(csub(e, a1)) / (ae + 1.0);
        if (pct > *pm) *pm = pct;
        if (pct >= p->maxErr) flags |= 1;
        else if (pct >= p->minErr) flags |= 2;
    }
    if (isnan(e.re) || isnan(e.im)) flags |= 4;
    return flags;
}

static int classify(const sched_ctx* c, const cplx* E, const cplx* A1, double scale,
                    double* pct_max_out) {
    const ofx_oracle_params* p = c->p;
    int flags = 0; double pm = 0.0;
    size_t tot = (size_t)p->N * (size_t)c->nb;
#pragma omp parallel for schedule(static) reduction(max : pm) reduction(| : flags) if (par_ok(tot))
    for (size_t i = 0; i < tot; ++i) flags |= classify_point(p, E[i], A1[i], scale, &pm);
    *pct_max_out = pm;
    return flags;
}

static void record(sched_ctx* c, int attempt, int k, int s, int flags, int accepted) {
    if (c->trace && attempt < c->trace_cap) {
        c->trace[3 * attempt + 0] = k;
        c->trace[3 * attempt + 1] = s;
        c->trace[3 * attempt + 2] = (flags & 3) | (accepted ? 8 : 0) | (flags & 4);
    }
}

/* accepted step's linear sub-step: absorber, FFT, dispersion x stepmod, snapshot,
 * stepmods record, IFFT, 1/N  (OPO_CUDA_BATCH_XTAL.cu:469-485, :255-305). */
static void dispersion_step(sched_ctx* c, work* w, cplx* E, cplx* A0, int s, int chunk,
                            int nchunks, int k) {
    const ofx_oracle_params* p = c->p;
    const int n = p->N;
    double inv_n = 1.0 / (double)n;
    for (int b = 0; b < c->nb; ++b) {
        cplx* e = E + (size_t)b * n;
#pragma omp parallel for schedule(static) if (par_ok((size_t)n))
        for (int i = 0; i < n; ++i) e[i] = cscale(e[i], w->abc[i]);
        fft_exec(&w->plan, e, 0);
        const cplx* f = disp_factor(w, c->beta, c->alpha, (double)s);
#pragma omp parallel for schedule(static) if (par_ok((size_t)n))
        for (int i = 0; i < n; ++i) e[i] = cmul(e[i], f[i]);
        if (c->Ap) {
            long long off = ((long long)(c->b0 + b) * nchunks + chunk) * (long long)n;
            if (off >= 0 && off + n <= c->ap_len) memcpy(c->Ap + off, e, sizeof(cplx) * (size_t)n);
            else c->stats->status |= OFX_ORACLE_STATUS_AP_RANGE;
        }
        fft_exec(&w->plan, e, 1);
        cplx* a0 = A0 + (size_t)b * n;
#pragma omp parallel for schedule(static) if (par_ok((size_t)n))
        for (int i = 0; i < n; ++i) a0[i] = cscale(e[i], inv_n);
    }
    if (c->stepmods && k < p->stepmods_limit && k < p->S && k >= 0) c->stepmods[k] = (double)s;
}

static int get_flags(sched_ctx* c, int attempt, int computed) {
    if (c->forced && attempt < c->n_forced) return (c->forced[attempt] & 3) | (computed & 4);
    return computed;
}

/* OPO_CUDA_BATCH_XTAL.cu:373-525 and its variants */
static void run_heun_mex(sched_ctx* c, work* w) {
    const ofx_oracle_params* p = c->p;
    const int n = p->N;
    const double sel = p->sel;
    double k = 0.0, stepprev = 4.0, stepmod = stepprev, stepend;
    int nchunks = (int)((double)p->S / sel);
    if (p->chunk_mode == OFX_CHUNKS_CEIL && (double)nchunks * sel < (double)p->S) nchunks += 1;
    int attempt = 0;
    double pm;
    for (int chunk = 0; chunk < nchunks; ++chunk) {
        stepmod = stepprev;
        double cend = (double)(chunk + 1) * sel;
        for (; k < cend && (p->chunk_mode != OFX_CHUNKS_CEIL || k < (double)p->S); k = k + stepmod) {
            int kidx = (int)k;
            double hmod = stepmod * p->h;
            stage(c, w, w->A0, w->K1, k, hmod, kidx);
            size_t tot = (size_t)n * c->nb;
#pragma omp parallel for schedule(static) if (par_ok(tot))
            for (size_t i = 0; i < tot; ++i)
                w->A1[i] = cadd(w->A0[i], cadd(cscale(w->K1[i], 0.5), cscale(w->K1[i], 0.5)));
            stage(c, w, w->A1, w->K2, k + stepmod, hmod, kidx);
#pragma omp parallel for schedule(static) if (par_ok(tot))
            for (size_t i = 0; i < tot; ++i)
                w->E[i] = cadd(w->A0[i], cadd(cscale(w->K2[i], 0.5), cscale(w->K1[i], 0.5)));
            int fl = classify(c, w->E, w->A1, 100.0, &pm);
            fl = get_flags(c, attempt, fl);
            if (fl & 4) c->stats->status |= OFX_ORACLE_STATUS_NAN;
            c->stats->pct_max_last = pm;
            if ((fl & 1) && stepmod > 1.0 && (k - stepmod) > 0.0) {
                record(c, attempt, kidx, (int)stepmod, fl, 0);
                c->stats->rejected++;
                k = k - stepmod;
                stepmod = stepmod - 1.0;
                stepprev = stepmod;
            } else {
                record(c, attempt, kidx, (int)stepmod, fl, 1);
                c->stats->accepted++;
                c->stats->z_steps += (long long)stepmod;
                dispersion_step(c, w, w->E, w->A0, (int)stepmod, chunk, nchunks, kidx);
                if (k + stepmod >= cend && k < cend - 1.0) {
                    stepend = (cend - k) - 1.0;
                    stepprev = stepmod;
                    stepmod = stepend;
                } else {
                    if (!(fl & 2) && !(fl & 1) && (k + stepmod + 1.0) < cend - 1.0)
                        stepmod = stepmod + 1.0;
                    stepprev = stepmod;
                }
            }
            attempt++;
        }
    }
    c->stats->attempts = attempt;
    c->stats->k_final = k;
    c->stats->stepmod_final = stepmod;
    c->stats->nchunks = nchunks;
    if (c->n_attempts) *c->n_attempts = attempt;
}

#ifdef _OPENMP
/* Team size for one pass: the largest power of two within the thread count that
 * leaves each thread at least 1024 points; 1 (the loop-by-loop path) for a lone
 * thread, a batch sharing one schedule, or a call already inside a parallel region. */
static int team_size(int n, int nb) {
    if (!t_inner || nb != 1 || n < OFX_PAR_MIN || omp_in_parallel()) return 1;
    int t = 1, m = omp_get_max_threads();
    while (2 * t <= m && n / (2 * t) >= 1024) t *= 2;
    return t;
}

/* dispersion_step for the points [tid n/T, (tid+1) n/T) of one pulse, called by
 * every thread of a team after the barrier that completes E: the absorber is
 * applied in the bit-reversal gather into y (a free n-point buffer), the dispersion
 * factor (this thread's points of the cached table for step size s; my_s is the
 * thread's view of the cache slots) in the gather back into E, then A0 = E / N on
 * the thread's points.  With records (the MEX schedules) the spectrum is also
 * snapshotted into Ap and thread 0 records stepmods[kidx].  Ends without a
 * barrier: the caller adds one after any further writes of its own points. */
static void dispersion_team(sched_ctx* c, work* w, cplx* y, double* my_s, int s, int chunk, int nchunks,
                            int kidx, int tid, int T, int records) {
    const ofx_oracle_params* p = c->p;
    const int n = p->N, span = n / T, lo = tid * span, hi = lo + span;
    const double inv_n = 1.0 / (double)n;
    const int slot = disp_slot((double)s);
    cplx* f = w->disp + (size_t)slot * (size_t)n;
    if (my_s[slot] != (double)s) {
        for (int i = lo; i < hi; ++i)
            f[i] = cscale(cexpi(-c->beta[i] * (double)s), pow(c->alpha[i], (double)s));
        my_s[slot] = (double)s;
    }
    const int* rev = w->plan.rev;
    cplx* e = w->E;
    for (int i = lo; i < hi; ++i) y[i] = cscale(e[rev[i]], w->abc[rev[i]]);
    fft_team_stages(&w->plan, y, 0, tid, T);
    if (records && c->Ap) {
        long long off = ((long long)c->b0 * nchunks + chunk) * (long long)n;
        if (off >= 0 && off + n <= c->ap_len) {
            for (int i = lo; i < hi; ++i) c->Ap[off + i] = cmul(y[i], f[i]);
        } else if (tid == 0) c->stats->status |= OFX_ORACLE_STATUS_AP_RANGE;
    }
    for (int i = lo; i < hi; ++i) e[i] = cmul(y[rev[i]], f[rev[i]]);
    fft_team_stages(&w->plan, e, 1, tid, T);
    for (int i = lo; i < hi; ++i) w->A0[i] = cscale(e[i], inv_n);
    if (records && tid == 0 && c->stepmods && kidx < p->stepmods_limit && kidx < p->S && kidx >= 0)
        c->stepmods[kidx] = (double)s;
}

/* Both Heun stages and the error test for points [lo, hi) of one pulse.  The
 * centred difference in K needs NL one point further out on each side, and the
 * second stage needs A1 (hence K1) one point further out again, so the span
 * recomputes NL1 on [lo-2, hi+2) and K1, A1, NL2 on [lo-1, hi+1) (indices
 * periodic).  Every value is the expression run_heun_mex evaluates for that
 * point.  Scratch: 4 (hi - lo + 4) values.  Returns the classify flags; *pm the
 * largest percentage. */
static int heun_span(const ofx_oracle_params* p, const cplx* A0, cplx* E, const cplx* cw0, int lo, int hi,
                     cplx ez1, cplx ez2, double hmod, double g, double c_shock, cplx* scratch, double* pm) {
    const int n = p->N, m = hi - lo + 4;
    cplx *nl1 = scratch, *k1 = scratch + m, *a1 = scratch + 2 * m, *nl2 = scratch + 3 * m;
#define OFX_WRAP(i) ((i) < 0 ? (i) + n : ((i) >= n ? (i) - n : (i)))
    for (int l = 0; l < m; ++l) {                       /* point lo - 2 + l */
        const int gi = OFX_WRAP(lo - 2 + l);
        nl1[l] = nl_point(A0[gi], cw0[gi], ez1);
    }
    for (int l = 1; l < m - 1; ++l) {
        const int gi = OFX_WRAP(lo - 2 + l);
        k1[l] = k_point(nl1[l + 1], nl1[l - 1], nl1[l], hmod, g, c_shock);
        a1[l] = cadd(A0[gi], cadd(cscale(k1[l], 0.5), cscale(k1[l], 0.5)));
        nl2[l] = nl_point(a1[l], cw0[gi], ez2);
    }
#undef OFX_WRAP
    int flags = 0;
    for (int l = 2; l < m - 2; ++l) {
        const int i = lo - 2 + l;
        cplx k2 = k_point(nl2[l + 1], nl2[l - 1], nl2[l], hmod, g, c_shock);
        E[i] = cadd(A0[i], cadd(cscale(k2, 0.5), cscale(k1[l], 0.5)));
        flags |= classify_point(p, E[i], a1[l], 100.0, pm);
    }
    return flags;
}

/* run_heun_mex for one pulse on a team of T threads (one parallel region for the
 * whole pass).  Every thread runs the step control on its own copy of the
 * schedule state; the flags and the largest percentage are combined exactly (OR,
 * max) so every copy takes the same decisions.  Thread 0 alone writes the
 * statistics, trace and stepmods.  Per attempt: the span update, one barrier for
 * the error test; per accepted step: absorber, FFT, dispersion, snapshot, inverse
 * FFT and 1/N on each thread's own points, with barriers only where a step reads
 * other threads' points.  The results are bit-identical to run_heun_mex.
 * Returns 0, or -1 (nothing done) when the team or its scratch is unavailable. */
static int run_heun_mex_team(sched_ctx* c, work* w, int T) {
    const ofx_oracle_params* p = c->p;
    const int n = p->N, span = n / T;
    const double sel = p->sel, c_shock = 1.0 / (2.0 * p->dt * p->w0);
    int nchunks = (int)((double)p->S / sel);
    if (p->chunk_mode == OFX_CHUNKS_CEIL && (double)nchunks * sel < (double)p->S) nchunks += 1;
    cplx* scratch = (cplx*)malloc(sizeof(cplx) * 4 * (size_t)(span + 4) * (size_t)T);
    double* part_pm = (double*)malloc(sizeof(double) * 2 * (size_t)T);
    int* part_fl = (int*)malloc(sizeof(int) * 2 * (size_t)T);
    int ran = 0;
    if (scratch && part_pm && part_fl) {
#pragma omp parallel num_threads(T)
        if (omp_get_num_threads() == T) {
            const int tid = omp_get_thread_num(), lo = tid * span, hi = lo + span;
            cplx* mine = scratch + 4 * (size_t)(span + 4) * (size_t)tid;
            double k = 0.0, stepprev = 4.0, stepmod = stepprev, stepend, pm = 0.0;
            double my_s[OFX_DISP_SLOTS];        /* this thread's view of the table slots (its own points) */
            for (int j = 0; j < OFX_DISP_SLOTS; ++j) my_s[j] = -1.0;
            int attempt = 0;
            for (int chunk = 0; chunk < nchunks; ++chunk) {
                stepmod = stepprev;
                double cend = (double)(chunk + 1) * sel;
                for (; k < cend && (p->chunk_mode != OFX_CHUNKS_CEIL || k < (double)p->S); k = k + stepmod) {
                    const int kidx = (int)k;
                    const double hmod = stepmod * p->h, g = g_at(c, kidx, 0);
                    const cplx ez1 = cexpi(-(p->bdiffw0 * k * p->h));
                    const cplx ez2 = cexpi(-(p->bdiffw0 * (k + stepmod) * p->h));
                    double my_pm = 0.0;
                    const int slot = attempt & 1;
                    part_fl[slot * T + tid] = heun_span(p, w->A0, w->E, w->cw0, lo, hi, ez1, ez2, hmod, g,
                                                        c_shock, mine, &my_pm);
                    part_pm[slot * T + tid] = my_pm;
#pragma omp barrier
                    int fl = 0;
                    pm = 0.0;
                    for (int t = 0; t < T; ++t) {
                        fl |= part_fl[slot * T + t];
                        if (part_pm[slot * T + t] > pm) pm = part_pm[slot * T + t];
                    }
                    fl = get_flags(c, attempt, fl);
                    if (tid == 0) {
                        if (fl & 4) c->stats->status |= OFX_ORACLE_STATUS_NAN;
                        c->stats->pct_max_last = pm;
                    }
                    if ((fl & 1) && stepmod > 1.0 && (k - stepmod) > 0.0) {
                        if (tid == 0) { record(c, attempt, kidx, (int)stepmod, fl, 0); c->stats->rejected++; }
                        k = k - stepmod;
                        stepmod = stepmod - 1.0;
                        stepprev = stepmod;
                    } else {
                        const int s = (int)stepmod;
                        if (tid == 0) {
                            record(c, attempt, kidx, s, fl, 1);
                            c->stats->accepted++;
                            c->stats->z_steps += (long long)stepmod;
                        }
                        dispersion_team(c, w, w->K1, my_s, s, chunk, nchunks, kidx, tid, T, 1);
#pragma omp barrier
                        if (k + stepmod >= cend && k < cend - 1.0) {
                            stepend = (cend - k) - 1.0;
                            stepprev = stepmod;
                            stepmod = stepend;
                        } else {
                            if (!(fl & 2) && !(fl & 1) && (k + stepmod + 1.0) < cend - 1.0)
                                stepmod = stepmod + 1.0;
                            stepprev = stepmod;
                        }
                    }
                    attempt++;
                }
            }
            if (tid == 0) {
                c->stats->attempts = attempt;
                c->stats->k_final = k;
                c->stats->stepmod_final = stepmod;
                c->stats->nchunks = nchunks;
                if (c->n_attempts) *c->n_attempts = attempt;
                ran = 1;
            }
        }
    }
    free(scratch); free(part_pm); free(part_fl);
    return ran ? 0 : -1;
}

/* The three Bogacki-Shampine stages after K1 and the error test for points
 * [lo, hi) of one pulse (run_rk23_mex's attempt).  K4 at a point needs the drive
 * of E one point out, E needs K3 there, K3 the drive of A1' = A0 + 3/4 K2 two
 * points out and K2 the drive of A1 three points out, so the span recomputes
 * NL2, K2 and A1' on [lo-3, hi+3) and [lo-2, hi+2), K3 and E on [lo-1, hi+1)
 * (indices periodic), reading A0, A1 and K1 of the whole pulse.  Every value is
 * the expression run_rk23_mex evaluates for that point.  Writes E and K4 on
 * [lo, hi); the new A1 is only classified.  Scratch: 6 (hi - lo + 6) values. */
static int rk23_span(const ofx_oracle_params* p, const cplx* A0, const cplx* A1, const cplx* K1, cplx* E, cplx* K4,
                     const cplx* cw0, int lo, int hi, cplx ez2, cplx ez3, cplx ez4, double hmod, double g,
                     double c_shock, cplx* scratch, double* pm) {
    const int n = p->N, m = hi - lo + 6;
    cplx *nl2 = scratch, *k2 = scratch + m, *nl3 = scratch + 2 * m, *k3 = scratch + 3 * m;
    cplx *ev = scratch + 4 * m, *nl4 = scratch + 5 * m;
#define OFX_WRAP(i) ((i) < 0 ? (i) + n : ((i) >= n ? (i) - n : (i)))
    for (int l = 0; l < m; ++l) {                       /* point lo - 3 + l */
        const int gi = OFX_WRAP(lo - 3 + l);
        nl2[l] = nl_point(A1[gi], cw0[gi], ez2);
    }
    for (int l = 1; l < m - 1; ++l) {
        const int gi = OFX_WRAP(lo - 3 + l);
        k2[l] = k_point(nl2[l + 1], nl2[l - 1], nl2[l], hmod, g, c_shock);
        nl3[l] = nl_point(cadd(A0[gi], cscale(k2[l], 0.75)), cw0[gi], ez3);
    }
    for (int l = 2; l < m - 2; ++l) {
        const int gi = OFX_WRAP(lo - 3 + l);
        k3[l] = k_point(nl3[l + 1], nl3[l - 1], nl3[l], hmod, g, c_shock);
        cplx e = cadd(A0[gi], cadd(cscale(k3[l], 4.0 / 9.0), cscale(k2[l], 1.0 / 3.0)));
        ev[l] = cadd(e, cscale(K1[gi], 2.0 / 9.0));
        nl4[l] = nl_point(ev[l], cw0[gi], ez4);
    }
#undef OFX_WRAP
    int flags = 0;
    for (int l = 3; l < m - 3; ++l) {
        const int i = lo - 3 + l;
        cplx k4 = k_point(nl4[l + 1], nl4[l - 1], nl4[l], hmod, g, c_shock);
        cplx a = cadd(A0[i], cadd(cscale(k4, 1.0 / 8.0), cscale(k3[l], 1.0 / 3.0)));
        a = cadd(a, cscale(k2[l], 1.0 / 4.0));
        a = cadd(a, cscale(K1[i], 7.0 / 24.0));
        E[i] = ev[l];
        K4[i] = k4;
        flags |= classify_point(p, ev[l], a, 200.0, pm);
    }
    return flags;
}

/* K1 = f(A0) at z = pos with the drive's G value g, and A1 = A0 + K1 / 2, on
 * [lo, hi) (NL recomputed one point out on each side). */
static void rk23_k1_span(const ofx_oracle_params* p, const cplx* A0, cplx* K1, cplx* A1, const cplx* cw0, int lo,
                         int hi, cplx ez, double hmod, double g, double c_shock, cplx* scratch) {
    const int n = p->N, m = hi - lo + 2;
    cplx* nl = scratch;
    for (int l = 0; l < m; ++l) {
        int gi = lo - 1 + l;
        gi = gi < 0 ? gi + n : (gi >= n ? gi - n : gi);
        nl[l] = nl_point(A0[gi], cw0[gi], ez);
    }
    for (int l = 1; l < m - 1; ++l) {
        const int i = lo - 1 + l;
        K1[i] = k_point(nl[l + 1], nl[l - 1], nl[l], hmod, g, c_shock);
        A1[i] = cadd(A0[i], cscale(K1[i], 0.5));
    }
}

/* run_rk23_mex for one pulse on a team of T threads (as run_heun_mex_team): the
 * stages on each thread's span, one barrier for the error test, K1 (FSAL: the
 * accepted attempt's K4) and A1 = A0 + K1/2 kept for the whole pulse between
 * attempts.  Bit-identical to run_rk23_mex.  Returns 0, or -1 (nothing done). */
static int run_rk23_mex_team(sched_ctx* c, work* w, int T) {
    const ofx_oracle_params* p = c->p;
    const int n = p->N, span = n / T;
    const double sel = p->sel, c_shock = 1.0 / (2.0 * p->dt * p->w0);
    int nchunks = (int)((double)p->S / sel);
    if (p->chunk_mode == OFX_CHUNKS_CEIL && (double)nchunks * sel < (double)p->S) nchunks += 1;
    cplx* scratch = (cplx*)malloc(sizeof(cplx) * 6 * (size_t)(span + 6) * (size_t)T);
    double* part_pm = (double*)malloc(sizeof(double) * 2 * (size_t)T);
    int* part_fl = (int*)malloc(sizeof(int) * 2 * (size_t)T);
    int ran = 0;
    if (scratch && part_pm && part_fl) {
#pragma omp parallel num_threads(T)
        if (omp_get_num_threads() == T) {
            const int tid = omp_get_thread_num(), lo = tid * span, hi = lo + span;
            cplx* mine = scratch + 6 * (size_t)(span + 6) * (size_t)tid;
            cplx *K1 = w->K1, *K4 = w->K4;
            double k = 0.0, stepprev = 4.0, stepmod = stepprev, stepend, pm = 0.0;
            double my_s[OFX_DISP_SLOTS];
            for (int j = 0; j < OFX_DISP_SLOTS; ++j) my_s[j] = -1.0;
            int attempt = 0;
            /* initial K1 at k = 0 (:432-438) */
            rk23_k1_span(p, w->A0, K1, w->A1, w->cw0, lo, hi, cexpi(-(p->bdiffw0 * k * p->h)),
                         stepmod * p->h, g_at(c, 0, 0), c_shock, mine);
#pragma omp barrier
            for (int chunk = 0; chunk < nchunks; ++chunk) {
                stepmod = stepprev;
                double cend = (double)(chunk + 1) * sel;
                for (; k < cend && (p->chunk_mode != OFX_CHUNKS_CEIL || k < (double)p->S); k = k + stepmod) {
                    const int kidx = (int)k;
                    const double hmod = stepmod * p->h, g = g_at(c, kidx, 0);
                    const cplx ez2 = cexpi(-(p->bdiffw0 * (k + 0.5 * stepmod) * p->h));
                    const cplx ez3 = cexpi(-(p->bdiffw0 * (k + 0.75 * stepmod) * p->h));
                    const cplx ez4 = cexpi(-(p->bdiffw0 * (k + stepmod) * p->h));
                    double my_pm = 0.0;
                    const int slot = attempt & 1;
                    part_fl[slot * T + tid] = rk23_span(p, w->A0, w->A1, K1, w->E, K4, w->cw0, lo, hi, ez2, ez3,
                                                        ez4, hmod, g, c_shock, mine, &my_pm);
                    part_pm[slot * T + tid] = my_pm;
#pragma omp barrier
                    int fl = 0;
                    pm = 0.0;
                    for (int t = 0; t < T; ++t) {
                        fl |= part_fl[slot * T + t];
                        if (part_pm[slot * T + t] > pm) pm = part_pm[slot * T + t];
                    }
                    fl = get_flags(c, attempt, fl);
                    if (tid == 0) {
                        if (fl & 4) c->stats->status |= OFX_ORACLE_STATUS_NAN;
                        c->stats->pct_max_last = pm;
                    }
                    if ((fl & 1) && stepmod > 1.0 && (k - stepmod) > 0.0) {
                        if (tid == 0) { record(c, attempt, kidx, (int)stepmod, fl, 0); c->stats->rejected++; }
                        k = k - stepmod;
                        stepmod = stepmod - 1.0;
                        stepprev = stepmod;
                        /* K1 recomputed at the new start, G index k (:484-487) */
                        rk23_k1_span(p, w->A0, K1, w->A1, w->cw0, lo, hi,
                                     cexpi(-(p->bdiffw0 * (k + stepmod) * p->h)), stepmod * p->h,
                                     g_at(c, (int)k, 0), c_shock, mine);
#pragma omp barrier
                    } else {
                        const int s = (int)stepmod;
                        if (tid == 0) {
                            record(c, attempt, kidx, s, fl, 1);
                            c->stats->accepted++;
                            c->stats->z_steps += (long long)stepmod;
                        }
                        dispersion_team(c, w, w->K3, my_s, s, chunk, nchunks, kidx, tid, T, 1);
                        cplx* tk = K1; K1 = K4; K4 = tk;     /* FSAL swap (:512-514) */
                        for (int i = lo; i < hi; ++i) w->A1[i] = cadd(w->A0[i], cscale(K1[i], 0.5));
#pragma omp barrier
                        if (k + stepmod >= cend && k < cend - 1.0) {
                            stepend = (cend - k) - 1.0;
                            stepprev = stepmod;
                            stepmod = stepend;
                        } else {
                            if (!(fl & 2) && !(fl & 1) && (k + stepmod + stepmod) < cend - 1.0)
                                stepmod = stepmod * 2.0;
                            stepprev = stepmod;
                        }
                    }
                    attempt++;
                }
            }
            if (tid == 0) {
                c->stats->attempts = attempt;
                c->stats->k_final = k;
                c->stats->stepmod_final = stepmod;
                c->stats->nchunks = nchunks;
                if (c->n_attempts) *c->n_attempts = attempt;
                ran = 1;
            }
        }
    }
    free(scratch); free(part_pm); free(part_fl);
    return ran ? 0 : -1;
}

/* Both stages of NEE_CPU.m's Heun step and its error measure for points [lo, hi)
 * (halo as heun_span): A1 = A0 + K1, E = (A0 + K1/2) + K2/2, the largest
 * 100 |E - A1| / (|E| + 1) into *pm, and *nan set when A0 holds a NaN on these
 * points (the schedule tests A0 before the step; the caller discards the step
 * then).  Writes E on [lo, hi).  Scratch: 4 (hi - lo + 4) values. */
static void nee_span(const ofx_oracle_params* p, const cplx* A0, cplx* E, const cplx* cw0, int lo, int hi,
                     cplx ez1, cplx ez2, double hmod, double g, double c_shock, cplx* scratch, double* pm, int* nan) {
    const int n = p->N, m = hi - lo + 4;
    cplx *nl1 = scratch, *k1 = scratch + m, *a1 = scratch + 2 * m, *nl2 = scratch + 3 * m;
#define OFX_WRAP(i) ((i) < 0 ? (i) + n : ((i) >= n ? (i) - n : (i)))
    for (int l = 0; l < m; ++l) {
        const int gi = OFX_WRAP(lo - 2 + l);
        nl1[l] = nl_point(A0[gi], cw0[gi], ez1);
    }
    for (int l = 1; l < m - 1; ++l) {
        const int gi = OFX_WRAP(lo - 2 + l);
        k1[l] = k_point(nl1[l + 1], nl1[l - 1], nl1[l], hmod, g, c_shock);
        a1[l] = cadd(A0[gi], k1[l]);
        nl2[l] = nl_point(a1[l], cw0[gi], ez2);
    }
#undef OFX_WRAP
    for (int l = 2; l < m - 2; ++l) {
        const int i = lo - 2 + l;
        if (isnan(A0[i].re) || isnan(A0[i].im)) *nan = 1;
        cplx k2 = k_point(nl2[l + 1], nl2[l - 1], nl2[l], hmod, g, c_shock);
        cplx e = cadd(cadd(A0[i], cscale(k1[l], 0.5)), cscale(k2, 0.5));
        E[i] = e;
        double v = 100.0 * cabs2(csub(e, a1[l])) / (cabs2(e) + 1.0);
        if (v > *pm) *pm = v;
    }
}

/* run_heun_nee for one pulse on a team of T threads (as run_heun_mex_team), with
 * the chunk-end snapshot ApFT(:, chunk) = fft(A0) taken by the team too.
 * Bit-identical to run_heun_nee.  Returns 0, or -1 (nothing done). */
static int run_heun_nee_team(sched_ctx* c, work* w, int T) {
    const ofx_oracle_params* p = c->p;
    const int n = p->N, span = n / T;
    const double c_shock = 1.0 / (2.0 * p->dt * p->w0);
    const int nchunks = (int)floor((double)p->S / p->sel);
    cplx* scratch = (cplx*)malloc(sizeof(cplx) * 4 * (size_t)(span + 4) * (size_t)T);
    double* part_pm = (double*)malloc(sizeof(double) * 2 * (size_t)T);
    int* part_fl = (int*)malloc(sizeof(int) * 2 * (size_t)T);
    int ran = 0;
    if (scratch && part_pm && part_fl) {
#pragma omp parallel num_threads(T)
        if (omp_get_num_threads() == T) {
            const int tid = omp_get_thread_num(), lo = tid * span, hi = lo + span;
            cplx* mine = scratch + 4 * (size_t)(span + 4) * (size_t)tid;
            double k = 1.0, stepmod = 4.0, pm = 0.0;
            double my_s[OFX_DISP_SLOTS];
            for (int j = 0; j < OFX_DISP_SLOTS; ++j) my_s[j] = -1.0;
            int attempt = 0, ev = 0;
            for (int chunk = 1; chunk <= nchunks; ++chunk) {
                while (k < (double)chunk * p->sel && k <= (double)p->S) {
                    const int kidx = (int)k - 1;                /* G33(k), 1-based */
                    const double hmod = p->h * stepmod, g = g_at(c, kidx, 0);
                    const cplx ez1 = cexpi(-(p->bdiffw0 * (k - 1.0) * p->h));
                    const cplx ez2 = cexpi(-(p->bdiffw0 * (k - 1.0 + stepmod) * p->h));
                    double my_pm = 0.0;
                    int my_nan = 0;
                    const int slot = ev & 1;
                    nee_span(p, w->A0, w->E, w->cw0, lo, hi, ez1, ez2, hmod, g, c_shock, mine, &my_pm, &my_nan);
                    part_fl[slot * T + tid] = my_nan;
                    part_pm[slot * T + tid] = my_pm;
                    ++ev;
#pragma omp barrier
                    int nan = 0;
                    pm = 0.0;
                    for (int t = 0; t < T; ++t) {
                        nan |= part_fl[slot * T + t];
                        if (part_pm[slot * T + t] > pm) pm = part_pm[slot * T + t];
                    }
                    if (nan) {
                        if (tid == 0) c->stats->status |= OFX_ORACLE_STATUS_NAN;
                        break;
                    }
                    int fl = (pm > p->maxErr ? 1 : 0) | (pm >= p->minErr ? 2 : 0);
                    fl = get_flags(c, attempt, fl);
                    if (tid == 0) c->stats->pct_max_last = pm;
                    if ((fl & 1) && stepmod > 1.0) {
                        if (tid == 0) { record(c, attempt, kidx + 1, (int)stepmod, fl, 0); c->stats->rejected++; }
                        stepmod = stepmod - 1.0;
                    } else {
                        if (tid == 0) {
                            record(c, attempt, kidx + 1, (int)stepmod, fl, 1);
                            c->stats->accepted++;
                            c->stats->z_steps += (long long)stepmod;
                        }
                        dispersion_team(c, w, w->K1, my_s, (int)stepmod, chunk - 1, nchunks, kidx, tid, T, 0);
#pragma omp barrier
                        if (!(fl & 2)) stepmod = stepmod + 1.0;     /* pcterr < minErr */
                        if (k < (double)p->S && (k + stepmod) > (double)p->S) stepmod = (double)p->S - k;
                        k = k + stepmod;
                    }
                    attempt++;
                }
                /* ApFT(:,chunk) = fft(Et) */
                if (c->Ap) {
                    long long off = ((long long)c->b0 * nchunks + (chunk - 1)) * (long long)n;
                    if (off >= 0 && off + n <= c->ap_len) {
                        cplx* ap = c->Ap + off;
                        for (int i = lo; i < hi; ++i) ap[i] = w->A0[w->plan.rev[i]];
                        fft_team_stages(&w->plan, ap, 0, tid, T);
                    } else if (tid == 0) c->stats->status |= OFX_ORACLE_STATUS_AP_RANGE;
                }
            }
            if (tid == 0) {
                c->stats->attempts = attempt;
                c->stats->k_final = k;
                c->stats->stepmod_final = stepmod;
                c->stats->nchunks = nchunks;
                if (c->n_attempts) *c->n_attempts = attempt;
                ran = 1;
            }
        }
    }
    free(scratch); free(part_pm); free(part_fl);
    return ran ? 0 : -1;
}
#endif

/* OPO_CUDA_ODE23.cu:375-557 */
static void run_rk23_mex(sched_ctx* c, work* w) {
    const ofx_oracle_params* p = c->p;
    const int n = p->N;
    const double sel = p->sel;
    const size_t tot = (size_t)n * c->nb;
    double k = 0.0, stepprev = 4.0, stepmod = stepprev, stepend;
    int nchunks = (int)((double)p->S / sel);
    if (p->chunk_mode == OFX_CHUNKS_CEIL && (double)nchunks * sel < (double)p->S) nchunks += 1;
    int attempt = 0;
    double pm;
    cplx *K1 = w->K1, *K4 = w->K4;
    stepmod = stepprev;
    /* initial K1 at k = 0 (:432-438) */
    stage(c, w, w->A0, K1, k, stepmod * p->h, 0);
#pragma omp parallel for schedule(static) if (par_ok(tot))
    for (size_t i = 0; i < tot; ++i) w->A1[i] = cadd(w->A0[i], cscale(K1[i], 0.5));
    for (int chunk = 0; chunk < nchunks; ++chunk) {
        stepmod = stepprev;
        double cend = (double)(chunk + 1) * sel;
        for (; k < cend && (p->chunk_mode != OFX_CHUNKS_CEIL || k < (double)p->S); k = k + stepmod) {
            int kidx = (int)k;
            double hmod = stepmod * p->h;
            stage(c, w, w->A1, w->K2, k + 0.5 * stepmod, hmod, kidx);
#pragma omp parallel for schedule(static) if (par_ok(tot))
            for (size_t i = 0; i < tot; ++i) w->A1[i] = cadd(w->A0[i], cscale(w->K2[i], 0.75));
            stage(c, w, w->A1, w->K3, k + 0.75 * stepmod, hmod, kidx);
#pragma omp parallel for schedule(static) if (par_ok(tot))
            for (size_t i = 0; i < tot; ++i) {
                cplx e = cadd(w->A0[i], cadd(cscale(w->K3[i], 4.0 / 9.0), cscale(w->K2[i], 1.0 / 3.0)));
                w->E[i] = cadd(e, cscale(K1[i], 2.0 / 9.0));
            }
            stage(c, w, w->E, K4, k + stepmod, hmod, kidx);
#pragma omp parallel for schedule(static) if (par_ok(tot))
            for (size_t i = 0; i < tot; ++i) {
                cplx a = cadd(w->A0[i], cadd(cscale(K4[i], 1.0 / 8.0), cscale(w->K3[i], 1.0 / 3.0)));
                a = cadd(a, cscale(w->K2[i], 1.0 / 4.0));
                w->A1[i] = cadd(a, cscale(K1[i], 7.0 / 24.0));
            }
            int fl = classify(c, w->E, w->A1, 200.0, &pm);
            fl = get_flags(c, attempt, fl);
            if (fl & 4) c->stats->status |= OFX_ORACLE_STATUS_NAN;
            c->stats->pct_max_last = pm;
            if ((fl & 1) && stepmod > 1.0 && (k - stepmod) > 0.0) {
                record(c, attempt, kidx, (int)stepmod, fl, 0);
                c->stats->rejected++;
                k = k - stepmod;
                stepmod = stepmod - 1.0;
                stepprev = stepmod;
                /* K1 recomputed at the new start, G index k (:484-487) */
                stage(c, w, w->A0, K1, k + stepmod, stepmod * p->h, (int)k);
#pragma omp parallel for schedule(static) if (par_ok(tot))
                for (size_t i = 0; i < tot; ++i) w->A1[i] = cadd(w->A0[i], cscale(K1[i], 0.5));
            } else {
                record(c, attempt, kidx, (int)stepmod, fl, 1);
                c->stats->accepted++;
                c->stats->z_steps += (long long)stepmod;
                dispersion_step(c, w, w->E, w->A0, (int)stepmod, chunk, nchunks, kidx);
                cplx* t = K1; K1 = K4; K4 = t;     /* FSAL swap (:512-514) */
#pragma omp parallel for schedule(static) if (par_ok(tot))
                for (size_t i = 0; i < tot; ++i) w->A1[i] = cadd(w->A0[i], cscale(K1[i], 0.5));
                if (k + stepmod >= cend && k < cend - 1.0) {
                    stepend = (cend - k) - 1.0;
                    stepprev = stepmod;
                    stepmod = stepend;
                } else {
                    if (!(fl & 2) && !(fl & 1) && (k + stepmod + stepmod) < cend - 1.0)
                        stepmod = stepmod * 2.0;
                    stepprev = stepmod;
                }
            }
            attempt++;
        }
    }
    c->stats->attempts = attempt;
    c->stats->k_final = k;
    c->stats->stepmod_final = stepmod;
    c->stats->nchunks = nchunks;
    if (c->n_attempts) *c->n_attempts = attempt;
}

/* NEE_CPU.m:1-122 (B = 1 per schedule; G33 indexed 1-based by k). */
static void run_heun_nee(sched_ctx* c, work* w) {
    const ofx_oracle_params* p = c->p;
    const int n = p->N;
    const size_t tot = (size_t)n * c->nb;
    double k = 1.0, stepmod = 4.0;
    double nchunks_d = (double)p->S / p->sel;
    int nchunks = (int)floor(nchunks_d);          /* for chunk = 1:nChunks */
    int attempt = 0;
    double pm;
    for (int chunk = 1; chunk <= nchunks; ++chunk) {
        while (k < (double)chunk * p->sel && k <= (double)p->S) {
            int nan = 0;
#pragma omp parallel for schedule(static) reduction(| : nan) if (par_ok(tot))
            for (size_t i = 0; i < tot; ++i) if (isnan(w->A0[i].re) || isnan(w->A0[i].im)) nan = 1;
            if (nan) { c->stats->status |= OFX_ORACLE_STATUS_NAN; break; }
            int kidx = (int)k - 1;                /* G33(k), 1-based */
            double hmod = p->h * stepmod;
            stage(c, w, w->A0, w->K1, k - 1.0, hmod, kidx);
#pragma omp parallel for schedule(static) if (par_ok(tot))
            for (size_t i = 0; i < tot; ++i) w->A1[i] = cadd(w->A0[i], w->K1[i]);
            stage(c, w, w->A1, w->K2, k - 1.0 + stepmod, hmod, kidx);
#pragma omp parallel for schedule(static) if (par_ok(tot))
            for (size_t i = 0; i < tot; ++i)
                w->E[i] = cadd(cadd(w->A0[i], cscale(w->K1[i], 0.5)), cscale(w->K2[i], 0.5));
            /* pcterr = 100 max(|Et-A1|/(|Et|+1)) over all points */
            pm = 0.0;
#pragma omp parallel for schedule(static) reduction(max : pm) if (par_ok(tot))
            for (size_t i = 0; i < tot; ++i) {
                double v = 100.0 * cabs2(csub(w->E[i], w->A1[i])) / (cabs2(w->E[i]) + 1.0);
                if (v > pm) pm = v;
            }
            int fl = (pm > p->maxErr ? 1 : 0) | (pm >= p->minErr ? 2 : 0);
            fl = get_flags(c, attempt, fl);
            c->stats->pct_max_last = pm;
            if ((fl & 1) && stepmod > 1.0) {
                record(c, attempt, kidx + 1, (int)stepmod, fl, 0);
                c->stats->rejected++;
                stepmod = stepmod - 1.0;
            } else {
                record(c, attempt, kidx + 1, (int)stepmod, fl, 1);
                c->stats->accepted++;
                c->stats->z_steps += (long long)stepmod;
                for (int b = 0; b < c->nb; ++b) {
                    cplx* e = w->E + (size_t)b * n;
#pragma omp parallel for schedule(static) if (par_ok((size_t)n))
                    for (int i = 0; i < n; ++i) e[i] = cscale(e[i], w->abc[i]);
                    fft_exec(&w->plan, e, 0);
                    const cplx* f = disp_factor(w, c->beta, c->alpha, stepmod);
#pragma omp parallel for schedule(static) if (par_ok((size_t)n))
                    for (int i = 0; i < n; ++i) e[i] = cmul(e[i], f[i]);
                    fft_exec(&w->plan, e, 1);
                    cplx* a0 = w->A0 + (size_t)b * n;
#pragma omp parallel for schedule(static) if (par_ok((size_t)n))
                    for (int i = 0; i < n; ++i) a0[i] = cscale(e[i], 1.0 / (double)n);
                }
                if (!(fl & 2)) stepmod = stepmod + 1.0;     /* pcterr < minErr */
                if (k < (double)p->S && (k + stepmod) > (double)p->S) stepmod = (double)p->S - k;
                k = k + stepmod;
            }
            attempt++;
        }
        /* ApFT(:,chunk) = fft(Et) */
        if (c->Ap) {
            for (int b = 0; b < c->nb; ++b) {
                long long off = ((long long)(c->b0 + b) * nchunks + (chunk - 1)) * (long long)n;
                if (off >= 0 && off + n <= c->ap_len) {
                    memcpy(c->Ap + off, w->A0 + (size_t)b * n, sizeof(cplx) * (size_t)n);
                    fft_exec(&w->plan, c->Ap + off, 0);
                } else c->stats->status |= OFX_ORACLE_STATUS_AP_RANGE;
            }
        }
    }
    c->stats->attempts = attempt;
    c->stats->k_final = k;
    c->stats->stepmod_final = stepmod;
    c->stats->nchunks = nchunks;
    if (c->n_attempts) *c->n_attempts = attempt;
}

static int run_schedule(sched_ctx* c) {
    const ofx_oracle_params* p = c->p;
    work w;
    int time_mode = p->method == OFX_ORACLE_HEUN_NEE ? OFX_TIME_NEE : p->time_mode;
    if (work_init(&w, p->N, c->nb, time_mode, p->method == OFX_ORACLE_HEUN_NEE, p->abc_mode, p->w0, p->dt)) {
        work_free(&w);
        return OFX_ORACLE_ENOMEM;
    }
    memcpy(w.A0, c->E_in + (size_t)c->b0 * p->N, sizeof(cplx) * (size_t)p->N * c->nb);
    memset(c->stats, 0, sizeof(*c->stats));
    if (p->method == OFX_ORACLE_HEUN_MEX) {
#ifdef _OPENMP
        int T = team_size(p->N, c->nb);
        if (T < 2 || run_heun_mex_team(c, &w, T) != 0) run_heun_mex(c, &w);
#else
        run_heun_mex(c, &w);
#endif
    } else if (p->method == OFX_ORACLE_RK23_MEX) {
#ifdef _OPENMP
        int T = team_size(p->N, c->nb);
        if (T < 2 || run_rk23_mex_team(c, &w, T) != 0) run_rk23_mex(c, &w);
#else
        run_rk23_mex(c, &w);
#endif
    }
    else {
#ifdef _OPENMP
        int T = team_size(p->N, c->nb);
        if (T < 2 || run_heun_nee_team(c, &w, T) != 0) run_heun_nee(c, &w);
#else
        run_heun_nee(c, &w);
#endif
    }
    memcpy(c->A_out + (size_t)c->b0 * p->N, w.A0, sizeof(cplx) * (size_t)p->N * c->nb);
    work_free(&w);
    return 0;
}

int ofx_oracle_run(const ofx_oracle_params* p,
                   const double* E_in, const double* alpha, const double* G, const double* beta,
                   double* A_out, double* Ap, long long ap_len_complex, double* stepmods,
                   int* trace, int trace_cap, int* n_attempts,
                   const int* forced_flags, int n_forced,
                   ofx_oracle_stats* stats, int nthreads) {
    if (!p || !E_in || !alpha || !G || !beta || !A_out || !stats) return OFX_ORACLE_EINVAL;
    if (p->N < 4 || (p->N & (p->N - 1)) || p->B < 1 || p->S < 1 || !(p->sel > 0)) return OFX_ORACLE_EINVAL;
    int nsched = p->shared_schedule ? 1 : p->B;
    int nb = p->shared_schedule ? p->B : 1;
    int rc_all = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    t_inner = (nthreads > 1 && nsched == 1);
#pragma omp parallel for schedule(dynamic, 1) reduction(| : rc_all) if (nsched > 1)
#endif
    for (int s = 0; s < nsched; ++s) {
        sched_ctx c;
        memset(&c, 0, sizeof(c));
        c.p = p; c.b0 = s * nb; c.nb = nb;
        c.E_in = (const cplx*)E_in; c.alpha = alpha; c.G = G; c.beta = beta;
        c.A_out = (cplx*)A_out;
        c.Ap = (cplx*)Ap; c.ap_len = ap_len_complex;
        c.stepmods = stepmods ? stepmods + (p->shared_schedule ? 0 : (size_t)s * p->S) : NULL;
        c.trace = trace ? trace + (size_t)s * 3 * (size_t)trace_cap : NULL;
        c.trace_cap = trace_cap;
        c.n_attempts = n_attempts ? n_attempts + s : NULL;
        c.forced = forced_flags ? forced_flags + (p->shared_schedule ? 0 : (size_t)s * n_forced) : NULL;
        c.n_forced = n_forced;
        c.stats = stats + s;
        rc_all |= run_schedule(&c);
    }
    return rc_all;
}

int ofx_oracle_version(void) { return 1; }
