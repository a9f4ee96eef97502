/*
 * oracle.h -- FP64 CPU restatement of OptiFax's crystal-pass solver.
 * TEST INFRASTRUCTURE ONLY (see oracle.c): never linked into the product.
 */
#ifndef OFX_ORACLE_H
#define OFX_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { OFX_ORACLE_HEUN_MEX = 0, OFX_ORACLE_RK23_MEX = 1, OFX_ORACLE_HEUN_NEE = 2 };
enum { OFX_TIME_SHIFTED = 0, OFX_TIME_UNSHIFTED = 1, OFX_TIME_NEE = 2 };
enum { OFX_ABC_SOFT = 0, OFX_ABC_NONE = 1, OFX_ABC_HARD = 2 };
enum { OFX_CHUNKS_CEIL = 0, OFX_CHUNKS_TRUNC = 1 };
enum { OFX_ORACLE_EINVAL = 1, OFX_ORACLE_ENOMEM = 2 };
enum { OFX_ORACLE_STATUS_NAN = 1, OFX_ORACLE_STATUS_AP_RANGE = 2 };

typedef struct {
    int method;          /* OFX_ORACLE_* */
    int time_mode;       /* OFX_TIME_* (ignored for NEE, which uses fftshift(t)) */
    int abc_mode;        /* OFX_ABC_* */
    int chunk_mode;      /* OFX_CHUNKS_* */
    int g_per_pulse;     /* 1: G is S x B (XTAL); 0: one S-array for all pulses */
    int stepmods_limit;  /* stepmods[k] recorded only for k < limit */
    int shared_schedule; /* 1: one step schedule for the batch (flags OR-ed); 0: per pulse */
    int N, B, S;
    double w0, bdiffw0, h, dt, maxErr, minErr, sel;
} ofx_oracle_params;

typedef struct {
    int attempts, accepted, rejected, nchunks;
    long long z_steps;        /* sum of stepmod over accepted steps */
    double k_final, stepmod_final, pct_max_last;
    int status;               /* OFX_ORACLE_STATUS_* bits */
    int pad;
} ofx_oracle_stats;

/* Complex arrays are interleaved (re, im) doubles.  E_in/A_out: N x B;
 * Ap: flat complex array of ap_len_complex values (reference layout
 * (b*Nchunks + chunk)*N + i); stepmods: S (shared schedule) or S x B.
 * trace: per schedule 3*trace_cap ints (k, stepmod, flags) where flags bit0 =
 * above maxErr, bit1 = above minErr, bit2 = NaN, bit3 = accepted.
 * forced_flags (optional): per schedule n_forced decisions replayed in place
 * of the computed ones (bits 0-1). stats: one per schedule.
 * nthreads: 0 = OpenMP's default team over the schedules, each schedule on one
 * thread; > 0 = that many threads, over the schedules when there are several,
 * else inside the one pass (point loops and FFT stages, N >= 4096).  Results
 * are bit-identical for every thread count. */
int ofx_oracle_run(const ofx_oracle_params* p,
                   const double* E_in, const double* alpha, const double* G, const double* beta,
                   double* A_out, double* Ap, long long ap_len_complex, double* stepmods,
                   int* trace, int trace_cap, int* n_attempts,
                   const int* forced_flags, int n_forced,
                   ofx_oracle_stats* stats, int nthreads);

int ofx_oracle_fft(const double* in, double* out, int n, int inverse);
int ofx_oracle_version(void);

#ifdef __cplusplus
}
#endif
#endif
