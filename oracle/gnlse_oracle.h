/*
 * gnlse_oracle.h -- TEST INFRASTRUCTURE ONLY.  FP64 C restatement of the chi(3)
 * fibre GNLSE solver (toolbox/lib/internal/main/gnlsefib.m), the same scheme as
 * oracle/gnlse_oracle.py, for independent pulses in parallel (OpenMP).
 */
#ifndef OFX_GNLSE_ORACLE_H
#define OFX_GNLSE_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int n;            /* grid points, a power of two */
    int n_saves;      /* >= 2: z = linspace(0, length, n_saves) */
    double gamma;     /* gamma / w0 with a shock frequency, else gamma (gnlsefib.m:29-35) */
    double fr;        /* Raman fraction (used when RW is given) */
    double dT;        /* time step */
    double alpha;     /* field loss coefficient: L = i B - alpha / 2 (gnlsefib.m:27) */
    double length;    /* fibre length */
    double rtol, atol;
} ofx_gnlse_params;

/* A: n_pulses x n complex input fields (natural time order, interleaved re/im).
 * B, W: n doubles, FFT order (dispersion sum_m beta_m V^m / m!, and V + w0 or 1).
 * RW: n complex, FFT order (n ifft(fftshift(hR))), or NULL without Raman.
 * AT_out, AW_out: n_pulses x n_saves x n complex (AW fftshifted and scaled by dT n,
 * gnlsefib.m:82-89).  trace (optional): per pulse trace_cap pairs (step in units of
 * length / 2^40, accepted).  forced (optional): per pulse n_forced such pairs
 * replayed in place of the step control.  attempts, accepted: per pulse.
 * Returns 0, or -1 for bad arguments / -2 when memory runs out / -3 when a forced
 * schedule ends before the fibre does / -4 when the error norm is not finite / -5
 * after 10^7 attempts. */
int ofx_gnlse_oracle_run(const ofx_gnlse_params* p, int n_pulses, const double* A, const double* B,
                         const double* W, const double* RW, double* AT_out, double* AW_out,
                         long long* trace, int trace_cap, const long long* forced, int n_forced,
                         int* attempts, int* accepted, int nthreads);

#ifdef __cplusplus
}
#endif

#endif
