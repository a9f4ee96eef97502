/*
 * optifax.h -- C ABI of the GB300 (sm_103a) chi(2) crystal-pass propagator.
 *
 * Drop-in for OptiFax's crystal-pass solver boundary.  In the reference the
 * boundary is the MATLAB function handle OpticalSim.Solver
 * (toolbox/lib/classes/OpticalSim.m:20,98-100,237-252) resolving to the MEX
 * gateway mexFunction (toolbox/lib/MEXlib/src/OPO_mex_BATCH.cpp:19-141) which
 * calls the host driver OPO_TEST_CUDA
 * (toolbox/lib/MEXlib/src/OPO_CUDA_BATCH_XTAL.cu:373-525,
 *  prototype toolbox/lib/MEXlib/src/OPO_BATCH_HEADER.hpp:8-28).
 *
 * All array arguments are DEVICE pointers owned by the caller; complex arrays
 * are interleaved (re, im) single precision, i.e. MATLAB complex single
 * gpuArrays / CUDA float2.  Every call is ordered on the given CUDA stream
 * (NULL = legacy default stream) and returns before the work completes.
 * Functions return OPTIFAX_OK or an optifax_status code; they never abort.
 * A handle may be used by one host thread at a time.  Its calls may go to
 * different streams: the handle's device scratch (descriptors, exchange
 * buffers, stage rows) is shared by its calls, so a call on another stream than
 * the previous call's waits on the GPU until the previous call's work is done.
 * Independent concurrent work takes one handle per stream.  Calls on a handle
 * are not for CUDA stream capture (descriptors are staged from host memory and
 * the first use of a grid size builds its tables synchronously).
 */
#ifndef OPTIFAX_H
#define OPTIFAX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct optifax_context* optifax_handle;

typedef enum {
    OPTIFAX_OK = 0,
    OPTIFAX_ERR_INVALID_ARGUMENT = 1,
    OPTIFAX_ERR_UNSUPPORTED = 2,
    OPTIFAX_ERR_CUDA = 3,
    OPTIFAX_ERR_NO_MEMORY = 4,
    OPTIFAX_ERR_NULL_HANDLE = 5
} optifax_status;

/* Integration scheme of the nonlinear sub-step. */
typedef enum {
    OPTIFAX_HEUN = 0,   /* OPO_CUDA_BATCH_XTAL.cu:432-506 (Euler + Heun, +1 growth) */
    OPTIFAX_RK23 = 1    /* ode23/OPO_CUDA_ODE23.cu:428-538 (Bogacki-Shampine, x2 growth) */
} optifax_method;

/* Reference source variant whose conventions are reproduced. */
typedef enum {
    OPTIFAX_VARIANT_BATCH_XTAL = 0, /* shifted time, sech^2 absorber, ceil chunk count + k<Nsteps guard, G is S x B */
    OPTIFAX_VARIANT_BATCH_OP = 1,   /* as XTAL with one G shared by all pulses (OPO_CUDA_BATCH_OP.cu:221) */
    OPTIFAX_VARIANT_NO_BC = 2,      /* unshifted time, no absorber, truncated chunk count (OPO_CUDA_NO_BC.cu) */
    OPTIFAX_VARIANT_HARD_BC = 3,    /* unshifted time, hard absorber (OPO_CUDA_HARD_BC.cu:118-129) */
    OPTIFAX_VARIANT_ODE23 = 4,      /* unshifted time, sech^2 absorber, truncated chunks, shared G (OPO_CUDA_ODE23.cu) */
    OPTIFAX_VARIANT_NEE = 5         /* NEE_CPU.m:1-122 (Heun): fftshift(t), t-based absorber, 1-based G, reject keeps k,
                                       grow below minErr, clamp only at the crystal end, snapshot fft(A) per chunk;
                                       grids up to 2^14 points */
} optifax_variant;

/* Per-pulse status bits returned in optifax_pulse_stats.status. */
#define OPTIFAX_PULSE_NAN           0x1  /* a non-finite field value was produced */
#define OPTIFAX_PULSE_ATTEMPT_LIMIT 0x2  /* the step-attempt safety limit was reached */

typedef struct {
    int32_t attempts;       /* step attempts (accepted + rejected) */
    int32_t accepted;
    int32_t rejected;
    int32_t status;         /* OPTIFAX_PULSE_* bits */
    int64_t z_steps;        /* sum of stepmod over accepted steps (distance / h) */
    float k_final;          /* final value of the reference's step counter k */
    float stepmod_final;
    int32_t n_chunks;
    int32_t reserved[3];
} optifax_pulse_stats;   /* reserved[0]: round trips completed */

/* Per round trip of a synchronously pumped OPO. */
typedef struct {
    int32_t attempts;
    int32_t accepted;
    int32_t rejected;
    int32_t status;         /* OPTIFAX_PULSE_* bits of this trip */
    double tally[4];        /* sum_k tally_w[i][k] |X_k|^2 of the crystal-output spectrum, FP64 */
} optifax_trip_record;

/* One crystal pass of one pulse (all pointers are device pointers). */
typedef struct {
    int32_t n_points;        /* N: power of two, 512 .. 65536 */
    int32_t n_steps;         /* S = floor(L / h) */
    const void* E_in;        /* N complex: fftshifted temporal field (t = 0 at index 0) */
    void* A_out;             /* N complex output field (may alias E_in) */
    const float* alpha;      /* N: per-step power transmission, FFT order (TStepShift) */
    const float* beta;       /* N: relative phase per step h, FFT order (hBshift) */
    const float* G;          /* S: QPM-signed coupling G33 per z-sample */
    void* Ap;                /* optional: spectral snapshots, N x n_chunks complex, reference layout */
    float* stepmods;         /* optional: S floats, stepmods[k] = stepmod of the accepted step at k */
    int32_t* trace;          /* optional: 3 ints per attempt (k, stepmod, flags) */
    const int32_t* forced;   /* optional: per-attempt decisions to replay (bit0 >maxErr, bit1 >minErr) */
    int32_t trace_cap;
    int32_t n_forced;
    float w0;                /* reference angular frequency (single, as the MEX casts it) */
    float h;                 /* step size [m] (single) */
    double bdiffw0;          /* beta0(w0) - beta1(w0) w0 */
    double dt;               /* time step [s] */
    float max_err;           /* percent */
    float min_err;           /* percent */
    float sel;               /* steps per progress chunk */
    int32_t stepmods_limit;  /* stepmods recorded for k < limit (0: the variant's own rule) */
    int32_t cta_points;      /* points per CTA for this pulse (0: the call's choice) */
} optifax_pulse;

/*
 * A synchronously pumped OPO cavity (reference: OpticalSim.run,
 * toolbox/lib/classes/OpticalSim.m:207-301; per-trip optics
 * OpticalPulse.m:137-197,256-261,518-527; Cavity.m:50-87).  Every round trip
 * runs one crystal pass of `pass`; the crystal-output spectrum X (natural FFT
 * order of the fftshifted field) then becomes the next crystal input
 *     Y_k = X_k feedback[k] + pump[k],
 * where feedback folds the refraction out of and back into the crystal, the
 * intracavity optics, the output coupler's intracavity share and the delay,
 * and pump is the in-crystal pump spectrum.  pass.E_in is the first trip's
 * crystal input; pass.A_out receives the crystal input of the trip after the
 * last one (so a run resumes by passing it back as E_in).  All pointers are
 * device pointers.
 */
typedef struct {
    optifax_pulse pass;
    const void* feedback;        /* N complex, natural FFT order */
    const void* pump;            /* N complex, natural FFT order */
    const float* tally_w;        /* n_tally x N energy weights (may be NULL if n_tally == 0) */
    optifax_trip_record* trips;  /* n_trips records (optional) */
    int32_t n_trips;
    int32_t n_tally;             /* 0..4 */
    int32_t steady_trips;        /* stop after this many consecutive flat trips (0: never) */
    int32_t steady_tally;        /* tally index tested for flatness */
    float steady_tol;            /* |T_n - T_{n-1}| <= tol |T_n| counts as flat */
    int32_t reserved;
    void* history;               /* optional: n_trips x N complex, crystal-output spectrum X of each trip */
    const float* esd_w;          /* optional: n_esd x N weights (OpticalSim.averageSimPulses, OpticalSim.m:303-315) */
    float* esd;                  /* n_esd x N accumulators: esd[i][k] += esd_w[i][k] |X_k|^2 every trip */
    int32_t n_esd;               /* 0..4 */
    int32_t reserved2;
    float* stepmods_trips;       /* optional: n_trips x n_steps, each trip's stepmods record
                                    (StepSizeModifiers, OpticalSim.m:172,237-252) */
} optifax_opo;

/* Create / destroy a context on a CUDA device.  The context owns the twiddle
 * tables and the pulse-descriptor staging buffers (device workspace). */
int optifax_create(optifax_handle* out, int device);
int optifax_destroy(optifax_handle h);
const char* optifax_status_string(int status);
/* Human-readable detail of the last failure on this handle. */
const char* optifax_last_error(optifax_handle h);

/*
 * The MEX-shaped entry: the 14 solver inputs of OPO_mex_BATCH.cpp:42-56 and
 * its 3 outputs (:120-122), replacing mexFunction + OPO_TEST_CUDA.
 *   E        prhs[0]  N x B complex, fftshifted time
 *   alpha_w  prhs[1]  N   (TStepShift)
 *   G        prhs[2]  S (BATCH_OP/ODE23 variants) or S x B (BATCH_XTAL)
 *   w0       prhs[3], bdiffw0 prhs[4], h prhs[5], n_steps prhs[6], dt prhs[7]
 *   beta_op  prhs[8]  N   (hBshift; N = numel)
 *   max_pct_err prhs[9], min_pct_err prhs[10], sel prhs[11]
 *   Ap_in    prhs[12] N x ap_chunks x B complex
 *   stepmods_in prhs[13] S
 * Outputs: A_out (plhs[0], N x B), Ap_out (plhs[1]), stepmods_out (plhs[2]);
 * the outputs may alias the inputs.  As in the reference, all pulses of the
 * batch share one adaptive step schedule (error flags are OR-ed over the
 * batch): for n_pulses > 1 the batch runs as one cooperative launch.
 */
int optifax_opo_mex_batch(optifax_handle h,
                          const void* E, const float* alpha_w, const float* G,
                          float w0, double bdiffw0, float step_h, int32_t n_steps, double dt,
                          const float* beta_op, float max_pct_err, float min_pct_err, float sel,
                          const void* Ap_in, const float* stepmods_in,
                          int32_t n_points, int32_t n_pulses, int32_t ap_chunks, int32_t variant,
                          void* A_out, void* Ap_out, float* stepmods_out, void* stream);

/*
 * Batched crystal passes with per-pulse grids and step schedules: each pulse
 * carries its own N, S, crystal and tolerances, and adapts its own step
 * (unlike the reference, whose batch shares one schedule).  `pulses` is a
 * HOST array of n_pulses descriptors holding device pointers.  stats
 * (optional) is a DEVICE array of n_pulses entries.  cta_points selects the
 * points held per CTA (512..4096, 0 = automatic); a pulse of N points runs on
 * a cluster of N / cta_points CTAs.
 */
int optifax_propagate(optifax_handle h, const optifax_pulse* pulses, int32_t n_pulses,
                      int32_t method, int32_t variant, int32_t cta_points,
                      optifax_pulse_stats* stats, void* stream);

/*
 * The same batch as optifax_propagate recorded once into a CUDA graph and then
 * replayed: the graph holds one persistent grid per (cta_points, cluster) group,
 * forked and joined as optifax_propagate launches them, with its own descriptors
 * and exchange scratch (no host staging on replay).  The pulses' device pointers
 * (inputs, outputs, stats) are fixed at capture: every replay reads the inputs'
 * current contents and rewrites the outputs.  No counterpart in the reference,
 * whose batch shares one cuFFT plan and one step.  The graph uses the handle's
 * twiddle tables: destroy it before the handle.  Replays of one graph are ordered
 * after each other; the caller orders them with other work on its stream.
 * optifax_graph_kernels returns the number of kernels one replay launches.
 */
typedef struct optifax_graph_s* optifax_graph;
int optifax_propagate_graph(optifax_handle h, const optifax_pulse* pulses, int32_t n_pulses,
                            int32_t method, int32_t variant, int32_t cta_points,
                            optifax_pulse_stats* stats, optifax_graph* out);
int optifax_graph_launch(optifax_graph g, void* stream);
int optifax_graph_kernels(optifax_graph g);
int optifax_graph_destroy(optifax_graph g);

/*
 * Run n_cavities independent OPO cavities (e.g. delay scans, replicas) for
 * their round trips in one launch, Heun schedule with the given variant's
 * conventions.  stats (optional, device): per-cavity totals, reserved[0] =
 * trips completed (fewer than n_trips when the steady-state test stopped it).
 */
int optifax_opo_run(optifax_handle h, const optifax_opo* cavities, int32_t n_cavities,
                    int32_t variant, int32_t cta_points, optifax_pulse_stats* stats, void* stream);

/*
 * One crystal pass (Heun schedule) that allocates no device memory, for callers
 * that cannot allocate GPU memory while they run -- a solver inside a MATLAB MEX
 * function whose device memory belongs to MATLAB's gpuArray manager, an
 * application that hands all device memory to its own caching allocator, or a
 * latency-critical loop that cannot let cudaMalloc/cudaFree synchronise the
 * device.  This entry point has no counterpart in the reference.
 *
 * The caller passes the pulse's inputs and outputs (device pointers, as for
 * optifax_propagate, validated by the same rules; stats optional) and no
 * handle.  The descriptor, twiddle tables and cluster exchange buffer live in
 * one static device array of 350,720 bytes (about 0.35 MB) that each GPU
 * loading the library reserves until the process exits.  n_points must be 8192
 * or 16384 (clusters of 2 or 4 CTAs of 4096 points); other sizes, including
 * anything above 16384, return OPTIFAX_ERR_UNSUPPORTED.  Variants BATCH_XTAL,
 * BATCH_OP, NO_BC and HARD_BC are accepted.
 *
 * Set-up: the first call in a CUDA context -- the first on a device, and again
 * the first after that device's context has been replaced (cudaDeviceReset, or
 * another context made current) -- finds the array's device address and builds
 * the twiddle tables in it.  That call should come before any stream capture;
 * made while its stream is capturing it returns OPTIFAX_ERR_UNSUPPORTED.  Every
 * call reuses the same array and leaves its contents behind: calls that overlap
 * on the GPU race and must be serialised by the caller.
 */
int optifax_propagate_noalloc(const optifax_pulse* pulse, int32_t variant,
                              optifax_pulse_stats* stats, void* stream);

/*
 * The plain full-FP64 crystal pass (Heun schedule of OPO_CUDA_BATCH_XTAL.cu:373-525
 * and its BATCH_OP / NO_BC / HARD_BC variants, computed in double precision
 * throughout, as the reference's FP64 MATLAB solver NEE_CPU.m computes it on the
 * CPU).  It is the FP64 comparator of the FP32 propagator: the same persistent
 * design (one launch per pass, the field on chip in a thread-block cluster of up
 * to 16 CTAs) with every value in double.  The reference has no FP64 GPU entry
 * point; this one takes the MEX argument list with double arrays.
 *
 * E_in, A_out: DEVICE arrays of n_pulses x n_points complex doubles (interleaved);
 * alpha, beta: DEVICE, n_points doubles; G: DEVICE, n_steps doubles, or
 * n_pulses x n_steps when g_per_pulse.  All pulses share one step schedule (the
 * reference's batch rule; n_pulses x clusters must fit one wave of SMs).
 * trace_host (optional, HOST, 3 x trace_cap int32): per attempt {k, stepmod,
 * flags | 8 if accepted}; stats_host (optional, HOST).  Variant ODE23 is not
 * offered; NEE follows NEE_CPU.m for grids up to 2^14 points (the snapshot
 * outputs are not produced by this entry).  Calls on one device are serialised
 * internally, and each call waits for its stream before returning.
 */
int optifax_propagate_fp64(int32_t n_points, int32_t n_pulses, int32_t n_steps,
                           const double* E_in, double* A_out, const double* alpha,
                           const double* beta, const double* G, int32_t g_per_pulse,
                           double w0, double bdiffw0, double step_h, double dt,
                           double max_err, double min_err, double sel, int32_t variant,
                           int32_t* trace_host, int32_t trace_cap,
                           optifax_pulse_stats* stats_host, void* stream);

/*
 * The float-float crystal pass: the same schedule, arguments and results as
 * optifax_propagate_fp64, with the field, the stage sums, the nonlinear drive
 * and every transform held as unevaluated sums of two FP32 values (~48-bit
 * significands) and the step decisions taken at FP64 precision.  For passes
 * whose parametric gain amplifies the FP32 field's rounding beyond the
 * tolerance (a long chirped crystal), at a fraction of the FP64 kernel's time:
 * GB300 runs FP32 about 64 times faster than FP64.  No counterpart in the
 * reference.  Variants BATCH_XTAL, BATCH_OP, NO_BC, HARD_BC.
 */
int optifax_propagate_f32x2(int32_t n_points, int32_t n_pulses, int32_t n_steps,
                            const double* E_in, double* A_out, const double* alpha,
                            const double* beta, const double* G, int32_t g_per_pulse,
                            double w0, double bdiffw0, double step_h, double dt,
                            double max_err, double min_err, double sel, int32_t variant,
                            int32_t* trace_host, int32_t trace_cap,
                            optifax_pulse_stats* stats_host, void* stream);

/*
 * Surrogate-network building block: C[M, N] (+)= A[M, K] . B[N, K]^T on the tensor
 * cores (tcgen05, TMA), A and B row-major BF16 DEVICE arrays with leading
 * dimensions lda, ldb (elements, multiples of 8, base addresses 16-byte aligned),
 * C row-major FP32 with leading dimension ldc.  a_rows >= max(M, 128) and
 * b_rows >= max(N, 64) rows must be readable (the 128 x 64 and 64 x 64 tiles
 * never read past them; rows past M or N may hold anything).  splits > 1 divides
 * K over CTAs and adds the partial sums atomically; accumulate = 1 adds into C.
 * No reference counterpart (the reference has no learned component).
 */
int optifax_gemm_bf16(const void* A, int64_t lda, int64_t a_rows, const void* B, int64_t ldb,
                      int64_t b_rows, float* C, int64_t ldc, int32_t M, int32_t N, int32_t K,
                      int32_t splits, int32_t accumulate, void* stream);

/* Reads (and with clear != 0 resets) the tensor-core kernels' error flag: nonzero
 * when a kernel gave up waiting for a copy or an MMA and skipped its output. */
int optifax_tc_error(int32_t* out, int32_t clear);

/*
 * Fourier-neural-operator surrogate of one crystal pass (no reference
 * counterpart).  Fixed architecture: 6 input channels (4 field channels, a
 * constant conditioning channel and the bin coordinate) over n_bins frequency
 * bins, width 64, four spectral layers keeping 32 modes, GELU between layers, 4 output channels with a
 * residual connection to the first 4 inputs.  Parameters are one FP32 vector of
 * optifax_fno_param_count() values (layout in ofx_fno.cu); the kernels use BF16
 * copies of the weights and BF16 activations with FP32 accumulation.
 * x: DEVICE float [batch][6][n_bins]; y, target: DEVICE float [batch][4][n_bins].
 * n_bins: a multiple of 64, >= 128.  One handle is used by one stream at a time.
 */
typedef struct optifax_fno_s* optifax_fno;
int64_t optifax_fno_param_count(void);
int optifax_fno_create(optifax_fno* out, int32_t n_bins, int32_t max_batch, int32_t device);
int optifax_fno_destroy(optifax_fno f);
/* copy params (DEVICE, FP32) into the network; resets the Adam moments */
int optifax_fno_set_params(optifax_fno f, const float* params, void* stream);
int optifax_fno_get_params(optifax_fno f, float* params, void* stream);
int optifax_fno_forward(optifax_fno f, const float* x, float* y, int32_t batch, void* stream);
/* forward + backward of loss = sum_b w_b sum ((y - target)^2) / numel(y) with per-sample
 * weights w (DEVICE, batch floats; NULL: all 1); loss (DEVICE scalar) and grads
 * (DEVICE, param_count floats) are optional copies of the results */
int optifax_fno_backward(optifax_fno f, const float* x, const float* target, const float* sample_w,
                         int32_t batch, float* loss, float* grads, void* stream);
/* replace the gradients of the last backward (DEVICE, param_count floats), e.g. by their
 * mean over data-parallel ranks, before optifax_fno_adam */
int optifax_fno_set_grads(optifax_fno f, const float* grads, void* stream);
/* AdamW step (decoupled weight decay) with the gradients of the last backward; step >= 1 */
int optifax_fno_adam(optifax_fno f, float lr, float beta1, float beta2, float eps,
                     float weight_decay, int32_t step, void* stream);

/*
 * OPO fast-forward helpers (no reference counterpart).  A crop is n_bins
 * consecutive bins of an n_points spectrum (natural FFT order of the fftshifted
 * field, DEVICE complex64) starting at bin k0 and wrapping at n_points; crop bins
 * j < split are the signal band.
 * optifax_ff_encode: n_spectra spectra (stride elements apart) -> network input
 * x[n][n_channels][n_bins]: channels 0/1 the pump band / pump_scale, 2/3 the signal
 * band / sigma, 4 and 5 (if n_channels = 6) log10(sigma / pump_scale) and the bin
 * coordinate j / n_bins.  sigma is the RMS of the signal-band bins (written to
 * sigma_out) unless sigma_in supplies it.
 * optifax_ff_step: X = the decoded network output y[4][n_bins] (with sigma[0]), or
 * X_in when y is NULL, times lin[k] (optional per-bin factor: the crystal's linear
 * propagation, when the network predicts the output in the interaction picture); writes
 * X_out (optional), Y_next = X feedback + pump and (optional) *energy = sum tally_w |X|^2
 * in FP64.  All pointers are device pointers.
 */
int optifax_ff_encode(const void* spectra, int64_t stride, int32_t n_spectra, int32_t n_points,
                      int32_t k0, int32_t n_bins, int32_t split, float pump_scale,
                      const float* sigma_in, float* x, int32_t n_channels, float* sigma_out,
                      void* stream);
int optifax_ff_step(const float* y, const float* sigma, const void* X_in, const void* feedback,
                    const void* pump, const void* lin, const float* tally_w, int32_t n_points,
                    int32_t k0, int32_t n_bins, int32_t split, float pump_scale, void* X_out,
                    void* Y_next, double* energy, void* stream);

/*
 * Envelope representation for the fast-forward (no reference counterpart).  band =
 * {kc_pump, lo_pump, hi_pump, kc_signal, lo_signal, hi_signal} (HOST int32[6]): each
 * band holds the bins whose signed offset o from its carrier bin kc lies in
 * [lo, hi), |o| < n_bins / 2; its envelope is e_j = sum_o b_o exp(2 pi i o j / n_bins),
 * j < n_bins (n_bins a power of two <= 4096).  optifax_ff_encode_env writes channels
 * 0/1 = pump envelope / pump_scale, 2/3 = signal envelope / sigma (sigma = RMS of the
 * signal envelope unless sigma_in is given), 4/5 (n_channels = 6) = log10(sigma /
 * pump_scale) and j / n_bins.  optifax_ff_decode_env inverts channels 0-3 of one
 * network output into the two bands of X_out (n_points complex, zero elsewhere).
 */
int optifax_ff_encode_env(const void* spectra, int64_t stride, int32_t n_spectra, int32_t n_points,
                          int32_t n_bins, const int32_t* band, float pump_scale,
                          const float* sigma_in, float* x, int32_t n_channels, float* sigma_out,
                          void* stream);
int optifax_ff_decode_env(const float* y, const float* sigma, int32_t n_points, int32_t n_bins,
                          const int32_t* band, float pump_scale, void* X_out, void* stream);

/*
 * Solver inputs computed on the device (OpticalSim.m:213-226 precompute) for many
 * pulses at once: per pulse the dispersion phase per step (phi_calc.m:14-45, MgO:LN
 * Sellmeier of Gayer et al., group delay at the reference removed), the per-step
 * transmission, the QPM drive from the given domain walls (QPMcrystal.m:20-51) and
 * the in-crystal input field (sech^2 pump, sechPulse.m / Laser.m:66-77, plus one
 * photon per mode with a counter-based phase keyed by `seed`, refracted into the
 * crystal).  Scalars (dt exactly as the host grid computes it, t_rms of the pump,
 * g_scale = chi2 w0 / (n0 4 c)) come from the host.  Outputs alpha, beta (N floats),
 * G (S floats) and E (N complex64) are DEVICE arrays in the solver's layout; walls
 * (DEVICE, ascending, < length) give the domain boundaries.  work: DEVICE scratch of
 * optifax_setup_work_bytes(max n_points) bytes, reused pulse by pulse.
 */
typedef struct {
    int32_t n_points, n_steps;
    double window, dt;                 /* temporal range and sample spacing [s] */
    double lambda_ref;                 /* grid reference wavelength [m] */
    double length, step_size, celsius; /* crystal length and solver step [m], temperature */
    double g_scale;
    const double* walls;
    int32_t n_walls;
    int32_t seed;
    double pump_lambda, pump_t_rms, pump_energy, waist, n_medium;
    double lambda_lo_nm, lambda_hi_nm; /* transmission window (inside 200-20000 nm) */
    float* alpha;
    float* beta;
    float* G;
    void* E;
} optifax_setup;
int64_t optifax_setup_work_bytes(int32_t max_points);
int optifax_setup_pulses(const optifax_setup* s, int32_t n, void* work, int64_t work_bytes,
                         void* stream);

/*
 * chi(3) fibre GNLSE (replaces toolbox/lib/internal/main/gnlsefib.m:1-89; its caller
 * is gnlsefibsim.m:30).  The interaction-picture spectral field AW obeys
 * gnlsefib.m:54-66: dAW/dz = i gamma W ifft(AT ((1 - fR)|AT|^2 + RS)) e^{-Lz},
 * AT = fft(AW e^{Lz}), RS = dT fR fft(ifft(|AT|^2) RW), L = iB - alpha/2 (MATLAB
 * fft/ifft conventions), from AW(0) = ifft(A) over [0, length], saved at
 * linspace(0, length, n_saves).  Integrated by an adaptive Dormand-Prince 5(4) pair
 * (FSAL) with the tolerances gnlsefib.m passes to ode45 (rtol, atol; NormControl
 * error norm), steps landing on the save points, positions in units of
 * length / 2^40.  One CTA per pulse; n_points a power of two in 512..4096.
 * Per pulse (all DEVICE pointers; arrays in FFT order unless stated):
 *   A       input field, natural time order (n complex64, sqrt(W))
 *   B       dispersion sum_m beta_m V^m / m! (n doubles, rad/m)
 *   W       V + w0 with a shock term, else ones (n floats)
 *   RW      n ifft(fftshift(hR)) (n complex64), NULL without Raman (or fR = 0)
 *   gamma   gamma / w0 with a shock term, else gamma; fr, dT, alpha (field loss), length
 *   AT_out  n_saves x n complex64: time-domain field at each save (natural order)
 *   AW_out  n_saves x n complex64: fftshift(AW e^{Lz}) dT n at each save (gnlsefib.m:82-89)
 *   trace   optional: 2 int64 per attempt (step in length/2^40 units, accepted)
 *   stats   optional: attempts, accepted, status (OPTIFAX_PULSE_* bits)
 * All pulses of one call share n_points and n_saves.
 */
typedef struct {
    int32_t attempts, accepted, status, reserved;
} optifax_gnlse_stats;
typedef struct {
    int32_t n_points, n_saves;
    const void* A;
    const double* B;
    const float* W;
    const void* RW;
    double gamma, fr, dT, alpha, length, rtol, atol;
    void* AT_out;
    void* AW_out;
    int64_t* trace;
    int32_t trace_cap, max_attempts;
    optifax_gnlse_stats* stats;
} optifax_gnlse_pulse;
int optifax_gnlse(optifax_handle h, const optifax_gnlse_pulse* pulses, int32_t n_pulses, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* OPTIFAX_H */
