// ofx_fp64.cu -- the plain full-FP64 crystal-pass solver on the GPU.
//
// A straightforward double-precision implementation of the same schedule as
// the reference driver (OPO_CUDA_BATCH_XTAL.cu:373-525): one kernel per
// sub-operation over global memory, the step decision on the host after a
// flag read-back each attempt, and this library's own radix-4 FFT (no cuFFT).
// It is the FP64 comparator of the FP32 propagator (precision study: 2^16
// points, 20 mm chirped PPLN) and the "plain FP64 solver" the OPO speed-up is measured
// against.  GB300's FP64 rate is a small fraction of its FP32 rate; this
// solver is not tuned beyond batching all pulses of a call in every launch.
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/optifax.h"
#include "ofx_fft64.cuh"

namespace {

struct Fp64Work {
    int n = 0, b = 0;
    double2 *A0 = nullptr, *A1 = nullptr, *NL = nullptr, *K1 = nullptr, *T = nullptr;
    double2* tw = nullptr;     // W_N^e, e < N/2
    int* flags = nullptr;      // per call: bit0 >= maxErr, bit1 >= minErr, bit2 NaN
    int* hflags = nullptr;     // pinned host copy
};

Fp64Work g_w[64];             // per device; a call allocates on first use or growth
std::mutex g_mu[64];


__device__ __forceinline__ double sample_time(int mode, int i, int n, double dt) {
    if (mode == 0) return (i > n / 2) ? dt * (double)(i - n / 2) : dt * (double)(i + n / 2);
    if (mode == 2) return (i < n / 2) ? dt * (double)i : dt * (double)(i - n);    // fftshift(t) (NEE)
    return dt * (double)i;
}

// NL = A^2 e^{i phi} + 2 |A|^2 e^{-i phi}, phi = w0 t_i - bdwz
__global__ void f64_nl(const double2* __restrict__ X, double2* __restrict__ NL, int n, double w0, double dt,
                       double bdwz, int time_mode) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    size_t o = (size_t)blockIdx.y * n + i;
    double s, c;
    sincos(w0 * sample_time(time_mode, i, n, dt) - bdwz, &s, &c);
    double2 a = X[o];
    double m2 = a.x * a.x + a.y * a.y;
    double2 a2 = make_double2(a.x * a.x - a.y * a.y, 2.0 * a.x * a.y);
    double2 e = make_double2(c, s);
    double2 t = dmul(a2, e);
    NL[o] = make_double2(t.x + 2.0 * m2 * c, t.y - 2.0 * m2 * s);
}

// K = -i hG (NL - i cs (NL[i+1] - NL[i-1])); mode 0: K1 = K, A1 = A0 + K;
// mode 1: E = A0 + (K/2 + K1/2), class |E - (A0 + K1)| against the thresholds
__global__ void f64_k(const double2* __restrict__ NL, const double2* __restrict__ A0, double2* __restrict__ K1,
                      double2* __restrict__ X, const double* __restrict__ G, int gstride, int kidx, double hmod,
                      double cs, int n, int mode, double maxE, double minE, int nee, int* flags) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int b = blockIdx.y;
    size_t base = (size_t)b * n;
    int ip = (i + 1 == n) ? 0 : i + 1, im = (i == 0) ? n - 1 : i - 1;
    double2 d = make_double2(NL[base + ip].x - NL[base + im].x, NL[base + ip].y - NL[base + im].y);
    double2 in = make_double2(NL[base + i].x + cs * d.y, NL[base + i].y - cs * d.x);
    double hg = hmod * G[(size_t)kidx + (size_t)b * gstride];   // kidx clamped to [0, S) by the host
    double2 k = make_double2(hg * in.y, -hg * in.x);
    double2 a0 = A0[base + i];
    if (mode == 0) {
        K1[base + i] = k;
        X[base + i] = make_double2(a0.x + (0.5 * k.x + 0.5 * k.x), a0.y + (0.5 * k.y + 0.5 * k.y));
    } else {
        double2 k1 = K1[base + i];
        double2 e, a1;
        if (nee) {    // NEE_CPU.m:73-75: A1 = A0 + K1, E = (A0 + K1/2) + K2/2
            e = make_double2((a0.x + 0.5 * k1.x) + 0.5 * k.x, (a0.y + 0.5 * k1.y) + 0.5 * k.y);
            a1 = make_double2(a0.x + k1.x, a0.y + k1.y);
        } else {
            e = make_double2(a0.x + (0.5 * k.x + 0.5 * k1.x), a0.y + (0.5 * k.y + 0.5 * k1.y));
            a1 = make_double2(a0.x + (0.5 * k1.x + 0.5 * k1.x), a0.y + (0.5 * k1.y + 0.5 * k1.y));
        }
        X[base + i] = e;
        double ae = hypot(e.x, e.y);
        int bits = 0;
        if (nee) {    // every point; maxErr strict (NEE_CPU.m:77-79)
            double pct = 100.0 * hypot(e.x - a1.x, e.y - a1.y) / (ae + 1.0);
            if (pct > maxE) bits |= 1;
            if (pct >= minE) bits |= 2;
        } else if (ae > 0.0) {
            double pct = 100.0 * hypot(e.x - a1.x, e.y - a1.y) / (ae + 1.0);
            if (pct >= maxE) bits = 1;
            else if (pct >= minE) bits = 2;
        }
        if (isnan(e.x) || isnan(e.y)) bits |= 4;
        bits = __reduce_or_sync(__activemask(), bits);
        if (bits && (threadIdx.x & 31) == 0) atomicOr(flags, bits);
    }
}

__global__ void f64_abc(double2* X, int n, int abc_mode, double dt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || abc_mode == 1) return;
    if (abc_mode == 3) {    // NEE_CPU.m:114-121
        const double t = sample_time(2, i, n, dt), range = (double)(n - 1) * dt, a2t = fabs(2.0 * t);
        if (!(range - a2t < 0.25 * range)) return;
        const double sh = 1.0 / cosh(24.0 * (1.0 - a2t / range));
        const size_t o = (size_t)blockIdx.y * n + i;
        X[o] = make_double2(X[o].x * (1.0 - sh * sh), X[o].y * (1.0 - sh * sh));
        return;
    }
    int gi1 = 6 * (n / 16), gi2 = 10 * (n / 16);
    if (!(i > gi1 && i < gi2)) return;
    size_t o = (size_t)blockIdx.y * n + i;
    double f;
    if (abc_mode == 2) f = 0.0;
    else {
        double pos = (48.0 / (double)n) * fabs((double)i - (double)n / 2.0);
        double g = cosh(pos);
        f = 1.0 - 1.0 / (g * g);
    }
    X[o] = make_double2(X[o].x * f, X[o].y * f);
}





__global__ void f64_disp(double2* X, const double* __restrict__ alpha, const double* __restrict__ beta, int n,
                         int s) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    size_t o = (size_t)blockIdx.y * n + i;
    double sn, cn;
    sincos(-beta[i] * (double)s, &sn, &cn);
    double a = pow(alpha[i], (double)s);
    X[o] = dmul(X[o], make_double2(cn * a, sn * a));
}

__global__ void f64_scale(const double2* __restrict__ x, double2* __restrict__ y, int n, double sc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    size_t o = (size_t)blockIdx.y * n + i;
    y[o] = make_double2(x[o].x * sc, x[o].y * sc);
}



int ensure(Fp64Work& w, int n, int b) {
    if (w.n == n && w.b >= b && w.A0) return 0;
    for (double2* p : {w.A0, w.A1, w.NL, w.K1, w.T, w.tw}) if (p) cudaFree(p);
    if (w.flags) cudaFree(w.flags);
    if (w.hflags) cudaFreeHost(w.hflags);
    w = Fp64Work();
    size_t sz = sizeof(double2) * (size_t)n * b;
    if (cudaMalloc(&w.A0, sz) || cudaMalloc(&w.A1, sz) || cudaMalloc(&w.NL, sz) || cudaMalloc(&w.K1, sz) ||
        cudaMalloc(&w.T, sz) || cudaMalloc(&w.tw, sizeof(double2) * (size_t)(n / 2)) ||
        cudaMalloc(&w.flags, sizeof(int)) || cudaMallocHost(&w.hflags, sizeof(int)))
        return OPTIFAX_ERR_NO_MEMORY;
    f64_twiddles<<<(n / 2 + 255) / 256, 256>>>(w.tw, n);
    if (cudaDeviceSynchronize() != cudaSuccess) return OPTIFAX_ERR_CUDA;
    w.n = n;
    w.b = b;
    return 0;
}

}  // namespace

extern "C" int optifax_propagate_fp64(int32_t n_points, int32_t n_pulses, int32_t n_steps,
                                      const double* E_in, double* A_out, const double* alpha, const double* beta,
                                      const double* G, int32_t g_per_pulse, double w0, double bdiffw0,
                                      double step_h, double dt, double max_err, double min_err, double sel,
                                      int32_t variant, int32_t* trace_host, int32_t trace_cap,
                                      optifax_pulse_stats* stats_host, void* stream) {
    const int n = n_points, B = n_pulses, S = n_steps;
    if (n < 16 || (n & (n - 1)) || B < 1 || S < 1 || !(sel >= 1.0) || !E_in || !A_out || !alpha || !beta || !G)
        return OPTIFAX_ERR_INVALID_ARGUMENT;
    int time_mode, abc_mode, guard, nee = 0;
    switch (variant) {
        case OPTIFAX_VARIANT_BATCH_XTAL:
        case OPTIFAX_VARIANT_BATCH_OP: time_mode = 0; abc_mode = 0; guard = 1; break;
        case OPTIFAX_VARIANT_NO_BC: time_mode = 1; abc_mode = 1; guard = 0; break;
        case OPTIFAX_VARIANT_HARD_BC: time_mode = 1; abc_mode = 2; guard = 0; break;
        case OPTIFAX_VARIANT_NEE: time_mode = 2; abc_mode = 3; guard = 0; nee = 1; break;
        default: return OPTIFAX_ERR_INVALID_ARGUMENT;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return OPTIFAX_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_mu[dev]);
    Fp64Work& w = g_w[dev];
    int rc = ensure(w, n, B);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t sz = sizeof(double2) * (size_t)n * B;
    if (cudaMemcpyAsync(w.A0, E_in, sz, cudaMemcpyDeviceToDevice, st) != cudaSuccess) return OPTIFAX_ERR_CUDA;
    const dim3 grid((n + 255) / 256, B);
    const double cs = 1.0 / (2.0 * dt * w0);
    const int gstride = g_per_pulse ? S : 0;
    int nchunks = (int)((double)S / sel);
    if (guard && (double)nchunks * sel < (double)S) nchunks += 1;
    double k = nee ? 1.0 : 0.0, stepprev = 4.0, stepmod = 4.0;   // NEE_CPU.m: k is 1-based
    long long q = 0;
    int attempt = 0, acc = 0, rej = 0, status = 0;
    const long long max_attempts = 64LL * (S + 16) + 64;
    for (int chunk = 0; chunk < nchunks; ++chunk) {
        if (!nee) stepmod = stepprev;
        const double cend = (double)(chunk + 1) * sel;
        while (k < cend && (nee ? k <= (double)S : (!guard || k < (double)S))) {
            if (attempt >= max_attempts) { status |= OPTIFAX_PULSE_ATTEMPT_LIMIT; goto done; }
            const double kg = nee ? k - 1.0 : k;     // G33(k) and the z of stage 1 are 1-based in NEE_CPU.m
            const int kidx = kg < 0.0 ? 0 : ((int)kg >= S ? S - 1 : (int)kg);
            const int krec = (int)k;
            const double hmod = stepmod * step_h;
            cudaMemsetAsync(w.flags, 0, sizeof(int), st);
            f64_nl<<<grid, 256, 0, st>>>(w.A0, w.NL, n, w0, dt, bdiffw0 * kg * step_h, time_mode);
            f64_k<<<grid, 256, 0, st>>>(w.NL, w.A0, w.K1, w.A1, G, gstride, kidx, hmod, cs, n, 0, max_err, min_err,
                                        nee, w.flags);
            f64_nl<<<grid, 256, 0, st>>>(w.A1, w.NL, n, w0, dt, bdiffw0 * (kg + stepmod) * step_h, time_mode);
            f64_k<<<grid, 256, 0, st>>>(w.NL, w.A0, w.K1, w.A1, G, gstride, kidx, hmod, cs, n, 1, max_err, min_err,
                                        nee, w.flags);
            cudaMemcpyAsync(w.hflags, w.flags, sizeof(int), cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) return OPTIFAX_ERR_CUDA;
            const int fl = *w.hflags;
            if (fl & 4) status |= OPTIFAX_PULSE_NAN;
            bool accepted = false;
            if ((fl & 1) && stepmod > 1.0 && (nee || (k - stepmod) > 0.0)) {
                if (trace_host && attempt < trace_cap) {
                    trace_host[3 * attempt] = krec; trace_host[3 * attempt + 1] = (int)stepmod;
                    trace_host[3 * attempt + 2] = fl & 7;
                }
                ++rej;
                if (!nee) k = k - stepmod;
                stepmod = stepmod - 1.0;
                stepprev = stepmod;
            } else {
                if (trace_host && attempt < trace_cap) {
                    trace_host[3 * attempt] = krec; trace_host[3 * attempt + 1] = (int)stepmod;
                    trace_host[3 * attempt + 2] = (fl & 7) | 8;
                }
                ++acc;
                accepted = true;
                const int s_used = (int)stepmod;
                f64_abc<<<grid, 256, 0, st>>>(w.A1, n, abc_mode, dt);
                fft64(w.A1, w.T, w.tw, n, B, +1, st);
                f64_disp<<<grid, 256, 0, st>>>(w.T, alpha, beta, n, s_used);
                fft64(w.T, w.A1, w.tw, n, B, -1, st);
                f64_scale<<<grid, 256, 0, st>>>(w.A1, w.A0, n, 1.0 / (double)n);
                q += s_used;
                if (nee) {    // NEE_CPU.m:77-83
                    if (!(fl & 2)) stepmod = stepmod + 1.0;
                    if (k < (double)S && k + stepmod > (double)S) stepmod = (double)S - k;
                } else if (k + stepmod >= cend && k < cend - 1.0) {
                    double stepend = (cend - k) - 1.0;
                    stepprev = stepmod;
                    stepmod = stepend;
                } else {
                    if (!(fl & 2) && !(fl & 1) && (k + stepmod + 1.0) < cend - 1.0) stepmod = stepmod + 1.0;
                    stepprev = stepmod;
                }
            }
            ++attempt;
            if (!nee || accepted) k = k + stepmod;
        }
    }
done:
    if (cudaMemcpyAsync(A_out, w.A0, sz, cudaMemcpyDeviceToDevice, st) != cudaSuccess) return OPTIFAX_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return OPTIFAX_ERR_CUDA;
    if (stats_host) {
        memset(stats_host, 0, sizeof(*stats_host));
        stats_host->attempts = attempt;
        stats_host->accepted = acc;
        stats_host->rejected = rej;
        stats_host->status = status;
        stats_host->z_steps = q;
        stats_host->k_final = (float)k;
        stats_host->stepmod_final = (float)stepmod;
        stats_host->n_chunks = nchunks;
    }
    return OPTIFAX_OK;
}
