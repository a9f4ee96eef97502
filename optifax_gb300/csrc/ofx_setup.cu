// ofx_setup.cu -- per-pulse solver inputs computed on the device (FP64), so that
// sweeps of hundreds of crystals and pulses are not bound by host precompute.
//
// For each pulse it produces what OpticalSim.run computes on the host before the
// solver call (OpticalSim.m:213-226): the dispersion phase per step hB
// (phi_calc.m:14-45 with the MgO:LN Sellmeier of Gayer et al., group delay at the
// reference removed), the per-step transmission T^(1/S) (transmission window), the
// QPM drive G33 from the domain walls (QPMcrystal.m:20-51), and the in-crystal
// input field: a transform-limited sech^2 pump (sechPulse.m, Laser.m:66-77) plus
// one photon per mode with a counter-based random phase, refracted into the
// crystal.  Every array is in the layout the solver takes (natural FFT order of
// the fftshifted grid; FP32 alpha/beta/G, complex64 field).  Scalar inputs are
// computed by the host (a handful of values per pulse).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "../../include/optifax.h"
#include "ofx_fft64.cuh"

namespace {

constexpr double kC0 = 299792458.0;
constexpr double kEps0 = 8.854e-12;         // the reference's CONST/eps0.m value
constexpr double kHbar = 1.054571817e-34;
constexpr double kPi = 3.141592653589793238462643383279502884;

// Gayer et al., Appl. Phys. B 91, 343 (2008), 5 % MgO:CLN extraordinary index
__device__ double n_mgoln_e(double lam_um, double celsius) {
    const double fn = (celsius - 24.5) * (celsius + 570.82);
    const double l2 = lam_um * lam_um;
    const double a3 = 0.2020 + 6.113e-8 * fn;
    const double n2 = (5.756 + 2.860e-6 * fn) + (0.0983 + 4.700e-8 * fn) / (l2 - a3 * a3) +
                      (189.32 + 1.516e-4 * fn) / (l2 - 12.52 * 12.52) - 1.32e-2 * l2;
    double n = n2 > 0.0 ? sqrt(n2) : 0.0;
    if (!isfinite(n) || n < 1.0) n = 1.0;   // Dielectric.m:43-44
    return n;
}

struct Grid {
    int n;
    double dt, f0, w_ref;
    __device__ double omega(int j) const {    // ascending frequency index j
        return 2.0 * kPi * ((double)(j - n / 2) / ((double)n * dt) + f0);
    }
};

// phi_abs_j = L w_j n_j / c over the ascending grid
__global__ void k_phase(Grid g, double length, double celsius, double* __restrict__ phi_abs) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.n) return;
    const double w = g.omega(j);
    const double lam = 2.0 * kPi * kC0 / w;
    const double n = n_mgoln_e(lam * 1e6, celsius);
    phi_abs[j] = length * (w * n / kC0);
}

// del_phi_j = (GD_j - GD_ref) (w_rel_j - w_rel_{j-1}), GD by backward differences
__global__ void k_delphi(Grid g, const double* __restrict__ phi_abs, double* __restrict__ del) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.n) return;
    if (j == 0) { del[0] = 0.0; return; }
    const int r = g.n / 2;
    const double gd = (phi_abs[j] - phi_abs[j - 1]) / (g.omega(j) - g.omega(j - 1));
    const double gd_r = (phi_abs[r] - phi_abs[r - 1]) / (g.omega(r) - g.omega(r - 1));
    const double wr_j = g.omega(j) - g.w_ref, wr_p = g.omega(j - 1) - g.w_ref;
    del[j] = (gd - gd_r) * (wr_j - wr_p);
}

// trapezoidal running integral over the ascending indices with 0.2 um < lambda <
// 20 um (one contiguous range): cum[ja] = 0, cum[j] = cum[j-1] + (d_j + d_{j-1}) / 2.
// One block of 1024 threads, each a contiguous piece; block scan of the pieces.
__global__ void k_cumtrapz(Grid g, const double* __restrict__ del, double* __restrict__ cum) {
    __shared__ double part[1024];
    __shared__ int s_ja, s_jb;
    if (threadIdx.x == 0) { s_ja = g.n; s_jb = -1; }
    __syncthreads();
    for (int j = threadIdx.x; j < g.n; j += blockDim.x) {
        const double lam = 2.0 * kPi * kC0 / g.omega(j);
        if (lam > 2e-7 && lam < 2e-5) { atomicMin(&s_ja, j); atomicMax(&s_jb, j); }
        cum[j] = 0.0;
    }
    __syncthreads();
    const int ja = s_ja, jb = s_jb;
    if (jb <= ja) return;
    const int len = jb - ja;                            // increments at ja+1 .. jb
    const int per = (len + blockDim.x - 1) / blockDim.x;
    const int lo = ja + 1 + threadIdx.x * per, hi = min(jb + 1, lo + per);
    double s = 0.0;
    for (int j = lo; j < hi; ++j) s += 0.5 * (del[j] + del[j - 1]);
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double acc = 0.0;
        for (int i = 0; i < (int)blockDim.x; ++i) { const double v = part[i]; part[i] = acc; acc += v; }
    }
    __syncthreads();
    double acc = part[threadIdx.x];
    for (int j = lo; j < hi; ++j) { acc += 0.5 * (del[j] + del[j - 1]); cum[j] = acc; }
}

// solver arrays in natural FFT order: alpha, beta (per step), refraction factor,
// noise spectrum seed mask
__global__ void k_arrays(Grid g, const double* __restrict__ cum, double length, double step, double celsius,
                         double lam_lo, double lam_hi, float* __restrict__ alpha, float* __restrict__ beta,
                         double* __restrict__ rfac) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= g.n) return;
    const int j = (k + g.n / 2) % g.n;
    const double w = g.omega(j), lam = 2.0 * kPi * kC0 / w;
    const bool in = lam >= lam_lo && lam <= lam_hi;
    const double phi_rel = cum[j] - cum[g.n / 2];
    const double b = phi_rel / length * step;
    alpha[k] = in ? 1.f : 0.f;
    beta[k] = (in && isfinite(b)) ? (float)b : 0.f;
    rfac[k] = sqrt(1.0 / n_mgoln_e(lam * 1e6, celsius));
}

// QPM sign per z-sample: z = linspace(0, L, S); q = 1 + #walls <= z; G = -(2 (q mod 2) - 1) g
__global__ void k_qpm(int S, double length, const double* __restrict__ walls, int n_walls, double g_scale,
                      float* __restrict__ G) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S) return;
    const double step = length / (double)(S - 1);
    const double z = (i == S - 1) ? length : (double)i * step;
    int lo = 0, hi = n_walls;                          // first wall > z
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (walls[mid] <= z) lo = mid + 1; else hi = mid;
    }
    const int q = 1 + lo;
    G[i] = (float)((q & 1) ? -g_scale : g_scale);
}

struct PumpArgs {
    double t_rms, dw, energy, area, n_medium, T;
};

__device__ __forceinline__ double2 pump_u(const Grid& g, const PumpArgs& a, int j) {
    const double t = (double)(j - g.n / 2) / (double)g.n * a.T;
    const double u = 1.0 / cosh(t / a.t_rms);
    double s, c;
    sincos(a.dw * t, &s, &c);
    return make_double2(u * c, u * s);
}

__global__ void k_pump_norm(Grid g, PumpArgs a, double* __restrict__ sum) {
    __shared__ double red[32];
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (j < g.n) { const double2 u = pump_u(g, a, j); v = u.x * u.x + u.y * u.y; }
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
        atomicAdd(sum, s);
    }
}

// fftshift(pump field) in natural order
__global__ void k_pump_fill(Grid g, PumpArgs a, const double* __restrict__ sum, double2* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= g.n) return;
    const double scale = sqrt(2.0 * a.energy / (sum[0] * g.dt * a.area * a.n_medium * kEps0 * kC0));
    const double2 u = pump_u(g, a, (k + g.n / 2) % g.n);
    out[k] = make_double2(scale * u.x, scale * u.y);
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Y_k = (FFT(fftshift(pump))_k + noise_k) sqrt(1 / n_k): one photon per mode with a
// counter-based uniform phase on the seeded bins (w_k > 0, inside the window)
__global__ void k_spectrum(Grid g, const double2* __restrict__ P, const double* __restrict__ rfac,
                           const float* __restrict__ alpha, uint64_t seed, double area, double n_medium,
                           double2* __restrict__ Y) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= g.n) return;
    const int j = (k + g.n / 2) % g.n;
    const double w = g.omega(j);
    double2 v = P[k];
    if (w > 0.0 && alpha[k] > 0.f) {
        const double amp = sqrt(fmax(2.0 * kHbar * w * (double)g.n / (kC0 * n_medium * kEps0 * area * g.dt), 0.0));
        const uint64_t key = seed * 0x100000001B3ull;
        const uint64_t r = splitmix64((uint64_t)k + (key << 20));
        const double ph = 2.0 * kPi * ((double)(r >> 11) * (1.0 / 9007199254740992.0));
        double s, c;
        sincos(ph, &s, &c);
        v.x += amp * c;
        v.y += amp * s;
    }
    const double f = rfac[k];
    Y[k] = make_double2(v.x * f, v.y * f);
}

__global__ void k_field_out(int n, const double2* __restrict__ x, float2* __restrict__ E) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double inv = 1.0 / (double)n;
    E[k] = make_float2((float)(x[k].x * inv), (float)(x[k].y * inv));
}

inline unsigned nb(long long n) { return (unsigned)((n + 255) / 256); }

}  // namespace

extern "C" int64_t optifax_setup_work_bytes(int32_t max_points) {
    if (max_points < 16) return -1;
    return (int64_t)max_points * 64 + 256;
}

extern "C" int optifax_setup_pulses(const optifax_setup* s, int32_t n, void* work, int64_t work_bytes,
                                    void* stream) {
    if (!s || n < 1 || !work) return OPTIFAX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    for (int p = 0; p < n; ++p) {
        const optifax_setup& d = s[p];
        const int N = d.n_points, S = d.n_steps;
        if (N < 16 || (N & (N - 1)) || S < 2 || !(d.dt > 0.0) || !(d.lambda_ref > 0.0) || !(d.length > 0.0) ||
            !(d.step_size > 0.0) || !d.alpha || !d.beta || !d.G || !d.E || (d.n_walls > 0 && !d.walls) ||
            d.n_walls < 0 || !(d.pump_t_rms > 0.0) || !(d.waist > 0.0) || !(d.n_medium > 0.0))
            return OPTIFAX_ERR_INVALID_ARGUMENT;
        // the phase integration covers 0.2-20 um; the window must lie inside it
        if (!(d.lambda_lo_nm > 200.0 && d.lambda_hi_nm < 20000.0 && d.lambda_lo_nm < d.lambda_hi_nm))
            return OPTIFAX_ERR_UNSUPPORTED;
        if (work_bytes < optifax_setup_work_bytes(N)) return OPTIFAX_ERR_INVALID_ARGUMENT;
        char* base = static_cast<char*>(work);
        double2* tw = reinterpret_cast<double2*>(base);                  // N/2 complex
        double2* b1 = tw + N / 2;                                         // N complex
        double2* b2 = b1 + N;                                             // N complex
        double* d1 = reinterpret_cast<double*>(b2 + N);                   // N
        double* d2 = d1 + N;                                              // N
        double* rfac = d2 + N;                                            // N
        double* sum = rfac + N;                                           // 1
        Grid g{N, d.dt, kC0 / d.lambda_ref, 2.0 * kPi * kC0 / d.lambda_ref};
        f64_twiddles<<<nb(N / 2), 256, 0, st>>>(tw, N);
        k_phase<<<nb(N), 256, 0, st>>>(g, d.length, d.celsius, d1);
        k_delphi<<<nb(N), 256, 0, st>>>(g, d1, d2);
        k_cumtrapz<<<1, 1024, 0, st>>>(g, d2, d1);
        k_arrays<<<nb(N), 256, 0, st>>>(g, d1, d.length, d.step_size, d.celsius, d.lambda_lo_nm * 1e-9,
                                        d.lambda_hi_nm * 1e-9, d.alpha, d.beta, rfac);
        k_qpm<<<nb(S), 256, 0, st>>>(S, d.length, d.walls, d.n_walls, d.g_scale, d.G);
        const double w_p = 2.0 * kPi * kC0 / d.pump_lambda;
        const PumpArgs pa{d.pump_t_rms, w_p - g.w_ref, d.pump_energy, kPi * d.waist * d.waist, d.n_medium, d.window};
        if (cudaMemsetAsync(sum, 0, sizeof(double), st) != cudaSuccess) return OPTIFAX_ERR_CUDA;
        k_pump_norm<<<nb(N), 256, 0, st>>>(g, pa, sum);
        k_pump_fill<<<nb(N), 256, 0, st>>>(g, pa, sum, b1);
        fft64(b1, b2, tw, N, 1, +1, st);
        k_spectrum<<<nb(N), 256, 0, st>>>(g, b2, rfac, d.alpha, (uint64_t)(int64_t)d.seed, pa.area, d.n_medium, b1);
        fft64(b1, b2, tw, N, 1, -1, st);
        k_field_out<<<nb(N), 256, 0, st>>>(N, b2, static_cast<float2*>(d.E));
        if (cudaGetLastError() != cudaSuccess) return OPTIFAX_ERR_CUDA;
    }
    return OPTIFAX_OK;
}
