// ofx_gnlse.cu -- chi(3) fibre GNLSE on the GPU: one persistent CTA per pulse.
//
// Replaces toolbox/lib/internal/main/gnlsefib.m:1-89.  The interaction-picture
// spectral field AW (n modes, FFT order) obeys gnlsefib.m:54-66,
//     dAW/dz = i gamma W ifft(AT ((1 - fR)|AT|^2 + RS)) e^{-Lz},
//     AT = fft(AW e^{Lz}),  RS = dT fR fft(ifft(|AT|^2) RW),  L = iB - alpha/2,
// in MATLAB's fft/ifft conventions (fft: exp(-i), ifft: exp(+i)/n), from
// AW(0) = ifft(A).  The reference integrates it with MATLAB's ode45 (RelTol,
// AbsTol, NormControl; gnlsefib.m:77-80), outputs at linspace(0, L, n_saves).
// Here: the Dormand-Prince 5(4) pair with the same tolerances and error norm,
//     err = ||h sum_i e_i k_i|| / max(||y||, ||y_new||, AbsTol/RelTol) <= RelTol,
// under ode45's published step control (Shampine & Reichelt 1997): initial step
// min(L/10, 0.8 RelTol^(1/5) max(||y0||, thr) / ||f0||), steps of at most L/10
// stretched to the end when 1.1 h reaches it, a first failure scaling h by
// max(0.1, 0.8 (RelTol/err)^(1/5)) and later ones halving it, growth by
// min(5, 0.8 (RelTol/err)^(1/5)) only after a step that did not fail.  Steps do
// not stop at the save points: a save point inside an accepted step is output
// from a separate step of exactly that length from the step's start (its stages
// reuse the accepted step's k1 and rows k2..k6; y_new waits in an eighth scratch
// row).  Positions are integers in units of length / 2^40 so that every
// dispersion phase B_k z is a 64-bit fixed-point product (exact mod one turn; only
// the final angle goes
// through FP32).  FP32 field arithmetic, norms reduced across the CTA in FP64
// (per-thread partials of 16 modes in FP32), FP64 step control.
//
// Layout: the CTA's M/16 threads hold the spectral state y in registers, 16
// modes each, in the FFT's bit-reversed slot order (slot s <-> mode bitrev(s));
// the time-domain fields live in two padded shared-memory buffers; the seven
// stage derivatives k_i and y_new sit in an L2-resident global scratch (8 x n per
// pulse, each thread touching only its own 128-byte rows).  Each right-hand side costs
// four in-place M-point transforms (two without Raman): MATLAB's fft of a
// spectral array is conj(inverse(conj(.))), its ifft (1/n) conj(forward(conj(.))).
#include <cmath>
#include <cstdint>

#include "ofx_fft.cuh"
#include "ofx_gnlse.cuh"

namespace ofx {
namespace {

constexpr int kZBits = 40;

// Dormand-Prince 5(4) tableau (Dormand & Prince 1980): nodes here; stage weights
// (row 6 = the 5th-order weights, FSAL) and error weights b - b_hat below (kA, kE).
__constant__ double kDpC[7] = {0.0, 1.0 / 5, 3.0 / 10, 4.0 / 5, 8.0 / 9, 1.0, 1.0};

__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

// Sums of two per-thread values over the CTA in FP64; every thread gets them.
template <int T>
__device__ __forceinline__ void block_sum2(double a, double b, double* red, double (&out)[2]) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    const int t = threadIdx.x;
    __syncthreads();                       // red may still be read from the previous call
    if ((t & 31) == 0) {
        red[2 * (t >> 5)] = a;
        red[2 * (t >> 5) + 1] = b;
    }
    __syncthreads();
    double s0 = 0.0, s1 = 0.0;
#pragma unroll 1
    for (int w = 0; w < T / 32; ++w) {     // fixed order: identical totals in every thread
        s0 += red[2 * w];
        s1 += red[2 * w + 1];
    }
    out[0] = s0; out[1] = s1;
}

// Squared norms of a thread's 16 modes: FP32 partial sums (16 terms, relative
// error below 1e-6), widened once for the FP64 block reduction.  GB300's FP64
// pipe is narrow, so per-mode FP64 conversions and adds cost a visible share of
// the step.
__device__ __forceinline__ double norm2_16(const float2 (&a)[16]) {
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 16; ++j) s = fmaf(a[j].x, a[j].x, fmaf(a[j].y, a[j].y, s));
    return (double)s;
}

// Own 16 slots of stage array j in the global scratch (128 contiguous bytes)
__device__ __forceinline__ const float4* krow(const float2* K, int M, int j, int t) {
    return reinterpret_cast<const float4*>(K + (size_t)j * M + 16 * t);
}

// The same tableau as compile-time values, so that the stage combinations unroll
// (all their L2 loads in flight together) and skip the zero weights.
__host__ __device__ constexpr float dp_a(int r, int q) {
    switch (r * 8 + q) {
        case 8: return 1.0f / 5;
        case 16: return 3.0f / 40;
        case 17: return 9.0f / 40;
        case 24: return 44.0f / 45;
        case 25: return -56.0f / 15;
        case 26: return 32.0f / 9;
        case 32: return 19372.0f / 6561;
        case 33: return -25360.0f / 2187;
        case 34: return 64448.0f / 6561;
        case 35: return -212.0f / 729;
        case 40: return 9017.0f / 3168;
        case 41: return -355.0f / 33;
        case 42: return 46732.0f / 5247;
        case 43: return 49.0f / 176;
        case 44: return -5103.0f / 18656;
        case 48: return 35.0f / 384;
        case 50: return 500.0f / 1113;
        case 51: return 125.0f / 192;
        case 52: return -2187.0f / 6784;
        case 53: return 11.0f / 84;
        default: return 0.f;
    }
}
__host__ __device__ constexpr float dp_e(int q) {
    switch (q) {
        case 0: return 71.0f / 57600;
        case 2: return -71.0f / 16695;
        case 3: return 71.0f / 1920;
        case 4: return -17253.0f / 339200;
        case 5: return 22.0f / 525;
        case 6: return -1.0f / 40;
        default: return 0.f;
    }
}

// acc += sum_q w_q h K[(base + q) % 7] over the compile-time weights w_q (row R of
// kA, or kE when R < 0), q < NQ
template <int R, int NQ>
__device__ __forceinline__ void combine(float2 (&acc)[16], const float2* K, int M, int t, int base, float hz) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        const float wq = (R >= 0) ? dp_a(R, q) : dp_e(q);
        if (wq == 0.f) continue;
        const float a = hz * wq;
        const float4* kr = krow(K, M, (base + q) % 7, t);
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) {
            const float4 w = kr[jj];
            acc[2 * jj].x = fmaf(a, w.x, acc[2 * jj].x);
            acc[2 * jj].y = fmaf(a, w.y, acc[2 * jj].y);
            acc[2 * jj + 1].x = fmaf(a, w.z, acc[2 * jj + 1].x);
            acc[2 * jj + 1].y = fmaf(a, w.w, acc[2 * jj + 1].y);
        }
    }
}

}  // namespace

template <int M>
__global__ void __launch_bounds__(M / 16, 1)
gnlse_kernel(const GnlseDev* __restrict__ pulses, const Twiddle* __restrict__ tw1, const Twiddle* __restrict__ tw2) {
    constexpr int T = M / 16;
    constexpr int LOG2M = FftShape<M>::LOG2M;
    constexpr int PADM = M + M / 16;
    extern __shared__ __align__(16) unsigned char smem[];
    float2* bufA = reinterpret_cast<float2*>(smem);          // time domain: conj(AT), then conj(Q)
    float2* bufB = bufA + PADM;                                // Raman: |AT|^2, then conj(RS / (dT fR))
    uint64_t* rate_s = reinterpret_cast<uint64_t*>(bufB + PADM);   // B_k z per z unit, 2^-64 turns
    float2* rw_s = reinterpret_cast<float2*>(rate_s + M);
    float* w_s = reinterpret_cast<float*>(rw_s + M);
    double* red = reinterpret_cast<double*>(w_s + M);

    const int t = threadIdx.x;
    __shared__ GnlseDev sP;
    if (t == 0) sP = pulses[blockIdx.x];
    __syncthreads();
    const GnlseDev& P = sP;
    const bool raman = (P.RW != nullptr);
    const double unit = P.length / (double)(1ll << kZBits);
    const long long total = 1ll << kZBits;
    const long long hmax = total / 10;
    const double thr = P.atol / P.rtol;
    const float invM = 1.0f / (float)M;
    const float gam = (float)P.gamma, omfr = (float)(1.0 - P.fr), dtfr = (float)(P.dT * P.fr);
    const float awscale = (float)(P.dT * (double)M);
    float2* K = P.K;

    // per-mode tables in slot order (slot s holds mode bitrev(s))
#pragma unroll 1
    for (int j = 0; j < 16; ++j) {
        const int slot = 16 * t + j;
        const int k = bitrev(slot, LOG2M);
        double r = P.B[k] * unit * 0.15915494309189533577;     // turns per z unit
        r -= rint(r);
        double x = r * 18446744073709551616.0;
        if (x >= 9.2233720368547758e18) x -= 1.8446744073709552e19;
        rate_s[slot] = (uint64_t)(long long)llrint(x);
        w_s[slot] = P.W[k];
        rw_s[slot] = raman ? P.RW[k] : make_float2(0.f, 0.f);
    }
    // y(0) = ifft(A) = conj(forward(conj(A))) / M
#pragma unroll
    for (int j = 0; j < 16; ++j) bufA[phys(16 * t + j)] = conjf2(P.A[16 * t + j]);
    __syncthreads();
    float2 y[16], ys[16], v[16], e[16];
    fft_forward_to_regs<M>(bufA, tw1, tw2, t, v);
#pragma unroll
    for (int j = 0; j < 16; ++j) y[j] = cscale(conjf2(v[j]), invM);

    long long zc = 0, hc = 0, h = 0, side_z = 0;
    int save_idx = 0, stage = 0, base = 0;
    int attempts = 0, accepted = 0, status = 0;
    bool nofailed = true, new_step = true, side = false;
    double ny = 0.0, acc_nyn = 0.0, acc_err = 0.0;
    float hz = 0.f;
    const long long nm1 = P.n_saves - 1;
    auto save_point = [&](int i) -> long long { return ((long long)i * total + nm1 / 2) / nm1; };

    // save `save_idx` from the spectral state src at position zp: AW e^{Lz}
    // (fftshifted, x dT n) and AT = fft(AW e^{Lz})
    auto do_save = [&](const float2 (&src)[16], long long zp) {
        const float att = expf((float)(-0.5 * P.alpha * (double)zp * unit));
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int slot = 16 * t + j;
            const float2 aw = cscale(cmul(src[j], turn_to_unit(rate_s[slot] * (uint64_t)zp)), att);
            const int k = bitrev(slot, LOG2M);
            P.AW_out[(size_t)save_idx * M + ((k + M / 2) & (M - 1))] = cscale(aw, awscale);
            v[j] = conjf2(aw);
        }
        fft_inverse_from_regs<M>(bufA, tw1, tw2, t, v);
#pragma unroll
        for (int j = 0; j < 16; ++j)
            P.AT_out[(size_t)save_idx * M + 16 * t + j] = conjf2(bufA[phys(16 * t + j)]);
        ++save_idx;
    };
    do_save(y, 0);

    for (;;) {
        // ---- stage input ys and its position zs ----
        long long zs = zc;
#pragma unroll
        for (int j = 0; j < 16; ++j) ys[j] = y[j];
        if (stage > 0) {
            if (stage == 1 && !side) {
                if (new_step) {
                    h = h > hmax ? hmax : (h < 1 ? 1 : h);
                    hc = h;
                    if (1.1 * (double)hc >= (double)(total - zc)) hc = total - zc;   // stretch to the end
                    nofailed = true;
                    new_step = false;
                }
                hz = (float)((double)hc * unit);
            } else if (stage == 1) {
                hz = (float)((double)(side_z - zc) * unit);
            }
            switch (stage) {
                case 1: combine<1, 1>(ys, K, M, t, base, hz); break;
                case 2: combine<2, 2>(ys, K, M, t, base, hz); break;
                case 3: combine<3, 3>(ys, K, M, t, base, hz); break;
                case 4: combine<4, 4>(ys, K, M, t, base, hz); break;
                case 5: combine<5, 5>(ys, K, M, t, base, hz); break;
                default: combine<6, 6>(ys, K, M, t, base, hz); break;
            }
            zs = zc + llrint(kDpC[stage] * (double)(side ? side_z - zc : hc));
        }
        // ---- right-hand side f(zs, ys) (gnlsefib.m:54-66) into v ----
        {
            const double zd = (double)zs * unit;
            const float att = expf((float)(-0.5 * P.alpha * zd));
            const float iatt = expf((float)(0.5 * P.alpha * zd));
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                e[j] = turn_to_unit(rate_s[16 * t + j] * (uint64_t)zs);      // e^{i B z}
                v[j] = conjf2(cscale(cmul(ys[j], e[j]), att));
            }
            fft_inverse_from_regs<M>(bufA, tw1, tw2, t, v);                   // bufA = conj(AT)
            if (raman) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const float2 c = bufA[phys(16 * t + j)];
                    bufB[phys(16 * t + j)] = make_float2(c.x * c.x + c.y * c.y, 0.f);
                }
                __syncthreads();
                fft_forward_to_regs<M>(bufB, tw1, tw2, t, v);                 // forward(|AT|^2)
#pragma unroll
                for (int j = 0; j < 16; ++j)                                  // conj(ifft(|AT|^2) RW)
                    v[j] = conjf2(cscale(cmul(conjf2(v[j]), rw_s[16 * t + j]), invM));
                fft_inverse_from_regs<M>(bufB, tw1, tw2, t, v);               // bufB = conj(RS / (dT fR))
            }
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float2 at = conjf2(bufA[phys(16 * t + j)]);
                const float it = at.x * at.x + at.y * at.y;
                float2 g = make_float2(it, 0.f);
                if (raman) {
                    const float2 rb = bufB[phys(16 * t + j)];
                    g = make_float2(fmaf(omfr, it, dtfr * rb.x), -dtfr * rb.y);
                }
                bufA[phys(16 * t + j)] = conjf2(cmul(at, g));                  // conj(Q)
            }
            __syncthreads();
            fft_forward_to_regs<M>(bufA, tw1, tw2, t, v);                     // ifft(Q) = conj(v) / M
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float2 m = cmul(conjf2(v[j]), conjf2(e[j]));
                const float s = gam * w_s[16 * t + j] * iatt * invM;
                v[j] = make_float2(-m.y * s, m.x * s);                        // i gamma W M e^{-Lz}
            }
        }
        {
            float4* kw = reinterpret_cast<float4*>(K + (size_t)((base + stage) % 7) * M + 16 * t);
#pragma unroll
            for (int jj = 0; jj < 8; ++jj)
                kw[jj] = make_float4(v[2 * jj].x, v[2 * jj].y, v[2 * jj + 1].x, v[2 * jj + 1].y);
        }
        if (stage == 0) {
            // initial step (ode45, NormControl): min(hmax, 0.8 rtol^(1/5) max(||y||, thr) / ||f||)
            double s2[2];
            block_sum2<T>(norm2_16(y), norm2_16(v), red, s2);
            ny = sqrt(s2[0]);
            const double nf = sqrt(s2[1]);
            if (nf == 0.0) h = hmax;
            else {
                double hh = (0.8 * pow(P.rtol, 0.2)) * fmax(ny, thr) / nf / unit;
                long long hi = hh >= (double)hmax ? hmax : (long long)hh;
                h = hi < 1 ? 1 : hi;
            }
            stage = 1;
            continue;
        }
        bool finish = false;
        if (side) {
            if (stage < 5) { ++stage; continue; }
            // stages k2..k6 of the step to the save point done: y(side_z) = y + h' sum a_7j k_j
#pragma unroll
            for (int j = 0; j < 16; ++j) ys[j] = y[j];
            combine<6, 6>(ys, K, M, t, base, hz);
            do_save(ys, side_z);
            if (save_idx < P.n_saves && save_point(save_idx) < zc + hc) {
                side_z = save_point(save_idx);
                stage = 1;
                continue;
            }
            // back to the accepted step: y_new from the stash row
            const float4* sr = krow(K, M, 7, t);
#pragma unroll
            for (int jj = 0; jj < 8; ++jj) {
                const float4 w = sr[jj];
                ys[2 * jj] = make_float2(w.x, w.y);
                ys[2 * jj + 1] = make_float2(w.z, w.w);
            }
            side = false;
            finish = true;
        } else {
            if (stage < 6) { ++stage; continue; }

            // ---- stage 6 done: ys = y_new, error estimate and decision ----
            float2 ev[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) ev[j] = make_float2(0.f, 0.f);
            combine<-1, 7>(ev, K, M, t, base, hz);
            double s2[2];
            block_sum2<T>(norm2_16(ev), norm2_16(ys), red, s2);
            const double errn = sqrt(s2[0]), nyn = sqrt(s2[1]);
            const double err = errn / fmax(fmax(ny, nyn), thr);
            const bool ok = err <= P.rtol;
            if (t == 0 && P.trace && attempts < P.trace_cap) {
                P.trace[2 * attempts] = hc;
                P.trace[2 * attempts + 1] = ok ? 1 : 0;
            }
            ++attempts;
            if (!isfinite(errn) || !isfinite(nyn)) { status |= OPTIFAX_PULSE_NAN; break; }
            if (ok) {
                ++accepted;
                acc_err = err;
                acc_nyn = nyn;
                if (save_idx < P.n_saves && save_point(save_idx) < zc + hc) {
                    // a save point inside the step: stash y_new, then a step of exactly that length
                    float4* sw = reinterpret_cast<float4*>(K + (size_t)7 * M + 16 * t);
#pragma unroll
                    for (int jj = 0; jj < 8; ++jj)
                        sw[jj] = make_float4(ys[2 * jj].x, ys[2 * jj].y, ys[2 * jj + 1].x, ys[2 * jj + 1].y);
                    side = true;
                    side_z = save_point(save_idx);
                    stage = 1;
                    continue;
                }
                finish = true;
            } else {
                // a failed step: the first failure scales by max(0.1, 0.8 (rtol/err)^(1/5)),
                // later ones halve (the factor only scales an integer step: FP32 powf serves)
                if (nofailed) {
                    nofailed = false;
                    const float errf = (float)err;
                    const double fac = (double)fmaxf(0.1f, 0.8f * powf((float)P.rtol / errf, 0.2f));
                    const long long hi = (long long)((double)hc * fac);
                    hc = hi < 1 ? 1 : hi;
                } else {
                    hc = hc / 2 < 1 ? 1 : hc / 2;
                }
                if (attempts >= P.max_attempts) { status |= OPTIFAX_PULSE_ATTEMPT_LIMIT; break; }
                stage = 1;
                continue;
            }
        }
        if (finish) {
            zc += hc;
#pragma unroll
            for (int j = 0; j < 16; ++j) y[j] = ys[j];
            ny = acc_nyn;
            base = (base + 6) % 7;                          // FSAL: k7 becomes the next k1
            if (save_idx < P.n_saves && save_point(save_idx) == zc) do_save(y, zc);
            if (save_idx >= P.n_saves || zc >= total) break;
            // growth after a step with no failure: h / (1.25 (err/rtol)^(1/5)), at most 5 h
            if (nofailed) {
                const float ratio = (float)(acc_err / P.rtol);
                const float temp = 1.25f * powf(ratio, 0.2f);
                h = temp > 0.2f ? (long long)((double)hc / (double)temp) : 5 * hc;
            } else {
                h = hc;
            }
            new_step = true;
            if (attempts >= P.max_attempts) { status |= OPTIFAX_PULSE_ATTEMPT_LIMIT; break; }
            stage = 1;
        }
    }
    if (t == 0 && P.stats) {
        optifax_gnlse_stats st;
        st.attempts = attempts; st.accepted = accepted; st.status = status; st.reserved = 0;
        *P.stats = st;
    }
}

template <int M>
cudaError_t launch_one(const GnlseDev* d, int n_pulses, const Twiddle* tw1, const Twiddle* tw2, cudaStream_t st) {
    constexpr int PADM = M + M / 16;
    const size_t smem = sizeof(float2) * 2 * PADM + (sizeof(uint64_t) + sizeof(float2) + sizeof(float)) * M +
                        sizeof(double) * 2 * (M / 16 / 32 > 0 ? M / 16 / 32 : 1);
    cudaError_t e = cudaFuncSetAttribute(gnlse_kernel<M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    gnlse_kernel<M><<<n_pulses, M / 16, smem, st>>>(d, tw1, tw2);
    return cudaGetLastError();
}

cudaError_t launch_gnlse(int M, const GnlseDev* d, int n_pulses, const Twiddle* tw1, const Twiddle* tw2,
                         cudaStream_t st) {
    switch (M) {
        case 512: return launch_one<512>(d, n_pulses, tw1, tw2, st);
        case 1024: return launch_one<1024>(d, n_pulses, tw1, tw2, st);
        case 2048: return launch_one<2048>(d, n_pulses, tw1, tw2, st);
        case 4096: return launch_one<4096>(d, n_pulses, tw1, tw2, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace ofx
