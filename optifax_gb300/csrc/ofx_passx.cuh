// ofx_passx.cuh -- the persistent crystal-pass kernel with a wide field state.
//
// passx_kernel<R, M, C, NEE> runs the same Heun schedule as pass_kernel
// (ofx_pass.cuh; reference OPO_CUDA_BATCH_XTAL.cu:373-525 and its variants,
// NEE_CPU.m:1-122 with NEE) with every field value, stage sum and transform in
// the arithmetic type R:
//   R = double  the plain FP64 solver: the FP64 comparator of the FP32
//               propagator, computed as the FP64 oracle computes it;
//   R = ff      float-float (ofx_num.cuh), ~48-bit significands from FP32
//               operations, for high-gain passes in which FP32 rounding of the
//               field, amplified by the parametric gain, dominates the result.
// One thread-block cluster of C CTAs holds one pulse of N = C M points for the
// whole pass; each of the 256 threads of a CTA owns P = M / 256 consecutive
// time points (field A0 in registers).  Per attempt: the NL drive and shock
// stencil of both Heun stages (neighbour values through shared and distributed
// shared memory), the stage combine and the error class, an OR over the cluster
// (and the grid for a shared batch schedule).  Accepted steps: absorber, the
// N-point transform as C-point DFTs across the cluster (distributed shared
// memory, twiddles W_N^{n2 k1}) and an M-point Stockham transform in shared
// memory, the per-mode dispersion factor alpha^s exp(-i beta s), the inverse,
// 1/N.  Phases (carrier w0 t_i and z-carrier bdiffw0 z) are exact 64-bit
// fixed-point turns evaluated by FP64 sincospi; the dispersion factor and the
// absorber are FP64 (then rounded to R), as in the FP64 oracle.
#pragma once
#include <cooperative_groups.h>
#include <type_traits>
#include "ofx_num.cuh"
#include "ofx_pass.cuh"

namespace ofx {

// Per-pulse descriptor of the wide-state pass (device pointers).
struct PulseX {
    const double2* E_in;     // N complex doubles, fftshifted time
    double2* A_out;
    const double* alpha;     // N, FFT order
    const double* beta;      // N, FFT order
    const double* G;         // S
    int* trace;              // 3 ints per attempt (k, stepmod, flags | 8 accepted), or null
    const int* forced;
    optifax_pulse_stats* stats;
    void* cph;               // scratch: N carrier phasors exp(i w0 t_i) in R (written by the prologue)
    double* abc;             // scratch: N absorber factors
    void* ztab;              // scratch: zcap z-carrier phasors exp(-i bdiffw0 h p), p = 0..zcap-1, in R
    int zcap;
    uint64_t tau_theta;      // w0 dt in turns
    uint64_t tau_z;          // bdiffw0 h in turns (per z-sample)
    double w0, h, dt, max_err, min_err, sel, c_shock;
    int N, S, nchunks, trace_cap, n_forced;
};

// W_N^e (N = C M) for e in [0, N), in R; the local transforms use W_M^e = W_N^{C e}.
template <typename R>
struct XTables { const typename Num<R>::cplx* wn; };

constexpr int kXThreads = 256;

template <typename R, int M>
struct SmemX {
    using cplx = typename Num<R>::cplx;
    static constexpr int T = kXThreads;
    static constexpr size_t off_x = 0;                                    // stage output / transform
    static constexpr size_t off_k = off_x + sizeof(cplx) * M;             // K1 / transform ping-pong
    static constexpr size_t off_d = off_k + sizeof(cplx) * M;             // per-mode dispersion factor
    static constexpr size_t off_edge = off_d + sizeof(cplx) * M;          // 2 parities x 2 x T
    static constexpr size_t off_wc = off_edge + sizeof(cplx) * 4 * T;     // W_C^m, m < 8
    static constexpr size_t off_red = off_wc + sizeof(cplx) * 8;          // flag slots
    static constexpr size_t bytes = off_red + 256;
};

// exp(2 pi i u / 2^64) in FP64: the turn as a signed fraction in half-turns
__device__ __forceinline__ double2 turn_unit_d(uint64_t u) {
    const double x = (double)(long long)u * 0x1p-63;
    double s, c;
    sincospi(x, &s, &c);
    return make_double2(c, s);
}

// ---------------------------------------------------------------------------
// C-point DFT in registers by radix-2 DIF stages (bit-reversed output: v[q]
// holds output bitrev(q)); wc[m] = W_C^m (m < C/2), INV uses the conjugates.
// ---------------------------------------------------------------------------
template <typename R, int CP, bool INV>
__device__ __forceinline__ void dft_small(typename Num<R>::cplx* v, const typename Num<R>::cplx* wc) {
    using X = Num<R>;
#pragma unroll
    for (int hr = CP / 2; hr >= 1; hr >>= 1) {
#pragma unroll
        for (int q = 0; q < CP; ++q) {
            if (q & hr) continue;
            const int m = (q & (hr - 1)) * (CP / (2 * hr));
            const typename X::cplx a = v[q], b = v[q + hr];
            v[q] = X::add(a, b);
            const typename X::cplx d = X::sub(a, b);
            if (m == 0) v[q + hr] = d;
            else if (2 * m == CP / 2) v[q + hr] = INV ? X::mul_i(d) : X::mul_mi(d);    // W_C^{C/4} = -i
            else v[q + hr] = INV ? X::mulc(d, wc[m]) : X::mul(d, wc[m]);
        }
    }
}

// ---------------------------------------------------------------------------
// M-point Stockham autosort transform in shared memory (radix 4, one radix-2
// pass when log2 M is odd), ping-pong between a and b; returns the buffer that
// holds the result (natural order).  Pass over sub-transform length Ls: for
// j < M/R, k = j mod Ls, x_r = in[j + r M/R] W_{R Ls}^{r k}, y = DFT_R(x),
// out[(j - k) R + k + s Ls] = y_s.  Unnormalised; INV conjugates every twiddle.
// ---------------------------------------------------------------------------
template <typename R, int M, int C, bool INV>
__device__ __forceinline__ typename Num<R>::cplx* stockham(typename Num<R>::cplx* a, typename Num<R>::cplx* b,
                                                           const typename Num<R>::cplx* __restrict__ wn, int t) {
    using X = Num<R>;
    using cplx = typename X::cplx;
    constexpr int T = kXThreads;
    cplx* in = a;
    cplx* out = b;
    int Ls = 1;
#pragma unroll 1
    for (; Ls * 4 <= M; Ls *= 4) {
        const int stride = M / (4 * Ls);
#pragma unroll
        for (int u = 0; u < (M / 4 + T - 1) / T; ++u) {
            const int j = t + u * T;
            if (j >= M / 4) break;
            const int k = j & (Ls - 1);
            cplx x0 = in[j], x1 = in[j + M / 4], x2 = in[j + M / 2], x3 = in[j + 3 * (M / 4)];
            if (Ls > 1) {
                const int e = k * stride;
                const cplx w1 = wn[(size_t)e * C], w2 = wn[(size_t)(2 * e) * C], w3 = wn[(size_t)(3 * e) * C];
                x1 = INV ? X::mulc(x1, w1) : X::mul(x1, w1);
                x2 = INV ? X::mulc(x2, w2) : X::mul(x2, w2);
                x3 = INV ? X::mulc(x3, w3) : X::mul(x3, w3);
            }
            const cplx a0 = X::add(x0, x2), a1 = X::sub(x0, x2);
            const cplx b0 = X::add(x1, x3);
            const cplx d13 = X::sub(x1, x3);
            const cplx b1 = INV ? X::mul_i(d13) : X::mul_mi(d13);
            const int base = (j - k) * 4 + k;
            out[base] = X::add(a0, b0);
            out[base + Ls] = X::add(a1, b1);
            out[base + 2 * Ls] = X::sub(a0, b0);
            out[base + 3 * Ls] = X::sub(a1, b1);
        }
        __syncthreads();
        cplx* tmp = in; in = out; out = tmp;
    }
    if (Ls < M) {   // radix-2 pass, Ls = M / 2
#pragma unroll
        for (int u = 0; u < (M / 2 + T - 1) / T; ++u) {
            const int j = t + u * T;
            if (j >= M / 2) break;
            const int k = j;                       // j < Ls
            const cplx w = wn[(size_t)k * C];
            const cplx x0 = in[j];
            const cplx x1 = INV ? X::mulc(in[j + M / 2], w) : X::mul(in[j + M / 2], w);
            out[k] = X::add(x0, x1);
            out[k + Ls] = X::sub(x0, x1);
        }
        __syncthreads();
        cplx* tmp = in; in = out; out = tmp;
    }
    return in;
}

// Error class of one point from E and E - A1: pct = 100 |E - A1| / (|E| + 1) in
// FP64 (as the FP64 oracle), MEX rule (points with |E| = 0 skipped; >= maxErr,
// else >= minErr) or NEE rule (> maxErr; >= minErr).  Float-float first
// classifies from its FP32 leading parts and recomputes in FP64 only when pct
// lies within 1e-5 (relative) of a threshold, so decisions are FP64's.
template <typename R, bool NEE>
__device__ __forceinline__ int classify_x(typename Num<R>::cplx e, typename Num<R>::cplx d, double maxE,
                                          double minE) {
    double pct, ae;
    if constexpr (sizeof(R) == sizeof(ff) && !std::is_same<R, double>::value) {
        const float ae32 = sqrtf(e.rh * e.rh + e.ih * e.ih);
        const float p32 = 100.f * sqrtf(d.rh * d.rh + d.ih * d.ih) / (ae32 + 1.f);
        const bool near = fabsf(p32 - (float)maxE) <= 1e-5f * (float)maxE ||
                          fabsf(p32 - (float)minE) <= 1e-5f * (float)minE;
        if (!near) {
            pct = (double)p32;
            ae = (double)ae32;
        } else {
            const double2 ed = Num<R>::to_d(e), dd = Num<R>::to_d(d);
            ae = hypot(ed.x, ed.y);
            pct = 100.0 * hypot(dd.x, dd.y) / (ae + 1.0);
        }
    } else {
        const double2 ed = Num<R>::to_d(e), dd = Num<R>::to_d(d);
        ae = hypot(ed.x, ed.y);
        pct = 100.0 * hypot(dd.x, dd.y) / (ae + 1.0);
    }
    int bits = 0;
    if (NEE) {
        if (pct > maxE) bits |= 1;
        if (pct >= minE) bits |= 2;
    } else if (ae > 0.0) {
        if (pct >= maxE) bits |= 1;
        else if (pct >= minE) bits |= 2;
    }
    if (!Num<R>::finite(e)) bits |= 4;
    return bits;
}

// ---------------------------------------------------------------------------
// the kernel
// ---------------------------------------------------------------------------
template <typename R, int M, int C, bool NEE>
__global__ void __launch_bounds__(kXThreads, 1)
passx_kernel(const PulseX* __restrict__ pulses, XTables<R> tabs, KernelCfg cfg) {
    using X = Num<R>;
    using cplx = typename X::cplx;
    using real = typename X::real;
    constexpr int T = kXThreads;
    constexpr int P = M / T;
    constexpr int N = M * C;
    static_assert(P >= 1 && P <= 16 && M % T == 0, "M must be 256..4096");
    using SM = SmemX<R, M>;
    extern __shared__ __align__(16) unsigned char smem[];
    cplx* bufX = reinterpret_cast<cplx*>(smem + SM::off_x);
    cplx* bufK = reinterpret_cast<cplx*>(smem + SM::off_k);
    cplx* Dc = reinterpret_cast<cplx*>(smem + SM::off_d);
    cplx* edge = reinterpret_cast<cplx*>(smem + SM::off_edge);
    cplx* wc = reinterpret_cast<cplx*>(smem + SM::off_wc);
    int* red = reinterpret_cast<int*>(smem + SM::off_red);

    const int t = threadIdx.x;
    const int c = (C > 1) ? (int)cg::this_cluster().block_rank() : 0;
    const int p = blockIdx.x / C;
    __shared__ PulseX sP;
    if (t == 0) sP = pulses[p];
    __syncthreads();
    const PulseX& Pd = sP;
    const cplx* __restrict__ wn = tabs.wn;
    cplx* cph = reinterpret_cast<cplx*>(Pd.cph);

    // ---- prologue: field, carrier phasors, absorber, small-DFT twiddles ----
    for (int i = t; i < 64; i += T) red[i] = 0;
    if (C > 1 && t < C / 2) wc[t] = wn[(size_t)t * (N / C)];
    cplx a[P];
#pragma unroll
    for (int j = 0; j < P; ++j) {
        const int i = c * M + P * t + j;
        a[j] = X::from(Pd.E_in[i]);
        const uint64_t jt = (uint64_t)(long long)time_index(i, N, cfg.time_mode);
        cph[i] = X::from(turn_unit_d(Pd.tau_theta * jt));
        double f = 1.0;
        if (cfg.abc_mode == ABC_NEE) {   // NEE_CPU.m:114-121
            const int it = (i < N / 2) ? i : i - N;
            const double range = (double)(N - 1) * Pd.dt, a2t = fabs(2.0 * (double)it * Pd.dt);
            if (range - a2t < 0.25 * range) {
                const double sh = 1.0 / cosh(24.0 * (1.0 - a2t / range));
                f = 1.0 - sh * sh;
            }
        } else if (cfg.abc_mode != ABC_NONE) {   // OPO_CUDA_BATCH_XTAL.cu:105-137
            const int gi1 = 6 * (N / 16), gi2 = 10 * (N / 16);
            if (i > gi1 && i < gi2) {
                if (cfg.abc_mode == ABC_HARD) f = 0.0;
                else {
                    const double g = cosh((48.0 / (double)N) * fabs((double)i - (double)N / 2.0));
                    f = 1.0 - 1.0 / (g * g);
                }
            }
        }
        Pd.abc[i] = f;
    }
    // z-carrier phasor of every z-sample of the pass, shared by the cluster's CTAs
    // (the FP64 sincospi leaves the per-stage path)
    cplx* ztab = reinterpret_cast<cplx*>(Pd.ztab);
    for (int pz = c * T + t; pz < Pd.zcap; pz += C * T)
        ztab[pz] = X::from(turn_unit_d((uint64_t)0 - Pd.tau_z * (uint64_t)pz));
    if constexpr (C > 1) cg::this_cluster().sync(); else __syncthreads();

    const double h = Pd.h, sel = Pd.sel, Sd = (double)Pd.S, cs = Pd.c_shock;
    const double maxE = Pd.max_err, minE = Pd.min_err;
    const double invN = 1.0 / (double)N;
    const int guard = cfg.guard;
    const long long max_attempts = (long long)cfg.max_attempts_mul * (long long)(Pd.S + 16) + 64;
    const int nchunks = Pd.nchunks;
    const bool rec = (c == 0 && t == 0);

    double k = NEE ? 1.0 : 0.0, stepprev = 4.0, stepmod = 4.0;
    long long q = 0;
    int s_cached = -1;
    int attempt = 0, n_acc = 0, n_rej = 0, status = 0, par = 0;

    // NL drive of this thread's points at z-phasor zz (into nl), then the
    // neighbours' edge values through shared / distributed shared memory
    auto nl_stage = [&](const cplx (&src)[P], cplx zz, cplx (&nl)[P], cplx& L, cplx& Rr) {
#pragma unroll
        for (int j = 0; j < P; ++j) {
            const cplx e = X::mul(cph[c * M + P * t + j], zz);
            const cplx s = src[j];
            const real m2 = X::norm2(s);
            const cplx s2 = X::mul(s, s);
            // A^2 e + 2 |A|^2 conj(e)
            nl[j] = X::add(X::mul(s2, e), X::scale(X::pow2(X::conj(e), 2.0), m2));
        }
        cplx* eg = edge + par * 2 * T;
        eg[2 * t] = nl[0];
        eg[2 * t + 1] = nl[P - 1];
        csync<C>();
        if (t > 0) L = eg[2 * t - 1];
        else L = remote<C>(eg, (c + C - 1) % C)[2 * T - 1];
        if (t < T - 1) Rr = eg[2 * t + 2];
        else Rr = remote<C>(eg, (c + 1) % C)[0];
        par ^= 1;
    };
    // K = -i hG (NL - i cs (NL[+1] - NL[-1]))
    auto k_of = [&](cplx nm, cplx n0, cplx np, real hg, real csr) -> cplx {
        const cplx d = X::sub(np, nm);
        const cplx in = X::sub(n0, X::mul_i(X::scale(d, csr)));
        return X::mul_mi(X::scale(in, hg));
    };

    for (int chunk = 0; chunk < nchunks; ++chunk) {
        if (!NEE) stepmod = stepprev;
        const double cend = (double)(chunk + 1) * sel;
        while (k < cend && (NEE ? k <= Sd : (!guard || k < Sd))) {
            if (attempt >= max_attempts) { status |= OPTIFAX_PULSE_ATTEMPT_LIMIT; goto done; }
            const int kidx = NEE ? (int)k - 1 : (int)k;
            const int krec = (int)k;
            const double kpos = NEE ? k - 1.0 : k;
            bool accepted = false;
            const real hg = X::rfrom((stepmod * h) * Pd.G[kidx]);
            const real csr = X::rfrom(cs);
            int bits = 0;
            {
                cplx nl[P], L, Rr;
                // ---- stage 1: K1 = f(A0) at z = k ----
                auto zphasor = [&](long long pz) -> cplx {
                    return pz < Pd.zcap ? ztab[pz] : X::from(turn_unit_d((uint64_t)0 - Pd.tau_z * (uint64_t)pz));
                };
                cplx z = zphasor((long long)kpos);
                nl_stage(a, z, nl, L, Rr);
                // A1 = A0 + (K1/2 + K1/2) (MEX) or A0 + K1 (NEE_CPU.m:73); K1 kept in
                // shared memory, A1 formed again where it is needed
                auto a1_of = [&](int j) -> cplx {
                    const cplx k1 = bufK[P * t + j];
                    return NEE ? X::add(a[j], k1) : X::add(a[j], X::add(X::pow2(k1, 0.5), X::pow2(k1, 0.5)));
                };
#pragma unroll
                for (int j = 0; j < P; ++j)
                    bufK[P * t + j] = k_of(j == 0 ? L : nl[j - 1], nl[j], j == P - 1 ? Rr : nl[j + 1], hg, csr);
                // ---- stage 2: K2 = f(A1) at z = k + stepmod ----
                z = zphasor((long long)(kpos + stepmod));
                {
                    cplx a1[P];
#pragma unroll
                    for (int j = 0; j < P; ++j) a1[j] = a1_of(j);
                    nl_stage(a1, z, nl, L, Rr);
                }
#pragma unroll
                for (int j = 0; j < P; ++j) {
                    const cplx k2 = k_of(j == 0 ? L : nl[j - 1], nl[j], j == P - 1 ? Rr : nl[j + 1], hg, csr);
                    const cplx k1 = bufK[P * t + j];
                    // E = A0 + (K2/2 + K1/2) (MEX) or (A0 + K1/2) + K2/2 (NEE_CPU.m:75)
                    const cplx e = NEE ? X::add(X::add(a[j], X::pow2(k1, 0.5)), X::pow2(k2, 0.5))
                                       : X::add(a[j], X::add(X::pow2(k2, 0.5), X::pow2(k1, 0.5)));
                    // pct = 100 |E - A1| / (|E| + 1) (OPO_CUDA_BATCH_XTAL.cu:325-349; NEE_CPU.m:73-79)
                    bits |= classify_x<R, NEE>(e, X::sub(e, a1_of(j)), maxE, minE);
                    bufX[P * t + j] = X::scale(e, X::rfrom(Pd.abc[c * M + P * t + j]));
                }
            }
            int fl = reduce_flags<M, C>(bits, red, attempt, t, c, cfg);
            if (Pd.forced && attempt < Pd.n_forced) fl = (Pd.forced[attempt] & 3) | (fl & 4);
            if (fl & 4) status |= OPTIFAX_PULSE_NAN;

            if ((fl & 1) && stepmod > 1.0 && (NEE || (k - stepmod) > 0.0)) {
                if (rec && Pd.trace && attempt < Pd.trace_cap) {
                    Pd.trace[3 * attempt] = krec; Pd.trace[3 * attempt + 1] = (int)stepmod;
                    Pd.trace[3 * attempt + 2] = fl & 7;
                }
                ++n_rej;
                if (!NEE) k = k - stepmod;
                stepmod = stepmod - 1.0;
                stepprev = stepmod;
            } else {
                if (rec && Pd.trace && attempt < Pd.trace_cap) {
                    Pd.trace[3 * attempt] = krec; Pd.trace[3 * attempt + 1] = (int)stepmod;
                    Pd.trace[3 * attempt + 2] = (fl & 7) | 8;
                }
                ++n_acc;
                accepted = true;
                const int s_used = (int)stepmod;
                if (NEE) {
                    if (!(fl & 2)) stepmod = stepmod + 1.0;
                    if (k < Sd && k + stepmod > Sd) stepmod = Sd - k;
                } else if (k + stepmod >= cend && k < cend - 1.0) {
                    const double stepend = (cend - k) - 1.0;
                    stepprev = stepmod;
                    stepmod = stepend;
                } else {
                    if (!(fl & 2) && !(fl & 1) && (k + stepmod + 1.0) < cend - 1.0) stepmod = stepmod + 1.0;
                    stepprev = stepmod;
                }

                // ---- linear sub-step: A0 = IFFT(D FFT(E abc)) / N ----
                if (s_used != s_cached) {
                    // D_k = alpha_k^s exp(-i beta_k s) in FP64 (OPO_CUDA_BATCH_XTAL.cu:255-305)
#pragma unroll 1
                    for (int m = t; m < M; m += T) {
                        const int kk = c + C * m;
                        double sn, cn;
                        sincos(-Pd.beta[kk] * (double)s_used, &sn, &cn);
                        const double al = Pd.alpha[kk];
                        const double af = (al == 1.0) ? 1.0 : pow(al, (double)s_used);
                        Dc[m] = X::from(make_double2(cn * af, sn * af));
                    }
                    s_cached = s_used;
                }
                // forward: C-point DFTs across the cluster (this CTA takes n2 in
                // [c M/C, (c+1) M/C)), gathered from every CTA's E (complete at the
                // flag barrier) and stored into the owners' bufK; the barrier after
                // the stores also ends every gather, so bufX is free for the transform
                cplx* src = bufX;
                cplx* oth = bufK;
                if constexpr (C > 1) {
                    constexpr int PER = M / C;
                    constexpr int NPT = PER >= T ? PER / T : 1;
                    constexpr int LOGC = (C == 2) ? 1 : (C == 4) ? 2 : (C == 8) ? 3 : 4;
                    if (PER >= T || t < PER) {
                        cplx v[NPT][C];
#pragma unroll
                        for (int u = 0; u < NPT; ++u)
#pragma unroll
                            for (int n1 = 0; n1 < C; ++n1) v[u][n1] = remote<C>(bufX, n1)[c * PER + t + u * T];
#pragma unroll
                        for (int u = 0; u < NPT; ++u) {
                            const int n2 = c * PER + t + u * T;
                            dft_small<R, C, false>(v[u], wc);
#pragma unroll
                            for (int r = 0; r < C; ++r) {
                                const int k1 = bitrev(r, LOGC);
                                remote<C>(bufK, k1)[n2] = k1 == 0 ? v[u][r] : X::mul(v[u][r], wn[(size_t)n2 * k1]);
                            }
                        }
                    }
                    cg::this_cluster().sync();
                    src = bufK;
                    oth = bufX;
                } else {
                    __syncthreads();
                }
                cplx* fbuf = stockham<R, M, C, false>(src, oth, wn, t);
                cplx* obuf = (fbuf == bufX) ? bufK : bufX;
#pragma unroll 1
                for (int m = t; m < M; m += T) fbuf[m] = X::mul(fbuf[m], Dc[m]);
                __syncthreads();
                cplx* gbuf = stockham<R, M, C, true>(fbuf, obuf, wn, t);
                cplx* hbuf = (gbuf == bufX) ? bufK : bufX;
                const real sN = X::rfrom(invN);
                if constexpr (C > 1) {
                    // inverse: every CTA's inverse transform is complete at the first
                    // barrier (and nobody reads hbuf any more); gather the n2 slice,
                    // undo the twiddles, inverse C-point DFTs, 1/N, store into the owners' hbuf
                    constexpr int PER = M / C;
                    constexpr int NPT = PER >= T ? PER / T : 1;
                    constexpr int LOGC = (C == 2) ? 1 : (C == 4) ? 2 : (C == 8) ? 3 : 4;
                    cg::this_cluster().sync();
                    if (PER >= T || t < PER) {
                        cplx v[NPT][C];
#pragma unroll
                        for (int u = 0; u < NPT; ++u) {
                            const int n2 = c * PER + t + u * T;
#pragma unroll
                            for (int k1 = 0; k1 < C; ++k1) {
                                const cplx y = remote<C>(gbuf, k1)[n2];
                                v[u][k1] = k1 == 0 ? y : X::mulc(y, wn[(size_t)n2 * k1]);
                            }
                        }
#pragma unroll
                        for (int u = 0; u < NPT; ++u) {
                            const int n2 = c * PER + t + u * T;
                            dft_small<R, C, true>(v[u], wc);
#pragma unroll
                            for (int r = 0; r < C; ++r) remote<C>(hbuf, bitrev(r, LOGC))[n2] = X::scale(v[u][r], sN);
                        }
                    }
                    cg::this_cluster().sync();
#pragma unroll
                    for (int j = 0; j < P; ++j) a[j] = hbuf[P * t + j];
                } else {
#pragma unroll
                    for (int j = 0; j < P; ++j) a[j] = X::scale(gbuf[P * t + j], sN);
                }
                q += s_used;
                __syncthreads();
            }
            ++attempt;
            if (!NEE || accepted) k = k + stepmod;
        }
    }
done:
#pragma unroll
    for (int j = 0; j < P; ++j) Pd.A_out[c * M + P * t + j] = X::to_d(a[j]);
    if (rec && Pd.stats) {
        optifax_pulse_stats st;
        st.attempts = attempt; st.accepted = n_acc; st.rejected = n_rej; st.status = status;
        st.z_steps = q; st.k_final = (float)k; st.stepmod_final = (float)stepmod; st.n_chunks = nchunks;
        st.reserved[0] = 1; st.reserved[1] = st.reserved[2] = 0;
        *Pd.stats = st;
    }
}

}  // namespace ofx
