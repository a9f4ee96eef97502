// ofx_pass.cuh -- the persistent crystal-pass kernel.
//
// One thread-block cluster of C CTAs propagates one pulse of N = C * M points
// through the whole crystal in a single launch.  CTA rank c holds time points
// [c M, (c+1) M) for the nonlinear sub-steps and, after the forward
// transform, the spectral modes k = c + C k2 (k2 = 0..M-1).  Thread t owns
// time points 16t .. 16t+15 of its CTA (held in registers across steps) and
// spectral slots 16t .. 16t+15 (mode k2 = bitrev(slot)).
//
// Per step attempt (reference: OPO_CUDA_BATCH_XTAL.cu:432-506, Heun;
// ode23/OPO_CUDA_ODE23.cu:446-538, RK23):
//   RK stages: NL drive (A^2 e^{i phi} + 2|A|^2 e^{-i phi}, phi = w0 t - bdiffw0 z),
//   shock-term central difference, stage combine -- all in registers, with
//   the +-1 neighbours exchanged through shared memory (and distributed
//   shared memory across the cluster).  Error classification (max-norm,
//   percent) is an OR-reduction over the pulse (or over the batch when the
//   reference's shared schedule is requested).  Accepted steps run the
//   absorber, the forward FFT, the dispersion multiply, the inverse FFT and
//   the 1/N scale without leaving the SM (cluster exchange for C > 1).
//
// Precision: FP32 field and FFT; phases exact in 64-bit fixed point (time
// carrier w0 t, z carrier bdiffw0 z, accumulated dispersion beta z).  The
// linear sub-step is applied as an increment, A_new = E + IFFT((D-1) FFT(E))/N,
// with D - 1 = -2 sin^2(beta s/2) - i sin(beta s) evaluated without
// cancellation, so transform rounding scales with |D - 1| rather than |E|; the
// per-mode phase actually applied is tracked in fixed point and its FP32
// rounding fed back into the next step (no drift of the accumulated phase);
// the inverse FFT applies the exact reciprocal of each forward twiddle.
#pragma once
#include <cooperative_groups.h>
#include "ofx_fft.cuh"
#include "../../include/optifax.h"

namespace cg = cooperative_groups;

namespace ofx {

enum { TIME_SHIFTED = 0, TIME_UNSHIFTED = 1, TIME_NEE = 2 };
enum { ABC_SOFT = 0, ABC_NONE = 1, ABC_HARD = 2, ABC_NEE = 3 };

struct PulseDev {
    const float2* E_in;
    float2* A_out;
    const float* alpha;
    const float* beta;
    const float* G;
    float2* Ap;
    float* stepmods;
    int* trace;
    const int* forced;
    optifax_pulse_stats* stats;
    double bdiffw0, dt;
    uint64_t tau_theta;      // w0 dt in turns (fixed point)
    uint64_t tau_z4;         // bdiffw0 h / 4 in turns (fixed point), per quarter step
    float w0, h, max_err, min_err, sel, c_shock;
    int N, S, nchunks, stepmods_limit, trace_cap, n_forced;
    // synchronously pumped OPO (fb != nullptr): per-mode round-trip transfer
    const float2* fb;        // crystal-output spectrum -> next crystal-input spectrum
    const float2* pump;      // pump spectrum added at the crystal input each trip
    const float* tally_w;    // n_tally x N energy weights on the crystal-output spectrum
    optifax_trip_record* trips;
    int n_trips, n_tally, steady_trips, steady_tally;
    float steady_tol;
    float2* hist;            // optional per-trip crystal-output spectra (n_trips x N)
    const float* esd_w;      // n_esd x N spectral-energy weights (trip sums into esd)
    float* esd;
    int n_esd;
    float* smt;              // optional per-trip stepmods records (n_trips x S)
    float2* xs;              // trip-output scratch (N) for the ESD sums when hist is not given
    // cluster (C > 1) exchange scratch in global memory: 2 N complex
    float2* xch;
};

struct FftTables {
    const Twiddle* tw1;      // pass-1 outer twiddles [16][M/16]: W_M^{off r}
    const Twiddle* tw2;      // pass-2 outer twiddles [16][M/256]: W_{M/16}^{off r}
    // cluster exchange (copied to shared memory): W_N^e = W_M^{(64/C)(e >> 6)} W_N^{e & 63}
    const Twiddle* quad;     // W_M^y, y in [0, M/4)
    const Twiddle* low;      // W_N^i, i in [0, 64)
};

struct KernelCfg {
    int time_mode;
    int abc_mode;
    int guard;           // XTAL/BATCH_OP: ceil chunk count and k < Nsteps loop guard
    int shared_sched;    // 1: OR the error flags over every pulse of the launch (grid barrier)
    int max_attempts_mul;
    int* grid_flags;     // 3 ints (shared schedule only)
};

// Kernel flavours: the MEX Heun and RK23 schedules (OPTIFAX_HEUN, OPTIFAX_RK23) and
// the Heun schedule with NEE_CPU.m step control, a separate instantiation so the
// MEX kernels carry no NEE branches.
constexpr int kHeunNee = 2;

// ---------------------------------------------------------------------------
// pointwise physics
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 nl_eval(float2 a, float2 cph, float2 z) {
    float2 e = cmul(cph, z);
    float ax2 = a.x * a.x, ay2 = a.y * a.y;
    float2 a2 = make_float2(ax2 - ay2, 2.f * a.x * a.y);
    float m2 = 2.f * (ax2 + ay2);
    return make_float2(fmaf(a2.x, e.x, fmaf(-a2.y, e.y, m2 * e.x)),
                       fmaf(a2.x, e.y, fmaf(a2.y, e.x, -m2 * e.y)));
}

// K = -i hG (NL - i cs (NL[+1] - NL[-1]))
__device__ __forceinline__ float2 k_eval(float2 nlm, float2 nl0, float2 nlp, float hg, float cs) {
    float2 d = csub(nlp, nlm);
    float inx = fmaf(cs, d.y, nl0.x);
    float iny = fmaf(-cs, d.x, nl0.y);
    return make_float2(hg * iny, -hg * inx);
}

__device__ __forceinline__ int time_index(int i, int n, int mode) {
    if (mode == TIME_SHIFTED) return (i > n / 2) ? i - n / 2 : i + n / 2;
    if (mode == TIME_NEE) return (i < n / 2) ? i : i - n;      // fftshift(t), NEE_CPU.m:12,53
    return i;
}

__device__ __forceinline__ float abc_factor(int i, int n, int mode) {
    if (mode == ABC_NONE) return 1.f;
    if (mode == ABC_NEE) {
        // NEE_CPU.m:114-121: 1 - sech^2(24 (1 - |2t| / range(t))) where
        // range(t) - |2t| < range(t) / 4, range(t) = (n - 1) dt, t = fftshift(t)
        const int it = (i < n / 2) ? i : i - n;
        const float r = 1.f - 2.f * fabsf((float)it) / (float)(n - 1);
        if (!(r < 0.25f)) return 1.f;
        const float th = tanhf(24.f * r);
        return th * th;
    }
    int gi1 = 6 * (n / 16), gi2 = 10 * (n / 16);
    if (!(i > gi1 && i < gi2)) return 1.f;
    if (mode == ABC_HARD) return 0.f;
    // 1 - sech^2(pos) evaluated as tanh^2(pos): no cancellation near the window edge
    float pos = (48.f * fabsf((float)i - 0.5f * (float)n)) / (float)n;
    float th = tanhf(pos);
    return th * th;
}

// Error class of one point: pct = scale |d| / (|e| + 1) against the percent
// thresholds (OPO_CUDA_BATCH_XTAL.cu:325-349; points with |e| == 0 skipped).
// Compared in squares so only |e| needs a square root.
__device__ __forceinline__ int classify(float scale, float2 d, float2 e, float maxE, float minE) {
    float e2 = e.x * e.x + e.y * e.y;
    int bits = 0;
    if (e2 > 0.f) {
        float den = sqrtf(e2) + 1.f;
        float lhs = scale * scale * (d.x * d.x + d.y * d.y);
        float hi = maxE * den, lo = minE * den;
        if (maxE <= 0.f || lhs >= hi * hi) bits = 1;
        else if (minE <= 0.f || lhs >= lo * lo) bits = 2;
    }
    if (!(isfinite(e.x) && isfinite(e.y))) bits |= 4;
    return bits;
}

// NEE_CPU.m:73-79 class: pct = scale |d| / (|e| + 1) over every point; bit 0
// when pct > maxErr (strict), bit 1 when pct >= minErr.
__device__ __forceinline__ int classify_nee(float scale, float2 d, float2 e, float maxE, float minE) {
    const float den = sqrtf(e.x * e.x + e.y * e.y) + 1.f;
    const float lhs = scale * scale * (d.x * d.x + d.y * d.y);
    const float hi = maxE * den, lo = minE * den;
    int bits = 0;
    if (lhs > hi * hi) bits |= 1;
    if (lhs >= lo * lo) bits |= 2;
    if (!(isfinite(e.x) && isfinite(e.y))) bits |= 4;
    return bits;
}

// D - 1 = alpha^s exp(-i th) - 1 for the phase increment d32 (units of 2^-32
// turn; converted to FP32, *dapplied receives the integer actually used) and
// log2 alpha l2 (-inf: alpha = 0).
__device__ __forceinline__ float2 dispersion_dm1(int d32, float l2, int s, int* dapplied) {
    if (l2 == -INFINITY) { *dapplied = d32; return make_float2(-1.f, 0.f); }
    float df = (float)d32;
    if (df >= 2147483648.f) df = 2147483520.f;
    *dapplied = __float2int_rn(df);
    float th = df * 1.4629180792671596e-09f;   // radians (2 pi 2^-32 per unit)
    float2 dm1;
    if (fabsf(th) < 0.25f) {
        // exp(-i th) - 1 by its Taylor series (no cancellation)
        float t2 = th * th;
        float cm1 = t2 * fmaf(t2, fmaf(t2, fmaf(t2, 2.48015873e-05f, -1.38888889e-03f), 4.16666667e-02f), -0.5f);
        float sn = th * fmaf(t2, fmaf(t2, fmaf(t2, -1.98412698e-04f, 8.33333333e-03f), -1.66666667e-01f), 1.f);
        dm1 = make_float2(cm1, -sn);
    } else {
        float s2, c2;
        sincospif(df * 0x1p-32f, &s2, &c2);   // sin, cos of th/2
        dm1 = make_float2(-2.f * s2 * s2, -2.f * s2 * c2);
    }
    if (l2 != 0.f) {
        float x = (float)s * l2;
        float as = exp2f(x);
        float am1 = expm1f(x * 0.69314718055994531f);
        dm1 = make_float2(fmaf(dm1.x, as, am1), dm1.y * as);
    }
    return dm1;
}

// 16-byte stores of consecutive complex pairs to global memory (L2 only)
__device__ __forceinline__ void store_pair(float2* base, int j, float2 v, float2& prev) {
    if (j & 1) __stcg(reinterpret_cast<float4*>(base) + (j >> 1), make_float4(prev.x, prev.y, v.x, v.y));
    else prev = v;
}

__device__ __forceinline__ float2 zphase(uint64_t tau_z4, float pos) {
    uint64_t p4 = (uint64_t)(uint32_t)(4.0f * pos);
    return turn_to_unit((uint64_t)0 - tau_z4 * p4);
}

// ---------------------------------------------------------------------------
// shared-memory layout
// ---------------------------------------------------------------------------
template <int M, int METHOD, int C>
struct Smem {
    static constexpr int T = M / 16;
    static constexpr int PADM = M + M / 16;
    static constexpr int NBUF = (METHOD == OPTIFAX_RK23) ? 3 : 2;   // E, X (+K1 for RK23)
    static constexpr size_t off_buf = 0;
    static constexpr size_t off_tau = off_buf + sizeof(float2) * PADM * NBUF;
    static constexpr size_t off_l2a = off_tau + sizeof(uint64_t) * M;
    static constexpr size_t off_papp = off_l2a + sizeof(float) * M;
    static constexpr size_t off_abc = off_papp + sizeof(uint32_t) * M;
    // Heun: per-mode D - 1 and its fixed-point phase increment for the cached stepmod
    static constexpr int NCACHE = (METHOD != OPTIFAX_RK23) ? M : 0;
    static constexpr size_t off_dmc = off_abc + sizeof(float) * M;
    static constexpr size_t off_dfc = off_dmc + sizeof(float2) * NCACHE;
    static constexpr size_t off_edge = off_dfc + sizeof(int) * NCACHE;
    static constexpr size_t off_red = off_edge + sizeof(float2) * 4 * T;
    static constexpr size_t off_dred = off_red + 256;               // FP64 reduction slots
    // exchange twiddle tables (16-byte entries, clusters only): quarter-period W_M,
    // W_N^i for i < 64
    static constexpr size_t off_quad = (off_dred + sizeof(double) * (8 * 4 + 2 * 16 * 4 + 4) + 15) & ~size_t(15);
    static constexpr size_t off_low = off_quad + (C > 1 ? sizeof(Twiddle) * (M / 4) : 0);
    static constexpr size_t bytes = off_low + (C > 1 ? sizeof(Twiddle) * 64 : 0);
};

// ---------------------------------------------------------------------------
// cluster helpers
// ---------------------------------------------------------------------------
template <int C>
__device__ __forceinline__ void csync() {
    if constexpr (C > 1) cg::this_cluster().sync();
    else __syncthreads();
}

template <int C, typename Tp>
__device__ __forceinline__ Tp* remote(Tp* p, int rank) {
    if constexpr (C > 1) return cg::this_cluster().map_shared_rank(p, rank);
    else return p;
}

// 32-bit shared::cluster addressing: `mapa` turns a local shared address into the
// same offset in CTA `rank` of the cluster (half the registers of generic pointers;
// clusters of up to 4 -- with 8 the generic stores measured faster)
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint32_t cluster_addr(uint32_t local, int rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
    return r;
}
__device__ __forceinline__ float2 ld_cluster_f2(uint32_t addr) {
    float2 v;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr) : "memory");
    return v;
}
__device__ __forceinline__ void st_cluster_f2(uint32_t addr, float2 v) {
    asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(addr), "f"(v.x), "f"(v.y) : "memory");
}

// Publish this thread's first/last stencil values and fetch the neighbours'.
template <int M, int C>
__device__ __forceinline__ void exchange_edges(float2* edge, int& par, int t, int c, float2 first,
                                               float2 last, float2& left, float2& right) {
    constexpr int T = M / 16;
    float2* e = edge + par * 2 * T;
    e[2 * t] = first;
    e[2 * t + 1] = last;
    csync<C>();
    if (t > 0) left = e[2 * t - 1];
    else left = remote<C>(e, (c + C - 1) % C)[2 * T - 1];
    if (t < T - 1) right = e[2 * t + 2];
    else right = remote<C>(e, (c + 1) % C)[0];
    par ^= 1;
}

// N-point twiddle W_N^e, 0 <= e < N = C M, from the two shared-memory tables:
// W_M^{(64/C)(e >> 6)} (quarter table, exact) times W_N^{e & 63}.  The product is
// rounded once; the inverse multiplies by its exact reciprocal conj(w)(1 + d),
// d = 1/|w|^2 - 1 formed from w itself, so forward + inverse carry no gain.
template <int M, int C>
__device__ __forceinline__ float2 twn_val(const Twiddle* quad, const Twiddle* low, int e) {
    static_assert(64 % C == 0, "cluster size must divide 64");
    const Twiddle a = quad_tw<M>(quad, (64 / C) * (e >> 6));
    const Twiddle b = low[e & 63];
    return cmul(make_float2(a.c, a.s), make_float2(b.c, b.s));
}
template <int M, int C>
__device__ __forceinline__ float2 twn_fwd(float2 v, const Twiddle* quad, const Twiddle* low, int e) {
    return cmul(v, twn_val<M, C>(quad, low, e));
}
template <int M, int C>
__device__ __forceinline__ float2 twn_inv(float2 v, const Twiddle* quad, const Twiddle* low, int e) {
    const float2 w = twn_val<M, C>(quad, low, e);
    const float2 t = cmulc(v, w);
    const float d = inv_norm2_m1(w);
    return make_float2(fmaf(t.x, d, t.x), fmaf(t.y, d, t.y));
}

// Exchange results go straight into their owners' shared memory for clusters of
// up to 8 CTAs; 16-CTA clusters keep them in global memory (L2), where their
// wider fan-out measured faster (and the kernel stays free of spills).
template <int C>
constexpr bool kPushExchange = (C <= 8);
// The forward gather reads the C blocks' stage outputs straight from their CTAs'
// shared memory (ld.shared::cluster) for clusters of up to 4; larger clusters
// gather them from global memory (measured: 4 CTAs 13.9 -> 13.6 us per attempt,
// 8 CTAs 14.9 -> 15.0).
template <int C>
constexpr bool kPullGather = (C <= 4);

// Four-step split of the N = C M transform: forward step 1 (C-point DFTs over
// CTAs, twiddle W_N^{n2 k1}).  Each CTA gathers its n2 slice of the C blocks --
// from the blocks' stage outputs in their CTAs' shared memory (`bufe`, clusters
// of up to 4) or from global memory (`xx`, all loads in flight) -- computes the
// C-point DFTs and stores the results in their owners' shared memory (`buf`, the
// owner's FFT buffer, at phys(n2)) or, for 16-CTA clusters, in their blocks of
// `yy` (global).  Ordering comes from the cluster barriers around the calls
// (release/acquire at cluster scope covers global and distributed shared memory):
// the stage outputs are complete at the error-flag barrier before the call, and no
// CTA reads its FFT buffer again until the barrier after it.  Global accesses
// bypass L1.
template <int M, int C>
__device__ __forceinline__ void exchange_forward_g(const float2* __restrict__ xx, const float2* bufe,
                                                   float2* buf, float2* yy,
                                                   const Twiddle* quad, const Twiddle* low, int t, int c) {
    if constexpr (C > 1) {
        constexpr int T = M / 16, PER = 16 / C, LOGC = (C == 2) ? 1 : (C == 4) ? 2 : (C == 8) ? 3 : 4;
        float2 v[PER][C];
#pragma unroll
        for (int u = 0; u < PER; ++u)          // every load in flight before any use
#pragma unroll
            for (int n1 = 0; n1 < C; ++n1) {
                if constexpr (kPullGather<C>)
                    v[u][n1] = ld_cluster_f2(cluster_addr(smem_u32(bufe + phys(c * (M / C) + t + T * u)), n1));
                else v[u][n1] = __ldcg(xx + n1 * M + c * (M / C) + t + T * u);
            }
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            int n2 = c * (M / C) + t + T * u;
            dft_dif<C>(v[u]);
#pragma unroll
            for (int r = 0; r < C; ++r) {
                int k1 = bitrev(r, LOGC);
                const float2 y = k1 == 0 ? v[u][r] : twn_fwd<M, C>(v[u][r], quad, low, n2 * k1);
                if constexpr (kPullGather<C>) st_cluster_f2(cluster_addr(smem_u32(buf + phys(n2)), k1), y);
                else if constexpr (kPushExchange<C>) remote<C>(buf, k1)[phys(n2)] = y;
                else __stcg(yy + k1 * M + n2, y);
            }
        }
    }
}

// Inverse step: gather the n2 slice of the C inverse-transformed blocks from
// global memory, undo the twiddles, C-point inverse DFTs, scale by 1/N and store
// each result in its owner's shared memory (`buf` at phys(n2)) or, for 16-CTA
// clusters, in its block of `xx` (global).
template <int M, int C>
__device__ __forceinline__ void exchange_inverse_g(const float2* __restrict__ yy, float2* buf, float2* xx,
                                                   const Twiddle* quad, const Twiddle* low, int t, int c,
                                                   float invN) {
    if constexpr (C > 1) {
        constexpr int T = M / 16, PER = 16 / C, LOGC = (C == 2) ? 1 : (C == 4) ? 2 : (C == 8) ? 3 : 4;
        float2 v[PER][C];
#pragma unroll
        for (int u = 0; u < PER; ++u)          // every load in flight before any use
#pragma unroll
            for (int r = 0; r < C; ++r) v[u][r] = __ldcg(yy + bitrev(r, LOGC) * M + c * (M / C) + t + T * u);
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            int n2 = c * (M / C) + t + T * u;
#pragma unroll
            for (int r = 1; r < C; ++r) v[u][r] = twn_inv<M, C>(v[u][r], quad, low, n2 * bitrev(r, LOGC));
            dft_dit_inv<C>(v[u]);
#pragma unroll
            for (int n1 = 0; n1 < C; ++n1) {
                if constexpr (kPullGather<C>)
                    st_cluster_f2(cluster_addr(smem_u32(buf + phys(n2)), n1), cscale(v[u][n1], invN));
                else if constexpr (kPushExchange<C>) remote<C>(buf, n1)[phys(n2)] = cscale(v[u][n1], invN);
                else __stcg(xx + n1 * M + n2, cscale(v[u][n1], invN));
            }
        }
    }
}

// OR of per-thread flag bits over the CTA, the cluster and (shared schedule)
// the grid.  red[0..2] CTA slots (triple buffered by attempt), red[4..4+2*16)
// cluster slots (double buffered).
template <int M, int C>
__device__ __forceinline__ int reduce_flags(int bits, int* red, int attempt, int t, int c,
                                            const KernelCfg& cfg) {
    int w = __reduce_or_sync(0xffffffffu, bits);
    int slot = attempt % 3;
    if ((t & 31) == 0 && w) atomicOr(&red[slot], w);
    __syncthreads();
    int f = red[slot];
    if constexpr (C > 1) {
        int* cl = red + 4 + (attempt & 1) * 16;
        if (t == 0) {
#pragma unroll 1
            for (int r = 0; r < C; ++r) remote<C>(cl, r)[c] = f;
        }
        cg::this_cluster().sync();
        f = 0;
#pragma unroll 1
        for (int r = 0; r < C; ++r) f |= cl[r];
    }
    if (cfg.shared_sched) {
        int gslot = attempt % 3;
        if (t == 0 && c == 0 && f) atomicOr(&cfg.grid_flags[gslot], f);
        cg::this_grid().sync();
        f = *((volatile int*)&cfg.grid_flags[gslot]);
        if (blockIdx.x == 0 && t == 0) cfg.grid_flags[(attempt + 2) % 3] = 0;
    }
    if (t == 0) red[(attempt + 2) % 3] = 0;
    return f;
}

// ---------------------------------------------------------------------------
// FP64 sum of 4 per-thread values over the CTA and the cluster; every thread
// of every CTA returns the same totals (ranks summed in a fixed order).
// ---------------------------------------------------------------------------
template <int M, int C>
__device__ __forceinline__ void reduce_tallies(const float (&part)[4], double (&out)[4], double* dred,
                                               int t, int c, int parity) {
    constexpr int T = M / 16, NW = T / 32;
    double v[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        v[i] = (double)part[i];
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
    }
    if ((t & 31) == 0) {
#pragma unroll
        for (int i = 0; i < 4; ++i) dred[(t >> 5) * 4 + i] = v[i];
    }
    __syncthreads();
    double* cl = dred + 8 * 4 + parity * 16 * 4;
    if (t == 0) {
        double s[4] = {0, 0, 0, 0};
        for (int w = 0; w < NW; ++w)
            for (int i = 0; i < 4; ++i) s[i] += dred[w * 4 + i];
        for (int r = 0; r < C; ++r) {
            double* dst = remote<C>(cl, r) + c * 4;
            for (int i = 0; i < 4; ++i) dst[i] = s[i];
        }
    }
    csync<C>();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        double s = 0.0;
        for (int r = 0; r < C; ++r) s += cl[r * 4 + i];
        out[i] = s;
    }
}

// ---------------------------------------------------------------------------
// the kernel
// ---------------------------------------------------------------------------
// One launch runs n_trips crystal passes of every pulse.  With a round-trip
// transfer (OPO mode, reference OpticalSim.run, OpticalSim.m:230-288) the last
// accepted step of each pass maps its spectrum X through the cavity,
// Y = X fb + pump, and the next pass starts from IFFT(Y): refraction into
// and out of the crystal, the intracavity optics, the output coupler, the
// delay and the pump injection are all per-mode products folded into fb and
// pump by the host.  Per-trip energy tallies sum tally_w |X|^2 in FP64.
template <int M, int C, int METHOD>
__global__ void __launch_bounds__(M / 16, 1)
pass_kernel(const PulseDev* __restrict__ pulses, FftTables tabs, KernelCfg cfg) {
    constexpr int T = M / 16;
    constexpr int N = M * C;
    constexpr int LOG2M = FftShape<M>::LOG2M;
    using SM = Smem<M, METHOD, C>;
    extern __shared__ __align__(16) unsigned char smem[];
    float2* bufE = reinterpret_cast<float2*>(smem + SM::off_buf);
    float2* bufX = bufE + SM::PADM;
    float2* bufK = bufX + SM::PADM;   // RK23 only: FSAL K1 (own points)
    uint64_t* tau_s = reinterpret_cast<uint64_t*>(smem + SM::off_tau);
    float* l2a_s = reinterpret_cast<float*>(smem + SM::off_l2a);
    uint32_t* papp_s = reinterpret_cast<uint32_t*>(smem + SM::off_papp);
    float* abc_s = reinterpret_cast<float*>(smem + SM::off_abc);
    float2* dmc_s = reinterpret_cast<float2*>(smem + SM::off_dmc);
    int* dfc_s = reinterpret_cast<int*>(smem + SM::off_dfc);
    const Twiddle* __restrict__ tw1 = tabs.tw1;
    const Twiddle* __restrict__ tw2 = tabs.tw2;
    Twiddle* quad_s = reinterpret_cast<Twiddle*>(smem + SM::off_quad);
    Twiddle* low_s = reinterpret_cast<Twiddle*>(smem + SM::off_low);
    float2* edge = reinterpret_cast<float2*>(smem + SM::off_edge);
    int* red = reinterpret_cast<int*>(smem + SM::off_red);
    double* dred = reinterpret_cast<double*>(smem + SM::off_dred);

    const int t = threadIdx.x;
    const int c = (C > 1) ? (int)cg::this_cluster().block_rank() : 0;
    const int p = blockIdx.x / C;
    // The descriptor is read all through the loop; a shared-memory copy keeps
    // those reads off the global path (and out of reach of aliasing with the
    // kernel's global stores).
    __shared__ PulseDev sP;
    if (t == 0) sP = pulses[p];
    __syncthreads();
    const PulseDev& P = sP;

    // ---- prologue -------------------------------------------------------
    for (int i = t; i < 64; i += T) red[i] = 0;
    if constexpr (C > 1) {
        for (int i = t; i < M / 4; i += T) quad_s[i] = tabs.quad[i];
        for (int i = t; i < 64; i += T) low_s[i] = tabs.low[i];
    }
    float2 cph[16], a[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        int i = c * M + 16 * t + j;
        uint64_t jt = (uint64_t)time_index(i, N, cfg.time_mode);
        cph[j] = turn_to_unit(P.tau_theta * jt);
        a[j] = P.E_in[i];
        abc_s[j * T + t] = abc_factor(i, N, cfg.abc_mode);
    }
#pragma unroll 1
    for (int j = 0; j < 16; ++j) {
        int slot = 16 * t + j;
        int k = c + C * bitrev(slot, LOG2M);
        double b = (double)P.beta[k];
        constexpr double kTwoPi = 6.283185307179586476925286766559;
        constexpr double kTurnScale = 18446744073709551616.0 / kTwoPi;   // 2^64 / (2 pi)
        double r = b - kTwoPi * rint(b / kTwoPi);
        double x = r * kTurnScale;
        if (x >= 9.2233720368547758e18) x -= 1.8446744073709552e19;
        if (x < -9.2233720368547758e18) x += 1.8446744073709552e19;
        tau_s[j * T + t] = (uint64_t)(long long)llrint(x);
        l2a_s[j * T + t] = log2f(P.alpha[k]);
    }
    if constexpr (C > 1) cg::this_cluster().sync(); else __syncthreads();

    const float* G = P.G;
    const float h = P.h, sel = P.sel, cs = P.c_shock, Sf = (float)P.S;
    const float maxE = P.max_err, minE = P.min_err;
    const float invN = 1.0f / (float)N;
    const int guard = cfg.guard;
    const long long max_attempts = (long long)cfg.max_attempts_mul * (long long)(P.S + 16) + 64;
    const int nchunks = P.nchunks;
    const float pass_end = (float)nchunks * sel;
    const bool opo = P.fb != nullptr;
    const int n_trips = P.n_trips > 0 ? P.n_trips : 1;
    const bool rec = (c == 0 && t == 0);

    constexpr bool nee = (METHOD == kHeunNee);   // NEE_CPU.m: k is 1-based, no chunk clamp
    constexpr bool heun = (METHOD != OPTIFAX_RK23);
    float k = nee ? 1.f : 0.f, stepprev = 4.f, stepmod = 4.f;
    unsigned q = 0;                          // accumulated dispersion position (sum of stepmod)
    int s_cached = -1;                       // stepmod of the cached per-mode D - 1 (Heun)
    int attempt = 0, n_acc = 0, n_rej = 0, status = 0, par = 0, trip = 0, trips_done = 0;
    int gatt = 0, tot_att = 0, tot_acc = 0, tot_rej = 0, steady_count = 0;
    double prev_tally = 0.0;

    float2 k1r[16];   // RK23: K1 (first stage, FSAL) between attempts
    for (trip = 0; trip < n_trips; ++trip) {
        k = nee ? 1.f : 0.f; stepprev = 4.f; stepmod = 4.f; q = 0;
        attempt = 0; n_acc = 0; n_rej = 0;
        int trip_status = 0;
        double tally[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll 1
        for (int j = 0; j < 16; ++j) papp_s[j * T + t] = 0;
        if constexpr (METHOD == OPTIFAX_RK23) {
            // initial K1 at k = 0 with stepmod = 4 (OPO_CUDA_ODE23.cu:432-438)
            float hg = (stepmod * h) * G[0];
            float2 z = zphase(P.tau_z4, 0.f);
            float2 nl[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) nl[j] = nl_eval(a[j], cph[j], z);
            float2 L, R;
            exchange_edges<M, C>(edge, par, t, c, nl[0], nl[15], L, R);
#pragma unroll
            for (int j = 0; j < 16; ++j)
                k1r[j] = k_eval(j == 0 ? L : nl[j - 1], nl[j], j == 15 ? R : nl[j + 1], hg, cs);
        }

        for (int chunk = 0; chunk < nchunks; ++chunk) {
            if (!nee) stepmod = stepprev;
            const float cend = (float)(chunk + 1) * sel;
            while (k < cend && (nee ? k <= Sf : (!guard || k < Sf))) {
                if (attempt >= max_attempts) { status |= OPTIFAX_PULSE_ATTEMPT_LIMIT; goto done; }
                const int kidx = nee ? (int)k - 1 : (int)k;   // G33(k) is 1-based in NEE_CPU.m
                const int krec = (int)k;
                const float kpos = nee ? k - 1.f : k;          // z of the first stage, in steps
                bool accepted = false;
                const float hmod = stepmod * h;
                const float hg = hmod * G[kidx];
                int bits = 0;
                if constexpr (heun) {
                    // ---- stage 1: K1 = f(A0) at z = k ----
                    float2 nl[16], k1[16], L, R;
                    float2 z = zphase(P.tau_z4, kpos);
#pragma unroll
                    for (int j = 0; j < 16; ++j) nl[j] = nl_eval(a[j], cph[j], z);
                    exchange_edges<M, C>(edge, par, t, c, nl[0], nl[15], L, R);
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        k1[j] = k_eval(j == 0 ? L : nl[j - 1], nl[j], j == 15 ? R : nl[j + 1], hg, cs);
                    // ---- stage 2: K2 = f(A0 + K1) at z = k + stepmod ----
                    z = zphase(P.tau_z4, kpos + stepmod);
#pragma unroll
                    for (int j = 0; j < 16; ++j) nl[j] = nl_eval(cadd(a[j], k1[j]), cph[j], z);
                    exchange_edges<M, C>(edge, par, t, c, nl[0], nl[15], L, R);
                    float2 prev;
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        float2 k2 = k_eval(j == 0 ? L : nl[j - 1], nl[j], j == 15 ? R : nl[j + 1], hg, cs);
                        // E = A0 + (K2/2 + K1/2) (MEX) or (A0 + K1/2) + K2/2 (NEE_CPU.m:75)
                        float2 e = nee ? cadd(cadd(a[j], cscale(k1[j], 0.5f)), cscale(k2, 0.5f))
                                       : cadd(a[j], cadd(cscale(k2, 0.5f), cscale(k1[j], 0.5f)));
                        float2 d = csub(k2, k1[j]);                        // = 2 (E - A1)
                        bits |= nee ? classify_nee(50.f, d, e, maxE, minE) : classify(50.f, d, e, maxE, minE);
                        float2 ea = cscale(e, abc_s[j * T + t]);
                        bufE[phys(16 * t + j)] = ea;
                        if constexpr (C == 1) bufX[phys(16 * t + j)] = ea;
                        else if constexpr (!kPullGather<C>) store_pair(P.xch + c * M + 16 * t, j, ea, prev);
                    }
                } else {
                    // ---- RK23: K2 at k + s/2, K3 at k + 3s/4, K4 at k + s (FSAL) ----
                    float2 nl[16], k2[16], pp[16], L, R;
                    float2 z = zphase(P.tau_z4, k + 0.5f * stepmod);
#pragma unroll
                    for (int j = 0; j < 16; ++j) nl[j] = nl_eval(cadd(a[j], cscale(k1r[j], 0.5f)), cph[j], z);
                    exchange_edges<M, C>(edge, par, t, c, nl[0], nl[15], L, R);
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        k2[j] = k_eval(j == 0 ? L : nl[j - 1], nl[j], j == 15 ? R : nl[j + 1], hg, cs);
                    z = zphase(P.tau_z4, k + 0.75f * stepmod);
#pragma unroll
                    for (int j = 0; j < 16; ++j) nl[j] = nl_eval(cadd(a[j], cscale(k2[j], 0.75f)), cph[j], z);
                    exchange_edges<M, C>(edge, par, t, c, nl[0], nl[15], L, R);
                    float2 ev[16];
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        float2 k3 = k_eval(j == 0 ? L : nl[j - 1], nl[j], j == 15 ? R : nl[j + 1], hg, cs);
                        float2 e = cadd(a[j], cadd(cscale(k3, 4.f / 9.f), cscale(k2[j], 1.f / 3.f)));
                        ev[j] = cadd(e, cscale(k1r[j], 2.f / 9.f));
                        // E - A1 without K4: (4/9-1/3) K3 + (1/3-1/4) K2 + (2/9-7/24) K1
                        pp[j] = cadd(cadd(cscale(k3, 1.f / 9.f), cscale(k2[j], 1.f / 12.f)),
                                     cscale(k1r[j], -5.f / 72.f));
                    }
                    z = zphase(P.tau_z4, k + stepmod);
#pragma unroll
                    for (int j = 0; j < 16; ++j) nl[j] = nl_eval(ev[j], cph[j], z);
                    exchange_edges<M, C>(edge, par, t, c, nl[0], nl[15], L, R);
                    float2 prev;
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        float2 k4 = k_eval(j == 0 ? L : nl[j - 1], nl[j], j == 15 ? R : nl[j + 1], hg, cs);
                        float2 d = csub(pp[j], cscale(k4, 1.f / 8.f));  // = E - A1
                        bits |= classify(200.f, d, ev[j], maxE, minE);
                        float2 ea = cscale(ev[j], abc_s[j * T + t]);
                        bufE[phys(16 * t + j)] = ea;
                        if constexpr (C == 1) bufX[phys(16 * t + j)] = ea;
                        else if constexpr (!kPullGather<C>) store_pair(P.xch + c * M + 16 * t, j, ea, prev);
                        bufK[phys(16 * t + j)] = k4;   // FSAL candidate (own points)
                    }
                }

                int fl = reduce_flags<M, C>(bits, red, gatt, t, c, cfg);
                if (P.forced && gatt < P.n_forced) fl = (P.forced[gatt] & 3) | (fl & 4);
                if (fl & 4) trip_status |= OPTIFAX_PULSE_NAN;

                if ((fl & 1) && stepmod > 1.f && (nee || (k - stepmod) > 0.f)) {
                    // ---- reject: A0 unchanged; MEX: k moves back by one in net (the loop
                    // adds the new stepmod); NEE: k stays (NEE_CPU.m:68-70)
                    if (rec && P.trace && gatt < P.trace_cap) {
                        P.trace[3 * gatt] = krec; P.trace[3 * gatt + 1] = (int)stepmod;
                        P.trace[3 * gatt + 2] = fl & 7;
                    }
                    ++n_rej;
                    if (!nee) k = k - stepmod;
                    stepmod = stepmod - 1.f;
                    stepprev = stepmod;
                    if constexpr (METHOD == OPTIFAX_RK23) {
                        // K1 recomputed at z = k + stepmod with G[k] (OPO_CUDA_ODE23.cu:484-487)
                        float hg1 = (stepmod * h) * G[(int)k];
                        float2 z = zphase(P.tau_z4, k + stepmod);
                        float2 nl[16], L, R;
#pragma unroll
                        for (int j = 0; j < 16; ++j) nl[j] = nl_eval(a[j], cph[j], z);
                        exchange_edges<M, C>(edge, par, t, c, nl[0], nl[15], L, R);
#pragma unroll
                        for (int j = 0; j < 16; ++j)
                            k1r[j] = k_eval(j == 0 ? L : nl[j - 1], nl[j], j == 15 ? R : nl[j + 1], hg1, cs);
                    }
                } else {
                    // ---- accept ----
                    if (rec && P.trace && gatt < P.trace_cap) {
                        P.trace[3 * gatt] = krec; P.trace[3 * gatt + 1] = (int)stepmod;
                        P.trace[3 * gatt + 2] = (fl & 7) | 8;
                    }
                    ++n_acc;
                    accepted = true;
                    const int s_used = (int)stepmod;
                    if (!nee && rec && P.stepmods && kidx < P.stepmods_limit && kidx < P.S)
                        P.stepmods[kidx] = (float)s_used;
                    if (!nee && rec && P.smt && kidx < P.stepmods_limit && kidx < P.S)
                        P.smt[(size_t)trip * P.S + kidx] = (float)s_used;
                    // step control (OPO_CUDA_BATCH_XTAL.cu:487-506; ODE23 :519-538 doubles;
                    // NEE_CPU.m:77-83: grow below minErr, clamp only at the crystal end)
                    if (nee) {
                        if (!(fl & 2)) stepmod = stepmod + 1.f;
                        if (k < Sf && k + stepmod > Sf) stepmod = Sf - k;
                    } else if (k + stepmod >= cend && k < cend - 1.f) {
                        float stepend = (cend - k) - 1.f;
                        stepprev = stepmod;
                        stepmod = stepend;
                    } else {
                        if constexpr (heun) {
                            if (!(fl & 2) && !(fl & 1) && (k + stepmod + 1.f) < cend - 1.f) stepmod = stepmod + 1.f;
                        } else {
                            if (!(fl & 2) && !(fl & 1) && (k + stepmod + stepmod) < cend - 1.f) stepmod = stepmod * 2.f;
                        }
                        stepprev = stepmod;
                    }
                    const float knext = k + stepmod;
                    const bool last_in_chunk = !(knext < cend && (nee ? knext <= Sf : (!guard || knext < Sf)));
                    const bool pass_ends = !(knext < pass_end && (nee ? knext <= Sf : (!guard || knext < Sf)));
                    const bool cav = opo && pass_ends;
                    const unsigned qn = q + (unsigned)s_used;

                    // ---- linear sub-step ----
                    // Incremental form: A_new = E + IFFT((D - 1) FFT(E)) / N with
                    // D = alpha^s exp(-i beta s): transform rounding then scales with
                    // |D - 1| instead of |E|.  At the end of an OPO pass the full
                    // spectrum goes through the cavity instead: A_new = IFFT(D FFT(E) fb + pump) / N.
                    // clusters: the exchanged block lands in bufX (the FFT buffer; bufE keeps E),
                    // or in ybuf (global) for 16-CTA clusters
                    float2* fbuf = (C > 1) ? bufX : bufE;
                    float2* ybuf = (C > 1) ? P.xch + N + c * M : nullptr;
                    if constexpr (C > 1) {
                        exchange_forward_g<M, C>(P.xch, bufE, bufX, P.xch + N, quad_s, low_s, t, c);
                        cg::this_cluster().sync();
                    } else {
                        __syncthreads();
                    }
                    if constexpr (heun) {
                        // refresh the per-mode D - 1 cache when the step size changed (a
                        // compact loop: kept out of the unrolled mode loop below)
                        if (s_used != s_cached) {
#pragma unroll 1
                            for (int j = 0; j < 16; ++j) {
                                const int idx = j * T + t;
                                int dc;
                                const uint64_t inc = tau_s[idx] * (uint64_t)(unsigned)s_used;
                                dmc_s[idx] = dispersion_dm1((int)((long long)inc >> 32), l2a_s[idx], s_used, &dc);
                                dfc_s[idx] = dc;
                            }
                        }
                    }
                    float2 v[16];
                    fft_forward_to_regs<M>(fbuf, tw1, tw2, t, v, kPushExchange<C> ? nullptr : ybuf);
                    float2* apc = (last_in_chunk && P.Ap) ? P.Ap + (size_t)chunk * N : nullptr;
                    float part[4] = {0.f, 0.f, 0.f, 0.f};
                    // the trip's crystal output goes to the cavity scratch; the cavity
                    // work (tallies, ESD sums, history, transfer) runs after the loop
                    float2* const xsp = cav ? P.xs : nullptr;
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        // phase increment beta*s from the exact fixed-point target minus the
                        // phase applied so far (error feedback: FP32 rounding of the
                        // increment is carried into the next step instead of accumulating)
                        // increment beta*s: exact fixed-point target minus the phase applied
                        // so far (error feedback: nothing accumulates from FP32 rounding)
                        const int idx = j * T + t;
                        uint64_t target = tau_s[idx] * (uint64_t)qn;
                        uint32_t ph = papp_s[idx];
                        int d32 = (int)((long long)(target - ((uint64_t)ph << 32)) >> 32);
                        float2 dm1;
                        int dused;
                        if constexpr (heun) {
                            // D - 1 cached per mode for the current stepmod; the small
                            // difference eps between the wanted and the cached increment
                            // is applied to first order: D e^{-i eps} - 1 ~ (D - 1) - i eps D
                            float2 dc1 = dmc_s[idx];
                            int eps = d32 - dfc_s[idx];
                            dm1 = dc1;
                            if (eps != 0) {
                                float e = (float)eps * 1.4629180792671596e-09f;
                                float2 D = make_float2(1.f + dc1.x, dc1.y);
                                dm1 = make_float2(fmaf(e, D.y, dc1.x), fmaf(-e, D.x, dc1.y));
                            }
                            dused = d32;
                        } else {
                            dm1 = dispersion_dm1(d32, l2a_s[idx], s_used, &dused);
                        }
                        papp_s[idx] = ph + (uint32_t)dused;
                        float2 eh = v[j];
                        int kk = c + C * bitrev(16 * t + j, LOG2M);
                        if (apc) apc[kk] = cadd(eh, cmul(eh, dm1));
                        if (cav) xsp[kk] = cadd(eh, cmul(eh, dm1));
                        else v[j] = cmul(eh, dm1);
                    }
                    s_cached = s_used;
                    if (cav) {
                        // once per round trip, outside the unrolled mode loop (code size is
                        // this kernel's bound): energy tallies, ESD sums and history of the
                        // crystal output X, then Y = X fb + pump; every mode has one owner
                        // thread, which reads back only what it wrote
#pragma unroll 1
                        for (int j = 0; j < 16; ++j) {
                            const int kk = c + C * bitrev(16 * t + j, LOG2M);
                            const float2 X = xsp[kk];
                            const float x2 = X.x * X.x + X.y * X.y;
#pragma unroll
                            for (int i = 0; i < 4; ++i)
                                if (i < P.n_tally) part[i] = fmaf(P.tally_w[(size_t)i * N + kk], x2, part[i]);
#pragma unroll 1
                            for (int i = 0; i < P.n_esd; ++i)
                                P.esd[(size_t)i * N + kk] += P.esd_w[(size_t)i * N + kk] * x2;
                            if (P.hist) P.hist[(size_t)trip * N + kk] = X;
                            xsp[kk] = cadd(cmul(X, P.fb[kk]), P.pump[kk]);
                        }
#pragma unroll
                        for (int j = 0; j < 16; ++j) v[j] = xsp[c + C * bitrev(16 * t + j, LOG2M)];
                    }
                    fft_inverse_from_regs<M>(fbuf, tw1, tw2, t, v, ybuf);
                    if constexpr (C > 1) {
                        cg::this_cluster().sync();
                        exchange_inverse_g<M, C>(P.xch + N, bufX, P.xch, quad_s, low_s, t, c, invN);
                        cg::this_cluster().sync();
                        if constexpr (kPushExchange<C>) {
#pragma unroll
                            for (int j = 0; j < 16; ++j) {
                                const float2 d = bufX[phys(16 * t + j)];
                                a[j] = cav ? d : cadd(bufE[phys(16 * t + j)], d);
                            }
                        } else {
                            const float4* src = reinterpret_cast<const float4*>(P.xch + c * M + 16 * t);
#pragma unroll
                            for (int j = 0; j < 8; ++j) {
                                float4 w = __ldcg(src + j);
                                float2 d0 = make_float2(w.x, w.y), d1 = make_float2(w.z, w.w);
                                a[2 * j] = cav ? d0 : cadd(bufE[phys(16 * t + 2 * j)], d0);
                                a[2 * j + 1] = cav ? d1 : cadd(bufE[phys(16 * t + 2 * j + 1)], d1);
                            }
                        }
                    } else {
                        if (cav) {
#pragma unroll
                            for (int j = 0; j < 16; ++j) a[j] = cscale(bufE[phys(16 * t + j)], invN);
                        } else {
#pragma unroll
                            for (int j = 0; j < 16; ++j)
                                a[j] = cadd(bufX[phys(16 * t + j)], cscale(bufE[phys(16 * t + j)], invN));
                        }
                    }
                    if constexpr (METHOD == OPTIFAX_RK23) {
#pragma unroll
                        for (int j = 0; j < 16; ++j) k1r[j] = bufK[phys(16 * t + j)];
                    }
                    if (cav) reduce_tallies<M, C>(part, tally, dred, t, c, trip & 1);
                    q = qn;
                }
                ++attempt;
                ++gatt;
                if (!nee || accepted) k = k + stepmod;
            }
        }
        status |= trip_status;
        tot_att += attempt; tot_acc += n_acc; tot_rej += n_rej;
        trips_done = trip + 1;
        if (opo) {
            if (rec && P.trips) {
                optifax_trip_record tr;
                tr.attempts = attempt; tr.accepted = n_acc; tr.rejected = n_rej; tr.status = trip_status;
                for (int i = 0; i < 4; ++i) tr.tally[i] = tally[i];
                P.trips[trip] = tr;
            }
            if (P.steady_trips > 0) {
                double cur = tally[P.steady_tally & 3];
                bool flat = trip > 0 && cur != 0.0 && fabs(cur - prev_tally) <= (double)P.steady_tol * fabs(cur);
                steady_count = flat ? steady_count + 1 : 0;
                prev_tally = cur;
                if (steady_count >= P.steady_trips) break;
            }
        }
    }
done:
#pragma unroll
    for (int j = 0; j < 16; ++j) P.A_out[c * M + 16 * t + j] = a[j];
    if (rec && P.stats) {
        optifax_pulse_stats st;
        st.attempts = tot_att; st.accepted = tot_acc; st.rejected = tot_rej; st.status = status;
        st.z_steps = (long long)q; st.k_final = k; st.stepmod_final = stepmod; st.n_chunks = nchunks;
        st.reserved[0] = trips_done; st.reserved[1] = st.reserved[2] = 0;
        *P.stats = st;
    }
}

}  // namespace ofx
