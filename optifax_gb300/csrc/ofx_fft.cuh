// ofx_fft.cuh -- in-shared-memory complex FFT of one CTA's M points.
//
// Decimation in frequency with three register passes of radix 16/16/(M/256):
// each thread owns one radix-R butterfly group (16 points) per pass.  A pass
// over blocks of length L computes, for every offset `off` in [0, L/R),
//     y_r = W_L^{off r} * DFT_R(x[off + q L/R])_r
// with DFT_R done in registers by radix-2 stages whose twiddles are
// compile-time constants (bit-reversed output: register q holds r = bitrev(q)),
// and the outer twiddle W_L^{off r} read from a per-pass table laid out
// [r][off] so consecutive threads read consecutive entries.  The forward
// transform therefore leaves the spectrum in bit-reversed slot order; the
// inverse undoes every multiply with the exact reciprocal (conj(w)(1+d)) and
// returns natural order.  The last forward pass and the first inverse pass
// act on the same registers (thread t holds slots 16t .. 16t+15), so per-mode
// work sits between them without a shared-memory round trip.
//
// Unnormalised: forward followed by inverse multiplies by M.
#pragma once
#include "ofx_common.cuh"

namespace ofx {

template <int M>
struct FftShape {
    static_assert(M >= 512 && M <= 4096 && (M & (M - 1)) == 0, "M must be 512..4096");
    static constexpr int T = M / 16;      // threads per CTA
    static constexpr int L1 = M, R1 = 16;
    static constexpr int L2 = M / 16, R2 = 16;
    static constexpr int L3 = M / 256, R3 = M / 256;   // last pass: L == R
    static constexpr int LOG2M = (M == 512) ? 9 : (M == 1024) ? 10 : (M == 2048) ? 11 : 12;
    // outer-twiddle tables: pass 1 [16][M/16], pass 2 [16][M/256]
    static constexpr int TW1 = 16 * (M / 16);
    static constexpr int TW2 = 16 * (M / 256);
};

// W_16^m = exp(-2 pi i m / 16), m = 0..7, rounded to FP32; d = 1/|w|^2 - 1
__device__ __forceinline__ float w16c(int m) {
    constexpr float c[8] = {1.0f, 0.9238795042037964f, 0.7071067690849304f, 0.3826834261417389f,
                            0.0f, -0.3826834261417389f, -0.7071067690849304f, -0.9238795042037964f};
    return c[m];
}
__device__ __forceinline__ float w16s(int m) {
    constexpr float s[8] = {0.0f, -0.3826834261417389f, -0.7071067690849304f, -0.9238795042037964f,
                            -1.0f, -0.9238795042037964f, -0.7071067690849304f, -0.3826834261417389f};
    return s[m];
}
__device__ __forceinline__ float w16d(int m) {
    constexpr float d[8] = {0.0f, 5.7068572090201997e-08f, 3.422854177870249e-08f, 5.7068572090201997e-08f,
                            0.0f, 5.7068572090201997e-08f, 3.422854177870249e-08f, 5.7068572090201997e-08f};
    return d[m];
}

// v * W_16^m for a compile-time m in 0..7 (trivial cases folded)
__device__ __forceinline__ float2 mul_w16(float2 v, int m) {
    if (m == 0) return v;
    if (m == 4) return make_float2(v.y, -v.x);                 // * (-i)
    return cmul(v, make_float2(w16c(m), w16s(m)));
}
// v / W_16^m = v * conj(W_16^m) (1 + d)
__device__ __forceinline__ float2 div_w16(float2 v, int m) {
    if (m == 0) return v;
    if (m == 4) return make_float2(-v.y, v.x);                 // * i
    float2 t = cmulc(v, make_float2(w16c(m), w16s(m)));
    float d = w16d(m);
    return make_float2(fmaf(t.x, d, t.x), fmaf(t.y, d, t.y));
}

// DFT_R of v[0..R) by radix-2 DIF stages; register q ends holding output bitrev(q)
template <int R>
__device__ __forceinline__ void dft_dif(float2* v) {
#pragma unroll
    for (int hr = R / 2; hr >= 1; hr >>= 1) {
#pragma unroll
        for (int q = 0; q < R; ++q) {
            if (q & hr) continue;
            const int m16 = (q & (hr - 1)) * (R / (2 * hr)) * (16 / R);
            float2 a = v[q], b = v[q + hr];
            v[q] = cadd(a, b);
            v[q + hr] = mul_w16(csub(a, b), m16);
        }
    }
}

// exact reverse of dft_dif (unnormalised: each stage doubles)
template <int R>
__device__ __forceinline__ void dft_dit_inv(float2* v) {
#pragma unroll
    for (int hr = 1; hr <= R / 2; hr <<= 1) {
#pragma unroll
        for (int q = 0; q < R; ++q) {
            if (q & hr) continue;
            const int m16 = (q & (hr - 1)) * (R / (2 * hr)) * (16 / R);
            float2 a = v[q];
            float2 t = div_w16(v[q + hr], m16);
            v[q] = cadd(a, t);
            v[q + hr] = csub(a, t);
        }
    }
}

__device__ __forceinline__ int brev4(int q, int bits) {
    // bit reversal of q within `bits` (<= 4) bits, compile-time foldable
    int r = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b)
        if (b < bits && (q & (1 << b))) r |= 1 << (bits - 1 - b);
    return r;
}

// element index of (butterfly slot u, leg q) handled by thread t in a pass of
// radix R over blocks of length L.  LASTMAP assigns each thread contiguous
// butterflies (slots 16t..16t+15 in the last pass); otherwise consecutive
// threads take consecutive butterflies (coalesced, conflict-free).
template <int M, int R, int L, bool LASTMAP>
__device__ __forceinline__ int pass_index(int t, int u, int q, int& off) {
    constexpr int T = M / 16, NB = 16 / R, LR = L / R;
    int beta = LASTMAP ? t * NB + u : t + T * u;
    int b = beta / LR;
    off = beta - b * LR;
    return b * L + off + q * LR;
}

template <int M, int R, int L, bool LASTMAP>
__device__ __forceinline__ void pass_load(const float2* buf, int t, float2 (&v)[16], int (&offs)[16 / R]) {
#pragma unroll
    for (int u = 0; u < 16 / R; ++u)
#pragma unroll
        for (int q = 0; q < R; ++q) {
            int off;
            int m = pass_index<M, R, L, LASTMAP>(t, u, q, off);
            v[u * R + q] = buf[phys(m)];
            offs[u] = off;
        }
}

template <int M, int R, int L, bool LASTMAP>
__device__ __forceinline__ void pass_store(float2* buf, int t, const float2 (&v)[16]) {
#pragma unroll
    for (int u = 0; u < 16 / R; ++u)
#pragma unroll
        for (int q = 0; q < R; ++q) {
            int off;
            int m = pass_index<M, R, L, LASTMAP>(t, u, q, off);
            buf[phys(m)] = v[u * R + q];
        }
}

template <int M, int R, int L>
__device__ __forceinline__ void fwd_pass_smem(float2* buf, const Twiddle* __restrict__ tw, int t,
                                              const float2* gin = nullptr) {
    constexpr int LR = L / R, BITS = (R == 16) ? 4 : (R == 8) ? 3 : (R == 4) ? 2 : 1;
    float2 v[16];
    int offs[16 / R];
    if (gin) {
        // input from global memory (cluster exchange buffer, natural order, L2)
#pragma unroll
        for (int u = 0; u < 16 / R; ++u)
#pragma unroll
            for (int q = 0; q < R; ++q) {
                int off;
                int m = pass_index<M, R, L, false>(t, u, q, off);
                v[u * R + q] = __ldcg(gin + m);
                offs[u] = off;
            }
    } else {
        pass_load<M, R, L, false>(buf, t, v, offs);
    }
#pragma unroll
    for (int u = 0; u < 16 / R; ++u) {
        dft_dif<R>(v + u * R);
#pragma unroll
        for (int q = 1; q < R; ++q) v[u * R + q] = tw_fwd(v[u * R + q], tw[brev4(q, BITS) * LR + offs[u]]);
    }
    pass_store<M, R, L, false>(buf, t, v);
}

template <int M, int R, int L>
__device__ __forceinline__ void inv_pass_smem(float2* buf, const Twiddle* __restrict__ tw, int t,
                                              float2* gout = nullptr) {
    constexpr int LR = L / R, BITS = (R == 16) ? 4 : (R == 8) ? 3 : (R == 4) ? 2 : 1;
    float2 v[16];
    int offs[16 / R];
    pass_load<M, R, L, false>(buf, t, v, offs);
#pragma unroll
    for (int u = 0; u < 16 / R; ++u) {
#pragma unroll
        for (int q = 1; q < R; ++q) v[u * R + q] = tw_inv(v[u * R + q], tw[brev4(q, BITS) * LR + offs[u]]);
        dft_dit_inv<R>(v + u * R);
    }
    if (gout) {
#pragma unroll
        for (int u = 0; u < 16 / R; ++u)
#pragma unroll
            for (int q = 0; q < R; ++q) {
                int off;
                int m = pass_index<M, R, L, false>(t, u, q, off);
                __stcg(gout + m, v[u * R + q]);
            }
    } else {
        pass_store<M, R, L, false>(buf, t, v);
    }
}

// Forward passes 1 and 2 in shared memory, then the last pass into registers:
// on return v[j] holds slot 16t + j.  tw1/tw2: outer-twiddle tables of
// passes 1 and 2.  Pass 1 reads `gin` (global, natural order) when given,
// else buf.  The caller synchronises before (input complete).
template <int M>
__device__ __forceinline__ void fft_forward_to_regs(float2* buf, const Twiddle* __restrict__ tw1,
                                                    const Twiddle* __restrict__ tw2, int t, float2 (&v)[16],
                                                    const float2* gin = nullptr) {
    using S = FftShape<M>;
    fwd_pass_smem<M, S::R1, S::L1>(buf, tw1, t, gin);
    __syncthreads();
    fwd_pass_smem<M, S::R2, S::L2>(buf, tw2, t);
    __syncthreads();
    int offs[16 / S::R3];
    pass_load<M, S::R3, S::L3, true>(buf, t, v, offs);
#pragma unroll
    for (int u = 0; u < 16 / S::R3; ++u) dft_dif<S::R3>(v + u * S::R3);
}

// Inverse of fft_forward_to_regs: v holds slots 16t+j; on return buf (or
// `gout`, global, when given) holds the unnormalised inverse transform in
// natural order.  Each thread only writes its own slots before the first
// barrier, so no barrier is needed on entry.
template <int M>
__device__ __forceinline__ void fft_inverse_from_regs(float2* buf, const Twiddle* __restrict__ tw1,
                                                      const Twiddle* __restrict__ tw2, int t, float2 (&v)[16],
                                                      float2* gout = nullptr) {
    using S = FftShape<M>;
#pragma unroll
    for (int u = 0; u < 16 / S::R3; ++u) dft_dit_inv<S::R3>(v + u * S::R3);
    pass_store<M, S::R3, S::L3, true>(buf, t, v);
    __syncthreads();
    inv_pass_smem<M, S::R2, S::L2>(buf, tw2, t);
    __syncthreads();
    inv_pass_smem<M, S::R1, S::L1>(buf, tw1, t, gout);
    __syncthreads();
}

}  // namespace ofx
