// ofx_fft.cuh -- in-shared-memory complex FFT of one CTA's M points.
//
// Radix-2 decimation in frequency, grouped into three passes of register
// radix 16/16/(M/256): each thread owns 16 points per pass.  The forward
// transform leaves the spectrum in bit-reversed slot order; the inverse
// (decimation in time, the exact reverse of every forward butterfly) takes
// bit-reversed input and returns natural order.  Per-mode work (dispersion,
// snapshots, energies) therefore runs in slot order with the mode index
// k2 = bitrev(slot).  The last forward pass and the first inverse pass act on
// the same 16 registers, so the per-mode multiply sits between them without a
// shared-memory round trip: thread t holds slots 16t .. 16t+15.
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
};

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

// r = log2(R) forward DIF stages on v[0..R) with block length L and offset off
template <int M, int R, int L>
__device__ __forceinline__ void dif_stages(float2* v, int off, const Twiddle* __restrict__ tw) {
#pragma unroll
    for (int hr = R / 2; hr >= 1; hr >>= 1) {
#pragma unroll
        for (int q = 0; q < R; ++q) {
            if (q & hr) continue;
            int o = off + (q & (hr - 1)) * (L / R);
            int e = o * (R / (2 * hr)) * (M / L);
            float2 a = v[q], b = v[q + hr];
            v[q] = cadd(a, b);
            v[q + hr] = tw_fwd(csub(a, b), tw[e]);
        }
    }
}

// exact reverse of dif_stages (unnormalised: each stage doubles)
template <int M, int R, int L>
__device__ __forceinline__ void dit_stages(float2* v, int off, const Twiddle* __restrict__ tw) {
#pragma unroll
    for (int hr = 1; hr <= R / 2; hr <<= 1) {
#pragma unroll
        for (int q = 0; q < R; ++q) {
            if (q & hr) continue;
            int o = off + (q & (hr - 1)) * (L / R);
            int e = o * (R / (2 * hr)) * (M / L);
            float2 a = v[q];
            float2 t = tw_inv(v[q + hr], tw[e]);
            v[q] = cadd(a, t);
            v[q + hr] = csub(a, t);
        }
    }
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
__device__ __forceinline__ void fwd_pass_smem(float2* buf, const Twiddle* __restrict__ tw, int t) {
    float2 v[16];
    int offs[16 / R];
    pass_load<M, R, L, false>(buf, t, v, offs);
#pragma unroll
    for (int u = 0; u < 16 / R; ++u) dif_stages<M, R, L>(v + u * R, offs[u], tw);
    pass_store<M, R, L, false>(buf, t, v);
}

template <int M, int R, int L>
__device__ __forceinline__ void inv_pass_smem(float2* buf, const Twiddle* __restrict__ tw, int t) {
    float2 v[16];
    int offs[16 / R];
    pass_load<M, R, L, false>(buf, t, v, offs);
#pragma unroll
    for (int u = 0; u < 16 / R; ++u) dit_stages<M, R, L>(v + u * R, offs[u], tw);
    pass_store<M, R, L, false>(buf, t, v);
}

// Forward passes 1 and 2 in shared memory, then the last pass into registers:
// on return v[j] holds slot 16t + j.  Synchronisation between passes is the
// caller-supplied barrier functor (CTA barrier).
template <int M>
__device__ __forceinline__ void fft_forward_to_regs(float2* buf, const Twiddle* __restrict__ tw, int t,
                                                    float2 (&v)[16]) {
    using S = FftShape<M>;
    fwd_pass_smem<M, S::R1, S::L1>(buf, tw, t);
    __syncthreads();
    fwd_pass_smem<M, S::R2, S::L2>(buf, tw, t);
    __syncthreads();
    int offs[16 / S::R3];
    pass_load<M, S::R3, S::L3, true>(buf, t, v, offs);
#pragma unroll
    for (int u = 0; u < 16 / S::R3; ++u) dif_stages<M, S::R3, S::L3>(v + u * S::R3, 0, tw);
}

// Inverse of fft_forward_to_regs: v holds slots 16t+j; on return buf holds the
// unnormalised inverse transform in natural order.  Each thread only writes
// its own slots before the first barrier, so no barrier is needed on entry.
template <int M>
__device__ __forceinline__ void fft_inverse_from_regs(float2* buf, const Twiddle* __restrict__ tw, int t,
                                                      float2 (&v)[16]) {
    using S = FftShape<M>;
#pragma unroll
    for (int u = 0; u < 16 / S::R3; ++u) dit_stages<M, S::R3, S::L3>(v + u * S::R3, 0, tw);
    pass_store<M, S::R3, S::L3, true>(buf, t, v);
    __syncthreads();
    inv_pass_smem<M, S::R2, S::L2>(buf, tw, t);
    __syncthreads();
    inv_pass_smem<M, S::R1, S::L1>(buf, tw, t);
    __syncthreads();
}

}  // namespace ofx
