// ofx_common.cuh -- device helpers shared by the crystal-pass kernels.
//
// Complex arithmetic on float2, the fixed-point phase representation used to
// keep every accumulated phase exact to FP64 precision without FP64 work in
// the inner loops, and the twiddle-table entry layout.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ofx {

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float cabsf2(float2 a) { return hypotf(a.x, a.y); }

// A phase in turns held as an unsigned 64-bit fixed-point fraction
// (2^64 == one turn).  Products of a per-unit phase with an integer position
// wrap modulo one turn exactly, so z-positions up to 2^32 keep the phase
// exact to ~1e-19 turns.  turn_to_unit returns exp(2 pi i u / 2^64) with the
// top 24 bits evaluated by sincospif and the remaining bits applied as a
// first-order rotation (|remainder| < 2 pi 2^-24 rad), accurate to ~1 ulp.
__device__ __forceinline__ float2 turn_to_unit(uint64_t u) {
    int32_t hi = (int32_t)(u >> 32);
    int32_t a = hi >> 8;                               // top 24 bits, signed
    float x = (float)a * 0x1p-23f;                     // half-turns in [-1, 1)
    float s, c;
    sincospif(x, &s, &c);
    uint32_t r24 = (uint32_t)((u << 24) >> 40);       // next 24 bits
    float d = (float)r24 * (0x1p-48f * 6.28318530717958647692f);
    return make_float2(fmaf(-s, d, c), fmaf(c, d, s));
}

// Twiddle entry: w = (c, s) ~ exp(-2 pi i e / n) rounded to FP32, and
// d = 1/|w|^2 - 1 evaluated in FP64.  The inverse transform multiplies by
// conj(w) (1 + d), the exact reciprocal of w up to one rounding, so a forward
// plus inverse transform carries no systematic per-mode gain.
struct __align__(16) Twiddle { float c, s, d, pad; };

__device__ __forceinline__ float2 tw_fwd(float2 v, const Twiddle& w) {
    return cmul(v, make_float2(w.c, w.s));
}
__device__ __forceinline__ float2 tw_inv(float2 v, const Twiddle& w) {
    float2 t = cmulc(v, make_float2(w.c, w.s));
    return make_float2(fmaf(t.x, w.d, t.x), fmaf(t.y, w.d, t.y));
}

// W_M^x for 0 <= x < M from the quarter-period table q[y] = W_M^y, y < M/4
// (kept in shared memory): x = k M/4 + y gives W_M^y (-i)^k, a swap and sign
// changes, so the value and its d are those of a full table.
template <int M>
__device__ __forceinline__ Twiddle quad_tw(const Twiddle* q, int x) {
    const Twiddle w = q[x & (M / 4 - 1)];
    const int k = (x / (M / 4)) & 3;
    float c = (k & 1) ? w.s : w.c;
    float s = (k & 1) ? -w.c : w.s;
    if (k & 2) { c = -c; s = -s; }
    return Twiddle{c, s, w.d, 0.f};
}

// 1/|w|^2 - 1 for a computed |w| ~ 1.  g = |w|^2 - 1 is formed without
// rounding error beyond the last add (products split by fma; the subtractions
// are exact by Sterbenz's lemma), then 1/(1 + g) - 1 = -g + g^2 (g ~ 1e-7).
__device__ __forceinline__ float inv_norm2_m1(float2 w) {
    const float p1 = w.x * w.x, p2 = w.y * w.y;
    const float e1 = fmaf(w.x, w.x, -p1), e2 = fmaf(w.y, w.y, -p2);
    const float big = fmaxf(p1, p2), small = fminf(p1, p2);
    const float g0 = (big >= 0.5f) ? (big - 1.0f) + small : (p1 - 0.5f) + (p2 - 0.5f);
    const float g = g0 + (e1 + e2);
    return fmaf(g, g, -g);
}

__device__ __forceinline__ int bitrev(int x, int bits) {
    return bits == 0 ? 0 : (int)(__brev((unsigned)x) >> (32 - bits));
}

// Shared-memory placement of a complex point: one float2 of padding per 16
// keeps both the per-thread contiguous (16 points) accesses of the RK stages
// and the strided FFT-pass accesses free of bank conflicts.
__device__ __forceinline__ int phys(int m) { return m + (m >> 4); }

}  // namespace ofx
