// ofx_fft64.cuh -- double-precision radix-4/radix-2 FFT over global memory, one
// kernel per pair of stages, batched over blockIdx.y (no cuFFT).  Used by the
// plain FP64 solver and by the device-side setup precompute.
#pragma once
#include <cuda_runtime.h>

namespace {

__device__ __forceinline__ double2 dmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__global__ void f64_bitrev(const double2* __restrict__ x, double2* __restrict__ y, int n, int log2n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    size_t base = (size_t)blockIdx.y * n;
    int r = (int)(__brev((unsigned)i) >> (32 - log2n));
    y[base + r] = x[base + i];
}

// two radix-2 DIT stages (len, 2 len) in place; `sign` +1 forward, -1 inverse
__global__ void f64_radix4(double2* x, const double2* __restrict__ tw, int n, int len, int sign) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    int h = len / 2;
    if (q >= n / 4) return;
    int blk = q / h, j = q - blk * h;
    size_t base = (size_t)blockIdx.y * n + (size_t)blk * 2 * len;
    double2 w1 = tw[j * (n / len)];
    double2 w2a = tw[j * (n / (2 * len))];
    double2 w2b = tw[(j + h) * (n / (2 * len))];
    if (sign < 0) { w1.y = -w1.y; w2a.y = -w2a.y; w2b.y = -w2b.y; }
    double2 a = x[base + j], b = x[base + j + h], c = x[base + len + j], d = x[base + len + j + h];
    double2 tb = dmul(b, w1), td = dmul(d, w1);
    double2 a1 = make_double2(a.x + tb.x, a.y + tb.y), b1 = make_double2(a.x - tb.x, a.y - tb.y);
    double2 c1 = make_double2(c.x + td.x, c.y + td.y), d1 = make_double2(c.x - td.x, c.y - td.y);
    double2 tc = dmul(c1, w2a), tdd = dmul(d1, w2b);
    x[base + j] = make_double2(a1.x + tc.x, a1.y + tc.y);
    x[base + len + j] = make_double2(a1.x - tc.x, a1.y - tc.y);
    x[base + j + h] = make_double2(b1.x + tdd.x, b1.y + tdd.y);
    x[base + len + j + h] = make_double2(b1.x - tdd.x, b1.y - tdd.y);
}

__global__ void f64_radix2(double2* x, const double2* __restrict__ tw, int n, int len, int sign) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    int h = len / 2;
    if (q >= n / 2) return;
    int blk = q / h, j = q - blk * h;
    size_t base = (size_t)blockIdx.y * n + (size_t)blk * len;
    double2 w = tw[j * (n / len)];
    if (sign < 0) w.y = -w.y;
    double2 a = x[base + j], t = dmul(x[base + j + h], w);
    x[base + j] = make_double2(a.x + t.x, a.y + t.y);
    x[base + j + h] = make_double2(a.x - t.x, a.y - t.y);
}

__global__ void f64_twiddles(double2* tw, int n) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n / 2) return;
    double s, c;
    sincospi(-2.0 * (double)e / (double)n, &s, &c);
    tw[e] = make_double2(c, s);
}

inline int ilog2i(int n) { int l = 0; while ((1 << l) < n) ++l; return l; }

// forward (sign +1) or unnormalised inverse (sign -1) of every pulse, from src into dst
inline void fft64(const double2* src, double2* dst, const double2* tw, int n, int b, int sign, cudaStream_t st) {
    int lg = ilog2i(n);
    dim3 grid((n + 255) / 256, b);
    f64_bitrev<<<grid, 256, 0, st>>>(src, dst, n, lg);
    int len = 2;
    if (lg & 1) {
        f64_radix2<<<dim3((n / 2 + 255) / 256, b), 256, 0, st>>>(dst, tw, n, 2, sign);
        len = 4;
    }
    for (; len <= n / 2; len *= 4) f64_radix4<<<dim3((n / 4 + 255) / 256, b), 256, 0, st>>>(dst, tw, n, len, sign);
}

}  // namespace
