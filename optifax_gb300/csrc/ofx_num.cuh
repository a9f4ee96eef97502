// ofx_num.cuh -- the two arithmetic types of the wide-state crystal pass
// (ofx_passx.cuh): native FP64, and float-float ("ff"), an unevaluated sum
// hi + lo of two FP32 values carrying about 48 significant bits.
//
// Why float-float on GB300: its FP64 rate is about 1/64 of its FP32 rate, so a
// complex multiply-add in float-float (~30 FP32 operations) costs less issue
// time than the same operation in FP64 (6 FP64 operations), while giving
// ~1e-14 relative precision -- enough for the high-gain cases in which the FP32
// field's rounding, amplified by the parametric gain, dominates the result.
//
// The float-float operations are the classical error-free transformations:
// TwoSum (Knuth, TAOCP vol. 2, 4.2.2), QuickTwoSum (Dekker 1971) and the exact
// product through a fused multiply-add (a*b - p = fma(a, b, -p)), combined as in
// the double-double literature (Hida, Li and Bailey, "Algorithms for quad-double
// precision floating point arithmetic", ARITH 2001), here one level down on FP32.
// Additions use the "sloppy" form: its error is bounded by a few units of 2^-48
// of max(|a|, |b|), which is the bound the FFT and the stage sums need (errors
// relative to the field's magnitude, not to a cancelled result).
//
// The translation unit that instantiates the float-float kernel is compiled with
// -fmad=false so that no a*b+c of an error-free transformation is contracted;
// every intended fused multiply-add is written as fmaf().
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ofx {

// ---------------------------------------------------------------------------
// float-float scalar
// ---------------------------------------------------------------------------
struct ff { float hi, lo; };

__device__ __forceinline__ ff ff_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return ff{s, e};
}
__device__ __forceinline__ ff ff_quick(float a, float b) {   // |a| >= |b|
    const float s = a + b;
    return ff{s, b - (s - a)};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    const ff s = ff_two_sum(a.hi, b.hi);
    return ff_quick(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = a.hi * b.hi;
    const float e = fmaf(a.hi, b.hi, -p);
    return ff_quick(p, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e)));
}
// a*b + c*d with one final normalisation
__device__ __forceinline__ ff ff_dot2(ff a, ff b, ff c, ff d) {
    const float p = a.hi * b.hi, q = c.hi * d.hi;
    const float ep = fmaf(a.hi, b.hi, -p), eq = fmaf(c.hi, d.hi, -q);
    const ff s = ff_two_sum(p, q);
    float t = s.lo + (ep + eq);
    t = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, t));
    t = fmaf(c.hi, d.lo, fmaf(c.lo, d.hi, t));
    return ff_quick(s.hi, t);
}
// scaling by an exact power of two (0.5, 2): exact
__device__ __forceinline__ ff ff_pow2(ff a, float s) { return ff{a.hi * s, a.lo * s}; }
__device__ __forceinline__ ff ff_from(double x) {
    const float h = (float)x;
    return ff{h, (float)(x - (double)h)};
}
__device__ __forceinline__ double ff_d(ff a) { return (double)a.hi + (double)a.lo; }

// ---------------------------------------------------------------------------
// complex types and the operations the kernel uses, per arithmetic type
// ---------------------------------------------------------------------------
// float-float complex, stored as {re.hi, re.lo, im.hi, im.lo}
struct __align__(16) cff { float rh, rl, ih, il; };

template <typename R> struct Num;

template <> struct Num<double> {
    using cplx = double2;
    using real = double;
    static __device__ __forceinline__ cplx make(real re, real im) { return make_double2(re, im); }
    static __device__ __forceinline__ cplx zero() { return make_double2(0.0, 0.0); }
    static __device__ __forceinline__ real re(cplx a) { return a.x; }
    static __device__ __forceinline__ real im(cplx a) { return a.y; }
    static __device__ __forceinline__ cplx add(cplx a, cplx b) { return make_double2(a.x + b.x, a.y + b.y); }
    static __device__ __forceinline__ cplx sub(cplx a, cplx b) { return make_double2(a.x - b.x, a.y - b.y); }
    static __device__ __forceinline__ cplx mul(cplx a, cplx b) {
        return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
    }
    static __device__ __forceinline__ cplx mulc(cplx a, cplx b) {   // a * conj(b)
        return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
    }
    static __device__ __forceinline__ cplx scale(cplx a, real s) { return make_double2(a.x * s, a.y * s); }
    static __device__ __forceinline__ cplx pow2(cplx a, double s) { return make_double2(a.x * s, a.y * s); }
    static __device__ __forceinline__ cplx conj(cplx a) { return make_double2(a.x, -a.y); }
    static __device__ __forceinline__ cplx mul_i(cplx a) { return make_double2(-a.y, a.x); }       // i a
    static __device__ __forceinline__ cplx mul_mi(cplx a) { return make_double2(a.y, -a.x); }      // -i a
    static __device__ __forceinline__ real rfrom(double x) { return x; }
    static __device__ __forceinline__ cplx from(double2 v) { return v; }
    static __device__ __forceinline__ double2 to_d(cplx v) { return v; }
    static __device__ __forceinline__ real norm2(cplx a) { return a.x * a.x + a.y * a.y; }
    static __device__ __forceinline__ real radd(real a, real b) { return a + b; }
    static __device__ __forceinline__ real rmul(real a, real b) { return a * b; }
    static __device__ __forceinline__ bool finite(cplx a) { return isfinite(a.x) && isfinite(a.y); }
};

template <> struct Num<ff> {
    using cplx = cff;
    using real = ff;
    static __device__ __forceinline__ cplx make(real re, real im) { return cff{re.hi, re.lo, im.hi, im.lo}; }
    static __device__ __forceinline__ cplx zero() { return cff{0.f, 0.f, 0.f, 0.f}; }
    static __device__ __forceinline__ real re(cplx a) { return ff{a.rh, a.rl}; }
    static __device__ __forceinline__ real im(cplx a) { return ff{a.ih, a.il}; }
    static __device__ __forceinline__ cplx add(cplx a, cplx b) { return make(ff_add(re(a), re(b)), ff_add(im(a), im(b))); }
    static __device__ __forceinline__ cplx sub(cplx a, cplx b) { return make(ff_sub(re(a), re(b)), ff_sub(im(a), im(b))); }
    static __device__ __forceinline__ cplx mul(cplx a, cplx b) {
        return make(ff_dot2(re(a), re(b), ff_neg(im(a)), im(b)), ff_dot2(re(a), im(b), im(a), re(b)));
    }
    static __device__ __forceinline__ cplx mulc(cplx a, cplx b) {
        return make(ff_dot2(re(a), re(b), im(a), im(b)), ff_dot2(im(a), re(b), ff_neg(re(a)), im(b)));
    }
    static __device__ __forceinline__ cplx scale(cplx a, real s) { return make(ff_mul(re(a), s), ff_mul(im(a), s)); }
    static __device__ __forceinline__ cplx pow2(cplx a, double s) {
        const float f = (float)s;
        return cff{a.rh * f, a.rl * f, a.ih * f, a.il * f};
    }
    static __device__ __forceinline__ cplx conj(cplx a) { return cff{a.rh, a.rl, -a.ih, -a.il}; }
    static __device__ __forceinline__ cplx mul_i(cplx a) { return cff{-a.ih, -a.il, a.rh, a.rl}; }
    static __device__ __forceinline__ cplx mul_mi(cplx a) { return cff{a.ih, a.il, -a.rh, -a.rl}; }
    static __device__ __forceinline__ real rfrom(double x) { return ff_from(x); }
    static __device__ __forceinline__ cplx from(double2 v) { return make(ff_from(v.x), ff_from(v.y)); }
    static __device__ __forceinline__ double2 to_d(cplx v) { return make_double2(ff_d(re(v)), ff_d(im(v))); }
    static __device__ __forceinline__ real norm2(cplx a) { return ff_dot2(re(a), re(a), im(a), im(a)); }
    static __device__ __forceinline__ real radd(real a, real b) { return ff_add(a, b); }
    static __device__ __forceinline__ real rmul(real a, real b) { return ff_mul(a, b); }
    static __device__ __forceinline__ bool finite(cplx a) { return isfinite(a.rh) && isfinite(a.ih); }
};

}  // namespace ofx
