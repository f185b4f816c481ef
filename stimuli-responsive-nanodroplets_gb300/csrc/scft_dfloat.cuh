/*
 * scft_dfloat.cuh — double-float arithmetic for the propagator passes of the
 * FP32x2 form.
 *
 * A value is the unevaluated sum hi + lo of two FP32 numbers with
 * |lo| <= ulp(hi)/2: about 48 significant bits over FP32's exponent range.
 * GB300 runs FP64 FMAs at about 1/60 of its FP32 rate, so a propagator pass
 * computed on these pairs (10-20 FP32 instructions per operation) is several
 * times faster than the same pass in FP64, at a rounding error of ~2^-47
 * instead of 2^-53: far below what a field iteration run to RMS 1e-6 or 1e-8
 * can see, and far below the FP32 form's floor.
 *
 * Building blocks: Knuth's TwoSum, Dekker's Fast2Sum and the FMA-based
 * TwoProd. The sum is the "sloppy" double-word sum and the product the
 * FMA-based double-word product of Joldes, Muller and Popescu, "Tight and
 * rigorous error bounds for basic building blocks of double-word arithmetic",
 * ACM TOMS 44 (2017). The sloppy sum's error is bounded by a few 2^-48 of
 * |x| + |y| (not of |x + y|): the same normwise bound an FFT or a dot product
 * has in any precision. Every operation goes through the _rn intrinsics,
 * which the compiler never contracts into an FMA: a contraction would break
 * the error-free transforms.
 */
#pragma once

#include <cuda_runtime.h>

struct dfloat {
    float hi, lo;

    dfloat() = default;
    __host__ __device__ constexpr dfloat(float h, float l) : hi(h), lo(l) {}
    /* nearest pair to a double: hi = fl32(d), lo = fl32(d - hi) (d - hi is exact in FP64) */
    __host__ __device__ constexpr dfloat(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
    __host__ __device__ constexpr dfloat(int i) : dfloat((double)i) {}
    __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

namespace dfo {

/* s + e == a + b exactly (Knuth) */
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

/* s + e == a + b exactly when |a| >= |b| or a == 0 (Dekker) */
__device__ __forceinline__ dfloat fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return dfloat(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ dfloat add(dfloat x, dfloat y)
{
    float s, e;
    two_sum(x.hi, y.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(x.lo, y.lo));
    return fast_two_sum(s, e);
}

__device__ __forceinline__ dfloat neg(dfloat x) { return dfloat(-x.hi, -x.lo); }

__device__ __forceinline__ dfloat mul(dfloat x, dfloat y)
{
    const float p = __fmul_rn(x.hi, y.hi);
    float e = __fmaf_rn(x.hi, y.hi, -p);
    e = __fadd_rn(e, __fmaf_rn(x.hi, y.lo, __fmul_rn(x.lo, y.hi)));
    return fast_two_sum(p, e);
}

/* x*y - u*v with one renormalisation (the real or imaginary part of a complex product) */
__device__ __forceinline__ dfloat mul_sub(dfloat x, dfloat y, dfloat u, dfloat v)
{
    const float p = __fmul_rn(x.hi, y.hi);
    const float q = __fmul_rn(u.hi, v.hi);
    const float ep = __fmaf_rn(x.hi, y.hi, -p);
    const float eq = __fmaf_rn(u.hi, v.hi, -q);
    float s, e;
    two_sum(p, -q, s, e);
    float t = __fmaf_rn(x.hi, y.lo, __fmul_rn(x.lo, y.hi));
    t = __fsub_rn(t, __fmaf_rn(u.hi, v.lo, __fmul_rn(u.lo, v.hi)));
    e = __fadd_rn(e, __fadd_rn(__fsub_rn(ep, eq), t));
    return fast_two_sum(s, e);
}

/* x*y + u*v */
__device__ __forceinline__ dfloat mul_add(dfloat x, dfloat y, dfloat u, dfloat v)
{
    return mul_sub(x, y, neg(u), v);
}

/* Division: one FP32 quotient, the remainder x - q*y in double-float, one
 * correction term (the double-word division of the paper above). */
__device__ __forceinline__ dfloat div(dfloat x, dfloat y)
{
    const float q = __fdiv_rn(x.hi, y.hi);
    const dfloat r = add(x, neg(mul(dfloat(q, 0.0f), y)));
    return fast_two_sum(q, __fdiv_rn(r.hi, y.hi));
}

} // namespace dfo

__device__ __forceinline__ dfloat operator+(dfloat x, dfloat y) { return dfo::add(x, y); }
__device__ __forceinline__ dfloat operator-(dfloat x, dfloat y) { return dfo::add(x, dfo::neg(y)); }
__device__ __forceinline__ dfloat operator-(dfloat x) { return dfo::neg(x); }
__device__ __forceinline__ dfloat operator*(dfloat x, dfloat y) { return dfo::mul(x, y); }
__device__ __forceinline__ dfloat operator/(dfloat x, dfloat y) { return dfo::div(x, y); }
__device__ __forceinline__ dfloat &operator+=(dfloat &x, dfloat y) { return x = x + y; }
__device__ __forceinline__ dfloat &operator*=(dfloat &x, dfloat y) { return x = x * y; }

/* Dot-product accumulator: the running sum's high part is kept error-free
 * (TwoSum), product errors (TwoProd) and cross terms go to an FP32 low part,
 * renormalised once at the end (the compensated dot product of Ogita, Rump
 * and Oishi, extended to double-float operands). 12 FP32 instructions a term. */
struct DotDF {
    float hi, lo;
    __device__ __forceinline__ void zero() { hi = lo = 0.0f; }
    __device__ __forceinline__ void add(dfloat a, dfloat b)
    {
        const float p = __fmul_rn(a.hi, b.hi);
        float e = __fmaf_rn(a.hi, b.hi, -p);
        e = __fmaf_rn(a.hi, b.lo, e);
        e = __fmaf_rn(a.lo, b.hi, e);
        float s, se;
        dfo::two_sum(hi, p, s, se);
        hi = s;
        lo = __fadd_rn(lo, __fadd_rn(se, e));
    }
    __device__ __forceinline__ dfloat value() const { return dfo::fast_two_sum(hi, lo); }
};
