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
 * the error-free transforms. The same code compiles for the host, where the
 * tests check it against long double.
 */
#pragma once

#include <cuda_runtime.h>
#include <math.h>

struct dfloat {
    float hi, lo;

    dfloat() = default;
    __host__ __device__ constexpr dfloat(float h, float l) : hi(h), lo(l) {}
    /* nearest pair to a double: hi = fl32(d), lo = fl32(d - hi) (d - hi is exact in FP64) */
    __host__ __device__ constexpr dfloat(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
    /* an int exactly (through the exact double; at run time a few FP64 conversions) */
    __host__ __device__ constexpr dfloat(int i) : dfloat((double)i) {}
    __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

namespace dfo {

/* The FP32 primitives, each rounded to nearest and never contracted: the _rn
 * intrinsics on the device; on the host (unit tests of these algorithms)
 * IEEE float operations whose results pass through a volatile, so no
 * multiply is fused into a following add, and the C99 fused multiply-add. */
__host__ __device__ __forceinline__ float f_add(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    volatile float r = a + b;
    return r;
#endif
}
__host__ __device__ __forceinline__ float f_sub(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    volatile float r = a - b;
    return r;
#endif
}
__host__ __device__ __forceinline__ float f_mul(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    volatile float r = a * b;
    return r;
#endif
}
__host__ __device__ __forceinline__ float f_fma(float a, float b, float c)
{
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}
__host__ __device__ __forceinline__ float f_div(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    volatile float r = a / b;
    return r;
#endif
}

/* s + e == a + b exactly (Knuth) */
__host__ __device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = f_add(a, b);
    const float bb = f_sub(s, a);
    e = f_add(f_sub(a, f_sub(s, bb)), f_sub(b, bb));
}

/* s + e == a + b exactly when |a| >= |b| or a == 0 (Dekker) */
__host__ __device__ __forceinline__ dfloat fast_two_sum(float a, float b)
{
    const float s = f_add(a, b);
    return dfloat(s, f_sub(b, f_sub(s, a)));
}

__host__ __device__ __forceinline__ dfloat add(dfloat x, dfloat y)
{
    float s, e;
    two_sum(x.hi, y.hi, s, e);
    e = f_add(e, f_add(x.lo, y.lo));
    return fast_two_sum(s, e);
}

__host__ __device__ __forceinline__ dfloat neg(dfloat x) { return dfloat(-x.hi, -x.lo); }

__host__ __device__ __forceinline__ dfloat mul(dfloat x, dfloat y)
{
    const float p = f_mul(x.hi, y.hi);
    float e = f_fma(x.hi, y.hi, -p);
    e = f_add(e, f_fma(x.hi, y.lo, f_mul(x.lo, y.hi)));
    return fast_two_sum(p, e);
}

/* x*y - u*v with one renormalisation (the real or imaginary part of a complex product) */
__host__ __device__ __forceinline__ dfloat mul_sub(dfloat x, dfloat y, dfloat u, dfloat v)
{
    const float p = f_mul(x.hi, y.hi);
    const float q = f_mul(u.hi, v.hi);
    const float ep = f_fma(x.hi, y.hi, -p);
    const float eq = f_fma(u.hi, v.hi, -q);
    float s, e;
    two_sum(p, -q, s, e);
    float t = f_fma(x.hi, y.lo, f_mul(x.lo, y.hi));
    t = f_sub(t, f_fma(u.hi, v.lo, f_mul(u.lo, v.hi)));
    e = f_add(e, f_add(f_sub(ep, eq), t));
    return fast_two_sum(s, e);
}

/* x*y + u*v */
__host__ __device__ __forceinline__ dfloat mul_add(dfloat x, dfloat y, dfloat u, dfloat v)
{
    return mul_sub(x, y, neg(u), v);
}

/* Division: one FP32 quotient, the remainder x - q*y in double-float, one
 * correction term (the double-word division of the paper above). */
__host__ __device__ __forceinline__ dfloat div(dfloat x, dfloat y)
{
    const float q = f_div(x.hi, y.hi);
    const dfloat r = add(x, neg(mul(dfloat(q, 0.0f), y)));
    return fast_two_sum(q, f_div(r.hi, y.hi));
}

} // namespace dfo

__host__ __device__ __forceinline__ dfloat operator+(dfloat x, dfloat y) { return dfo::add(x, y); }
__host__ __device__ __forceinline__ dfloat operator-(dfloat x, dfloat y) { return dfo::add(x, dfo::neg(y)); }
__host__ __device__ __forceinline__ dfloat operator-(dfloat x) { return dfo::neg(x); }
__host__ __device__ __forceinline__ dfloat operator*(dfloat x, dfloat y) { return dfo::mul(x, y); }
__host__ __device__ __forceinline__ dfloat operator/(dfloat x, dfloat y) { return dfo::div(x, y); }
__host__ __device__ __forceinline__ dfloat &operator+=(dfloat &x, dfloat y) { return x = x + y; }
__host__ __device__ __forceinline__ dfloat &operator*=(dfloat &x, dfloat y) { return x = x * y; }

/* Dot-product accumulator: the running sum's high part is kept error-free
 * (TwoSum), product errors (TwoProd) and cross terms go to an FP32 low part,
 * renormalised once at the end (the compensated dot product of Ogita, Rump
 * and Oishi, extended to double-float operands). 12 FP32 instructions a term. */
struct DotDF {
    float hi, lo;
    __host__ __device__ __forceinline__ void zero() { hi = lo = 0.0f; }
    __host__ __device__ __forceinline__ void add(dfloat a, dfloat b)
    {
        const float p = dfo::f_mul(a.hi, b.hi);
        float e = dfo::f_fma(a.hi, b.hi, -p);
        e = dfo::f_fma(a.hi, b.lo, e);
        e = dfo::f_fma(a.lo, b.hi, e);
        float s, se;
        dfo::two_sum(hi, p, s, se);
        hi = s;
        lo = dfo::f_add(lo, dfo::f_add(se, e));
    }
    __host__ __device__ __forceinline__ dfloat value() const { return dfo::fast_two_sum(hi, lo); }
};
