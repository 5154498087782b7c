// Float-float arithmetic for the FP64-quality translations on the FP32 pipes (GB300's FP64
// rate is a 64th of its FP32 rate).  A value is the unevaluated sum hi + lo of two FP32 numbers
// with |lo| <= ulp(hi) / 2: about 48 significant bits, with FP32's exponent range.
//
// The operations are built from the classical error-free transformations: Knuth's TwoSum
// (s + e = a + b exactly), Dekker's FastTwoSum (the same for |a| >= |b|) and the FMA form of
// Dekker's TwoProd (p + e = a b exactly), combined as the double-word algorithms of Joldes,
// Muller and Popescu, "Tight and rigorous error bounds for basic building blocks of double-word
// arithmetic" (ACM TOMS 44, 2017): addition with both parts' errors carried (their accurate
// sum, relative error below 3 u^2 with u = 2^-24) and multiplication by TwoProd of the high
// parts plus the two cross products, the product of the low parts dropped (relative error a
// few u^2).  Nothing here is reassociated (device code keeps IEEE order without fast-math), and
// no product is contracted into an FMA behind the algorithms' back: the high parts' product
// is __fmul_rn, and the only fused operations are the explicit fmaf calls.
#pragma once
#include <cuda_runtime.h>
#include "fmm_common.cuh"

namespace fmm {

// mk2 for float-float below lives in this namespace (so that the complex helpers of
// fmm_common.cuh find it by argument-dependent lookup); the FP32 / FP64 overloads stay visible
using ::mk2;

struct ff {
    float hi, lo;
    ff() = default;
    __host__ __device__ constexpr ff(float v) : hi(v), lo(0.f) {}
    __host__ __device__ constexpr ff(float h, float l) : hi(h), lo(l) {}
};

struct ff2 {
    ff x, y;
};

__device__ __forceinline__ void ff_two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void ff_fast_two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    e = b - (s - a);
}

__device__ __forceinline__ ff operator+(ff a, ff b)
{
    float s, e, t, f;
    ff_two_sum(a.hi, b.hi, s, e);
    ff_two_sum(a.lo, b.lo, t, f);
    e += t;
    ff_fast_two_sum(s, e, s, e);
    e += f;
    ff_fast_two_sum(s, e, s, e);
    return ff(s, e);
}

__device__ __forceinline__ ff operator-(ff a) { return ff(-a.hi, -a.lo); }
__device__ __forceinline__ ff operator-(ff a, ff b) { return a + (-b); }

__device__ __forceinline__ ff operator*(ff a, ff b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    float s, t;
    ff_fast_two_sum(p, e, s, t);
    return ff(s, t);
}

__device__ __forceinline__ ff &operator+=(ff &a, ff b)
{
    a = a + b;
    return a;
}

// c + a b for the accumulations of the translations: TwoProd of the high parts with the two
// cross products, then one TwoSum of the high parts with the low parts and the product's error
// added without their own TwoSum (Dekker's "sloppy" addition, 15 FP32 instructions against 27
// for the product and the accurate sum above).  Its error is bounded relative to |c| + |a b|,
// not to |c + a b|: a sum of n such terms is accurate to about n 2^-47 of the sum of the terms'
// magnitudes, the same form of bound as FP64 summation (n 2^-53).
__device__ __forceinline__ ff ff_fma(ff a, ff b, ff c)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    float s, t;
    ff_two_sum(c.hi, p, s, t);
    t = __fadd_rn(t, __fadd_rn(c.lo, e));
    ff_fast_two_sum(s, t, s, t);
    return ff(s, t);
}

__device__ __forceinline__ ff2 mk2(ff a, ff b) { return ff2{a, b}; }

// nearest float-float to a double, and back
__device__ __forceinline__ ff ff_from(double d)
{
    const float h = (float)d;
    return ff(h, (float)(d - (double)h));
}
__device__ __forceinline__ double ff_to(ff a) { return (double)a.hi + (double)a.lo; }

} // namespace fmm
