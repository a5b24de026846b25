// ff.cuh -- double-float arithmetic: a value as an unevaluated sum hi + lo of
// two floats (about 48 significant bits).
//
// GB300 runs FP64 at 1/64 of its FP32 rate (1.24 vs 78 TFLOP/s measured), so
// the quantities that need more than FP32 -- 1 - cos(theta) and sin(theta/2)
// for small scattering angles, where the Gaussian q resolution amplifies
// relative error several hundredfold -- are carried as float pairs.  The
// algorithms are the classical error-free transformations: Knuth's TwoSum,
// Dekker's FastTwoSum, TwoProduct through a fused multiply-add, and one
// Newton correction for quotient and square root.  Only additions and
// explicit fmaf appear where the error terms are formed, so FMA contraction
// cannot change them.
#pragma once

#include <cuda_runtime.h>

namespace xrdt {

struct ff {
    float hi, lo;
};

__host__ __device__ inline ff ff_from_double(double d)
{
    const float h = (float)d;
    return {h, (float)(d - (double)h)};
}

__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ ff fast_two_sum(float a, float b)
{
    const float s = a + b;
    return {s, b - (s - a)};
}

__device__ __forceinline__ ff two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ ff ff_add(ff a, ff b)
{
    ff s = two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ ff ff_neg(ff a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

// exact float minus a pair
__device__ __forceinline__ ff ff_fsub(float a, ff b)
{
    ff s = two_sum(a, -b.hi);
    s.lo -= b.lo;
    return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ ff ff_mul(ff a, ff b)
{
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}

__device__ __forceinline__ ff ff_mulf(ff a, float b)
{
    const float p = a.hi * b;
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    return fast_two_sum(p, e);
}

__device__ __forceinline__ ff ff_sqr(ff a)
{
    const float p = a.hi * a.hi;
    float e = fmaf(a.hi, a.hi, -p);
    e = fmaf(2.0f * a.hi, a.lo, e);
    return fast_two_sum(p, e);
}

// a / b: one correction of the float quotient
__device__ __forceinline__ ff ff_div(ff a, ff b)
{
    const float q1 = a.hi / b.hi;
    const ff r = ff_sub(a, ff_mulf(b, q1));
    const float q2 = r.hi / b.hi;
    return fast_two_sum(q1, q2);
}

// sqrt(a), a > 0: one Newton correction of the float root
__device__ __forceinline__ ff ff_sqrt(ff a)
{
    const float x = sqrtf(a.hi);
    const float p = x * x;
    const float e = fmaf(x, x, -p);
    const float r = ((a.hi - p) - e + a.lo) / (2.0f * x);
    return fast_two_sum(x, r);
}

} // namespace xrdt
