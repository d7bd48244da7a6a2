// ff.cuh -- float-float ("double-single") arithmetic on the FP32 pipes.
//
// GB300's FP64 rate is a small fraction of its FP32 rate, so residuals that need
// more than FP32 precision are accumulated as unevaluated sums hi + lo of two
// floats (Dekker / Knuth error-free transformations). All operations use
// explicit fmaf/__fadd_rn so the compiler cannot contract or reassociate them.
#pragma once

namespace tk {

struct ff
{
    float hi, lo;
};

__device__ __forceinline__ ff ff_zero() { return ff{0.f, 0.f}; }

// exact a*b = p + e
__device__ __forceinline__ ff two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    const float e = fmaf(a, b, -p);
    return ff{p, e};
}

// exact a+b = s + e (Knuth)
__device__ __forceinline__ ff two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return ff{s, e};
}

__device__ __forceinline__ ff fast_two_sum(float a, float b)  // |a| >= |b|
{
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return ff{s, e};
}

__device__ __forceinline__ ff ff_add(ff a, ff b)
{
    ff s = two_sum(a.hi, b.hi);
    const float lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return fast_two_sum(s.hi, lo);
}

// acc += (ah + al) * (bh + bl), dropping al*bl
__device__ __forceinline__ ff ff_fma(ff acc, float ah, float al, float bh, float bl)
{
    ff p = two_prod(ah, bh);
    p.lo = fmaf(ah, bl, fmaf(al, bh, p.lo));
    return ff_add(acc, p);
}

__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ ff ff_shfl_xor(ff a, int m)
{
    return ff{__shfl_xor_sync(0xffffffffu, a.hi, m), __shfl_xor_sync(0xffffffffu, a.lo, m)};
}

} // namespace tk
