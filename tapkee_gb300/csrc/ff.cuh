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

__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }

// a * b, dropping a.lo * b.lo
__device__ __forceinline__ ff ff_mul(ff a, ff b)
{
    ff p = two_prod(a.hi, b.hi);
    p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
    return fast_two_sum(p.hi, p.lo);
}

// a / n for a float n (one correction step: ~2^-46 relative)
__device__ __forceinline__ ff ff_div_f(ff a, float n)
{
    const float q = a.hi / n;
    const float r = fmaf(-q, n, a.hi) + a.lo;
    return fast_two_sum(q, r / n);
}

// 1 / sqrt(a) for a > 0: one Newton step from the FP32 estimate (~2^-44)
__device__ __forceinline__ ff ff_rsqrt(ff a)
{
    const float y = rsqrtf(a.hi);
    const ff yy = two_prod(y, y);
    const ff e = ff_add(ff{1.f, 0.f}, ff_neg(ff_mul(a, yy)));  // 1 - a y^2
    return fast_two_sum(y, 0.5f * y * (e.hi + e.lo));
}

__device__ __forceinline__ ff ff_shfl_xor(ff a, int m)
{
    return ff{__shfl_xor_sync(0xffffffffu, a.hi, m), __shfl_xor_sync(0xffffffffu, a.lo, m)};
}

} // namespace tk
