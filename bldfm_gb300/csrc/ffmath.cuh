// Float-float ("double-FP32") arithmetic on the FP32 pipe: a value is the
// unevaluated sum hi + lo of two floats with |lo| <= ulp(hi) / 2, about 48
// bits of significand.  Used where a result must be checked against a
// reference more accurate than FP32 without the FP64 pipe, which runs at
// 1/64 of the FP32 rate on GB300.  Algorithms: Knuth's TwoSum, the FMA
// TwoProduct, and the accurate sum of Hida, Li and Bailey (the same ones as
// the host's double-double code).  Every operation is an explicit
// round-to-nearest intrinsic, so the compiler neither contracts nor
// reorders it.
#pragma once

struct ff {
    float hi, lo;
};
struct cff {
    ff re, im;
};

__device__ __forceinline__ ff ff_from(float x) { return {x, 0.f}; }

// exact conversion of a double to a float pair (hi + lo equals d to ~2^-48)
__device__ __forceinline__ ff ff_from_double(double d)
{
    const float h = __double2float_rn(d);
    return {h, __double2float_rn(d - (double)h)};
}

__device__ __forceinline__ ff ff_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

__device__ __forceinline__ ff ff_quick(float s, float e)
{
    const float h = __fadd_rn(s, e);
    return {h, __fsub_rn(e, __fsub_rn(h, s))};
}

__device__ __forceinline__ ff ff_add(ff a, ff b)
{
    const ff s = ff_two_sum(a.hi, b.hi), t = ff_two_sum(a.lo, b.lo);
    ff r = ff_quick(s.hi, __fadd_rn(s.lo, t.hi));
    return ff_quick(r.hi, __fadd_rn(r.lo, t.lo));
}

__device__ __forceinline__ ff ff_neg(ff a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

__device__ __forceinline__ ff ff_mul(ff a, ff b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
    return ff_quick(p, e);
}

// a / b: quotient of the leading parts, corrected once by the remainder
__device__ __forceinline__ ff ff_div(ff a, ff b)
{
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const ff r = ff_sub(a, ff_mul(b, ff_from(q1)));
    const float q2 = __fdiv_rn(r.hi, b.hi);
    const ff q = ff_quick(q1, q2);
    const ff r2 = ff_sub(a, ff_mul(b, q));
    return ff_add(q, ff_from(__fdiv_rn(r2.hi, b.hi)));
}

// sqrt(a), a >= 0: one Newton correction of the float root
__device__ __forceinline__ ff ff_sqrt(ff a)
{
    if (!(a.hi > 0.f)) return {0.f, 0.f};
    const float s = __fsqrt_rn(a.hi);
    const ff r = ff_sub(a, ff_mul(ff_from(s), ff_from(s)));
    return ff_quick(s, __fdiv_rn(r.hi, __fmul_rn(2.f, s)));
}

__device__ __forceinline__ cff cff_add(cff a, cff b) { return {ff_add(a.re, b.re), ff_add(a.im, b.im)}; }
__device__ __forceinline__ cff cff_sub(cff a, cff b) { return {ff_sub(a.re, b.re), ff_sub(a.im, b.im)}; }
__device__ __forceinline__ cff cff_mul(cff a, cff b)
{
    return {ff_sub(ff_mul(a.re, b.re), ff_mul(a.im, b.im)), ff_add(ff_mul(a.re, b.im), ff_mul(a.im, b.re))};
}
__device__ __forceinline__ ff cff_norm2(cff a) { return ff_add(ff_mul(a.re, a.re), ff_mul(a.im, a.im)); }
// a / b as a conj(b) / |b|^2 (out of line: the accuracy check calls it in
// several places, and its code inlined at each pushed the check kernel out
// of the instruction cache)
__device__ __noinline__ cff cff_div(cff a, cff b)
{
    const ff n = cff_norm2(b);
    const cff t = cff_mul(a, cff{b.re, ff_neg(b.im)});
    return {ff_div(t.re, n), ff_div(t.im, n)};
}
// principal square root (Kahan's formulation)
__device__ __forceinline__ cff cff_sqrt(cff w)
{
    const ff ax = w.re.hi < 0.f ? ff_neg(w.re) : w.re;
    const ff t = ff_sqrt(ff_mul(ff_from(0.5f), ff_add(ax, ff_sqrt(cff_norm2(w)))));
    if (t.hi == 0.f) return {{0.f, 0.f}, {0.f, 0.f}};
    const ff t2 = ff_mul(ff_from(2.f), t);
    if (w.re.hi >= 0.f) return {t, ff_div(w.im, t2)};
    const ff ay = w.im.hi < 0.f ? ff_neg(w.im) : w.im;
    return {ff_div(ay, t2), w.im.hi < 0.f ? ff_neg(t) : t};
}
