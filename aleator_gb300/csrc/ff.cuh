// Two-float ("double-float") arithmetic on sm_103a: a value is hi + lo with
// |lo| <= ulp(hi) / 2, about 48 significant bits, at FP32 instruction rates
// (FP64 issues at a small fraction of the FP32 rate on this part). Error-free
// transformations: Knuth two-sum and the FMA two-product; the _rn intrinsics
// keep the compiler from contracting or reassociating them.
#pragma once

namespace alea {

struct ff {
    float hi, lo;
};
__device__ __forceinline__ ff ff_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
__device__ __forceinline__ ff ff_fast(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    ff s = ff_two_sum(a.hi, b.hi);
    s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return ff_fast(s.hi, s.lo);
}
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
    return ff_fast(p, e);
}
__device__ __forceinline__ ff ff_rcp(ff a) {  // one Newton step from the FP32 reciprocal
    const float y = __frcp_rn(a.hi);
    const ff ay = ff_mul(a, ff{y, 0.f});
    const ff r = ff_add(ff{1.f, 0.f}, ff{-ay.hi, -ay.lo});
    const ff c = ff_mul(ff{y, 0.f}, r);
    return ff_add(ff{y, 0.f}, c);
}
// s * v for an FP32 scalar s and a double-float v.
__device__ __forceinline__ ff ff_scale(float s, ff v) { return ff_mul(ff{s, 0.f}, v); }
// a + b for a double-float a and an FP32 b.
__device__ __forceinline__ ff ff_add_f(ff a, float b) {
    ff s = ff_two_sum(a.hi, b);
    s.lo = __fadd_rn(s.lo, a.lo);
    return ff_fast(s.hi, s.lo);
}
// hi + lo split of a double (lo rounded)
__host__ __device__ __forceinline__ ff ff_from(double v) {
    const float h = (float)v;
    return ff{h, (float)(v - (double)h)};
}

}  // namespace alea
