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

// FP32 forms, LJ pairs closer than sigma: sigma^2, 4 eps and the shift as
// double-float (the repulsive term reaches 1e4 K there, where FP32 rounding
// would leave ~1e-2 K).
struct PairCloseFF {
    float sig2h, sig2l, eps4h, eps4l, shifth, shiftl, dvdrc, pad;
};

// pairEnergy (lennard_jones.cc:70-86) in double-float from r^2 (trunc: the
// alea truncation code; the shift is 0 for plain truncation).
// r^2 is clamped from below at 1e-4 sigma^2 (r >= 0.01 sigma): closer, (sigma/r)^12
// would overflow FP32 and the double-float products turn inf - inf into NaN. The
// clamped energy is still above 1e26 K, so its Boltzmann factor is 0 as the exact
// one is, and every acceptance decision and weight is unchanged.
__device__ __forceinline__ ff lj_close_ff(const PairCloseFF& q, ff rr, float rcf, int trunc) {
    const float floor2 = 1e-4f * q.sig2h;
    if (!(rr.hi >= floor2)) rr = ff{floor2, 0.f};
    const ff s2 = ff_mul(ff{q.sig2h, q.sig2l}, ff_rcp(rr));
    const ff s6 = ff_mul(ff_mul(s2, s2), s2);
    ff e = ff_mul(ff{q.eps4h, q.eps4l}, ff_mul(s6, ff_add(s6, ff{-1.f, 0.f})));
    e = ff_add(e, ff{-q.shifth, -q.shiftl});
    if (trunc == ALEA_LINEAR_FORCE_SHIFTED) e = ff_add_f(e, -(sqrtf(rr.hi) - rcf) * q.dvdrc);
    return e;
}

// A displacement (double-float per component) brought to its image within a
// cutoff rc <= L_perp/2: the lattice shifts are chosen from the hi parts in
// FP32 (any pair within rc has a clear choice) and taken off in double-float,
// so the result keeps ~48 bits however far the image moved. lh/ll: the rows
// a_i as hi + lo (row-major 3x3), inv: the inverse (f = d . inv), ortho: the
// cell is orthorhombic.
__device__ __forceinline__ void ff_min_image(const float* lh, const float* ll, const float* inv,
                                             int ortho, ff& x, ff& y, ff& z) {
    if (ortho) {
        const float n0 = rintf(x.hi * inv[0]), n1 = rintf(y.hi * inv[4]), n2 = rintf(z.hi * inv[8]);
        x = ff_add(x, ff_scale(-n0, ff{lh[0], ll[0]}));
        y = ff_add(y, ff_scale(-n1, ff{lh[4], ll[4]}));
        z = ff_add(z, ff_scale(-n2, ff{lh[8], ll[8]}));
        return;
    }
    float n[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) n[a] = rintf(fmaf(x.hi, inv[a], fmaf(y.hi, inv[3 + a], z.hi * inv[6 + a])));
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        x = ff_add(x, ff_scale(-n[a], ff{lh[3 * a], ll[3 * a]}));
        y = ff_add(y, ff_scale(-n[a], ff{lh[3 * a + 1], ll[3 * a + 1]}));
        z = ff_add(z, ff_scale(-n[a], ff{lh[3 * a + 2], ll[3 * a + 2]}));
    }
}

}  // namespace alea
