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

// sqrt(a) for a > 0: the FP32 root and one Newton step, (a - s^2) / (2 s)
// with s^2 = p + pe exactly.
__device__ __forceinline__ ff ff_sqrt(ff a) {
    const float s = sqrtf(a.hi);
    const float p = __fmul_rn(s, s);
    const float pe = __fmaf_rn(s, s, -p);
    const float d = __fdiv_rn(__fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), pe), a.lo), __fmul_rn(2.f, s));
    return ff_fast(s, d);
}

// d_n = (-1)^n (2 / sqrt(pi)) 4^n / (n! (2n + 1)) as (hi, lo) FP32 pairs:
// erf(x) = x sum_n d_n (x^2 / 4)^n (the Maclaurin series, Abramowitz and
// Stegun 7.1.5, in w = x^2 / 4 so that the coefficients stay near 1).
static __device__ __constant__ float2 kErfSeries[30] = {
    {0x1.20dd760000000p+0f, -0x1.f7ac920000000p-25f},
    {-0x1.8127460000000p+0f, -0x1.606f3c0000000p-25f},
    {0x1.ce2f220000000p+0f, -0x1.7ef5080000000p-26f},
    {-0x1.b82ce40000000p+0f, 0x1.daee960000000p-25f},
    {0x1.565bce0000000p+0f, -0x1.e32b580000000p-25f},
    {-0x1.c02db40000000p-1f, -0x1.02e1620000000p-35f},
    {0x1.f9a3260000000p-2f, 0x1.f371360000000p-27f},
    {-0x1.f4d25c0000000p-3f, -0x1.f061760000000p-30f},
    {0x1.b9e6ca0000000p-4f, -0x1.1cd72e0000000p-31f},
    {-0x1.5f742e0000000p-5f, -0x1.887ce40000000p-30f},
    {0x1.fcc5720000000p-7f, 0x1.8930700000000p-37f},
    {-0x1.51d7180000000p-8f, -0x1.c5d36c0000000p-36f},
    {0x1.9e6ad60000000p-10f, -0x1.aa58d00000000p-38f},
    {-0x1.d8453c0000000p-12f, -0x1.6188de0000000p-37f},
    {0x1.f683ae0000000p-14f, 0x1.2a5c020000000p-40f},
    {-0x1.f56f080000000p-16f, 0x1.caef460000000p-41f},
    {0x1.d70b360000000p-18f, -0x1.9017140000000p-43f},
    {-0x1.a2007a0000000p-20f, -0x1.e688fe0000000p-45f},
    {0x1.5f791a0000000p-22f, -0x1.0e611e0000000p-48f},
    {-0x1.18cc8a0000000p-24f, -0x1.8711e60000000p-54f},
    {0x1.ab5cc40000000p-27f, -0x1.d6ec1a0000000p-52f},
    {-0x1.3676fc0000000p-29f, -0x1.2304d00000000p-55f},
    {0x1.af83c20000000p-32f, 0x1.f633f40000000p-57f},
    {-0x1.1f690c0000000p-34f, -0x1.593a9e0000000p-61f},
    {0x1.6f928a0000000p-37f, -0x1.10bffc0000000p-62f},
    {-0x1.c40ac00000000p-40f, 0x1.b063360000000p-69f},
    {0x1.0baeae0000000p-42f, -0x1.27dc280000000p-69f},
    {-0x1.31b7780000000p-45f, 0x1.2357dc0000000p-70f},
    {0x1.5121940000000p-48f, -0x1.06bb5a0000000p-74f},
    {-0x1.67657a0000000p-51f, -0x1.5c52280000000p-77f},
};
constexpr int kErfTerms = 30;
// Largest argument for ff_erfc: at x = 2 (w = 1) the 30 terms leave ~1e-14
// of erf, so erfc (>= 0.0047 there) keeps ~1e-12 relative.
constexpr float kErfcSeriesMax = 2.0f;

// erfc(x) = 1 - erf(x) for 0 <= x <= kErfcSeriesMax in double-float: the
// series by Horner's rule in w = x^2 / 4. The FP32 forms' near Coulomb pairs
// take their real-space term this way at FP32 instruction rates.
__device__ __forceinline__ ff ff_erfc(ff x) {
    const ff w = ff_scale(0.25f, ff_mul(x, x));
    const float2 cl = kErfSeries[kErfTerms - 1];
    ff s{cl.x, cl.y};
#pragma unroll 5
    for (int n = kErfTerms - 2; n >= 0; --n) {
        const float2 c = kErfSeries[n];
        s = ff_add(ff_mul(s, w), ff{c.x, c.y});
    }
    const ff e = ff_mul(x, s);
    return ff_add(ff{1.f, 0.f}, ff{-e.hi, -e.lo});
}

// q erfc(alpha r) / r of a near Coulomb pair from its double-float
// displacement (r above 1e-6 A) and charge; false (out untouched) when
// alpha r lies beyond the series, for the caller's FP64 evaluation.
__device__ __forceinline__ bool near_coulomb_ff(ff dx, ff dy, ff dz, ff q, ff alpha, double& out) {
    ff rr = ff_add(ff_add(ff_mul(dx, dx), ff_mul(dy, dy)), ff_mul(dz, dz));
    if (!(rr.hi > 1e-12f)) rr = ff{1e-12f, 0.f};
    const ff r = ff_sqrt(rr);
    const ff x = ff_mul(alpha, r);
    if (!(x.hi <= kErfcSeriesMax)) return false;
    const ff v = ff_mul(q, ff_mul(ff_erfc(x), ff_rcp(r)));
    out = (double)v.hi + (double)v.lo;
    return true;
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
