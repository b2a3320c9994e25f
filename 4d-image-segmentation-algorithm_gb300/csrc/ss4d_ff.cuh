// ss4d_ff.cuh — float-float arithmetic (an unevaluated sum h + l of two
// floats, about 48 significant bits) on the FP32 pipe: Dekker's and Knuth's
// error-free transformations (the rounding error of a float sum by Knuth's
// two-sum, that of a product by one fused multiply-add), conversions to and
// from double by integer operations, and float2 storage.  Used where FP64
// accuracy is needed but GB300's FP64 rate (about 1/64 of FP32) would bound
// the kernel: the mixed form's coefficient assembly and edge detector.
#pragma once

#include "ss4d_sweep.cuh"

namespace ss4d {
namespace ffa {

struct ff {
    float h, l;
};

__device__ __forceinline__ ff ff_make(float h, float l)
{
    ff r;
    r.h = h;
    r.l = l;
    return r;
}

// |a| >= |b| (or a == 0): s + e == a + b exactly
__device__ __forceinline__ ff fast_two_sum(float a, float b)
{
    const float s = a + b;
    return ff_make(s, b - (s - a));
}

__device__ __forceinline__ ff two_sum(float a, float b)
{
    const float s = a + b;
    const float v = s - a;
    return ff_make(s, (a - (s - v)) + (b - v));
}

__device__ __forceinline__ ff ff_add(ff a, ff b)
{
    ff s = two_sum(a.h, b.h);
    const float e = s.l + (a.l + b.l);
    return fast_two_sum(s.h, e);
}

// a + b keeping the rounding error of the high parts in the low part
// without renormalising: for operands that do not cancel (sums of positive
// terms, or a sum whose result is added again) the low part stays within a
// few units of 2^-24 of the high part
__device__ __forceinline__ ff ff_add_nr(ff a, ff b)
{
    ff s = two_sum(a.h, b.h);
    s.l += a.l + b.l;
    return s;
}

__device__ __forceinline__ ff ff_norm(ff a)
{
    return fast_two_sum(a.h, a.l);
}

__device__ __forceinline__ ff ff_mul(ff a, ff b)
{
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return fast_two_sum(p, e);
}

__device__ __forceinline__ ff ff_sqr(ff a)
{
    const float p = a.h * a.h;
    float e = fmaf(a.h, a.h, -p);
    e = fmaf(2.f * a.h, a.l, e);
    return fast_two_sum(p, e);
}

// double -> float-float by integer operations (no FP64 instruction): the high
// part is d truncated to 24 significant bits; the remainder d - h is the low
// 29 mantissa bits r times 2^(e - 1075), converted to float by truncation.
// The low part is dropped (left zero) where that scale is below the FP32
// normal range, i.e. for |d| < 2^-73.
__device__ __forceinline__ ff ff_from_d(double d)
{
    const float h = d2f_bits(d);
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const int e = (int)((hi >> 20) & 0x7FFu);
    const unsigned r = lo & 0x1FFFFFFFu;
    const int fe = e - 948; // FP32 biased exponent of 2^(e - 1075)
    float l = 0.f;
    if (r != 0u && fe >= 1 && e <= 1150) {
        l = __uint2float_rz(r) * __uint_as_float((unsigned)fe << 23);
        if (hi & 0x80000000u)
            l = -l;
    }
    return ff_make(h, l);
}

// ff_from_d for a positive double in [2^-74, 2^127) (the range of the edge
// detector's g = 1 / (1 + K x) in (0, 1]): the same pair by fewer integer
// operations (the high part's bits in one funnel shift); any other value
// takes ff_from_d
__device__ __forceinline__ ff ff_from_pos_d(double d)
{
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const unsigned e = hi >> 20; // biased exponent; the sign bit makes it >= 2048
    if (e - 949u > 1150u - 949u)
        return ff_from_d(d);
    const float h = __uint_as_float(__funnelshift_l(lo, hi - (896u << 20), 3));
    const float l = __uint2float_rz(lo & 0x1FFFFFFFu) * __uint_as_float((e - 948u) << 23);
    return ff_make(h, l);
}

__device__ __forceinline__ double ff_to_d(ff a)
{
    return f2d_bits(a.h) + f2d_bits(a.l);
}

// 1/sqrt(x), x > 0 and normal: FP32 seed y0 (relative error below 2^-21),
// one Newton step y = y0 + y0 (1 - x y0^2) / 2 with x y0^2 formed exactly
// enough (y0^2 as an exact pair, its product with x to float-float): error
// about 1.5 e0^2
__device__ __forceinline__ ff ff_rsqrt(ff x)
{
    const float y0 = rsqrtf(x.h);
    const float p = y0 * y0, pe = fmaf(y0, y0, -p); // y0^2 = p + pe exactly
    const float q = x.h * p;
    float qe = fmaf(x.h, p, -q);
    qe = fmaf(x.h, pe, qe);
    qe = fmaf(x.l, p, qe);                          // x y0^2 = q + qe
    const float hr = 0.5f * ((1.f - q) - qe);       // 1 - q is exact (q near 1)
    const float c = y0 * hr, ce = fmaf(y0, hr, -c); // y0 hr = c + ce exactly
    ff y = fast_two_sum(y0, c);
    y.l += ce;
    return y;
}

__device__ __forceinline__ ff ld_ff(const double *p, long long o)
{
    const float2 v = __ldg(reinterpret_cast<const float2 *>(p) + o);
    return ff_make(v.x, v.y);
}

__device__ __forceinline__ void st_ff(double *p, long long o, ff v)
{
    __stcs(reinterpret_cast<float2 *>(p) + o, make_float2(v.h, v.l));
}


__device__ __forceinline__ ff ff_neg(ff a)
{
    return ff_make(-a.h, -a.l);
}

// 1/x for normal x: FP32 seed y0 = 1/x.h (correctly rounded), one Newton
// step y = y0 + y0 (1 - x y0) with x y0 formed to float-float: error about e0^2
__device__ __forceinline__ ff ff_rcp(ff x)
{
    const float y0 = __frcp_rn(x.h);
    const float q = x.h * y0;
    float qe = fmaf(x.h, y0, -q);
    qe = fmaf(x.l, y0, qe);                // x y0 = q + qe
    const float r = (1.f - q) - qe;        // 1 - q is exact (q near 1)
    const float c = y0 * r, ce = fmaf(y0, r, -c);
    ff y = fast_two_sum(y0, c);
    y.l += ce;
    return y;
}

__device__ __forceinline__ ff ld_ff2(const float2 *p, long long o)
{
    const float2 v = p[o];
    return ff_make(v.x, v.y);
}

__device__ __forceinline__ void st_ff2(float2 *p, long long o, ff v)
{
    p[o] = make_float2(v.h, v.l);
}

} // namespace ffa
} // namespace ss4d
