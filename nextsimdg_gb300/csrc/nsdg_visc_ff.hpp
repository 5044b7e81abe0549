// The mixed-precision viscosity P/(8 alpha Delta), Delta = sqrt(inv + DeltaMin^2)
// (MEVPStressUpdateStep.hpp:63-77, 92-116), in two forms that share one FP32
// seed y0 ~ 1/sqrt(inv + DeltaMin^2):
//
//   viscNewton64  one Newton-Raphson step for 1/sqrt(t) in FP64,
//                 y1 = y0 + y0 (1 - t y0^2) / 2, z = Pa y1, rounded to FP32
//                 (the device kernels' five-FP64-instruction form; this is
//                 a host replica, operation for operation, for checks);
//   viscFloatFloat (host and device) the same Newton step with t, y1 and
//                 Pa carried as unevaluated pairs of floats (hi + lo, about
//                 48 significant bits): error-free sums and products (Knuth's
//                 TwoSum, the FMA-based TwoProduct, as in Dekker's
//                 double-float arithmetic) on the FP32 pipe and one FP64
//                 subtraction for the low part of Pa.
//
//   viscFloatFloatChecked (host and device) the float-float form with the
//                 last sum kept as an exact pair, and a flag telling whether
//                 the result is provably the FP64 form's: the device kernels'
//                 form 4 uses it and evaluates the FP64 form only where the
//                 flag is false, so their results are bitwise form 2's.
//
// Both approximate the same y1 from the same seed, so they round to the same
// float unless Pa y1 lies within about 2^-44 of a rounding midpoint.  Every
// FP32 operation is an explicit IEEE round-to-nearest operation (no
// contraction on either compiler); host builds that use this header must also
// compile with -ffp-contract=off.  float <-> double conversions work on the
// bit patterns (exponent rebias), as on the device, where FP64 conversions
// issue at the FP64 rate.
#pragma once

#include <cstdint>
#include <cstring>
#include <cmath>

#if defined(__CUDACC__)
#define NSDG_FF_HD __host__ __device__ __forceinline__
#else
#define NSDG_FF_HD inline
#endif

namespace nsdg_ff {

NSDG_FF_HD uint32_t bitsOf(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    std::memcpy(&u, &f, sizeof u);
    return u;
#endif
}
NSDG_FF_HD float floatOf(uint32_t u)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, sizeof f);
    return f;
#endif
}
NSDG_FF_HD uint64_t bitsOf(double d)
{
#if defined(__CUDA_ARCH__)
    return static_cast<uint64_t>(__double_as_longlong(d));
#else
    uint64_t u;
    std::memcpy(&u, &d, sizeof u);
    return u;
#endif
}
NSDG_FF_HD double doubleOf(uint64_t u)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double(static_cast<long long>(u));
#else
    double d;
    std::memcpy(&d, &u, sizeof d);
    return d;
#endif
}

// IEEE binary32 operations, round to nearest even, never fused
NSDG_FF_HD float add(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
NSDG_FF_HD float sub(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
NSDG_FF_HD float mul(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
NSDG_FF_HD float fma(float a, float b, float c)
{
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fmaf(a, b, c);
#endif
}

// positive normal float -> double (exact)
NSDG_FF_HD double widenPos(float f)
{
    return doubleOf((static_cast<uint64_t>(bitsOf(f)) << 29) + (896ull << 52));
}
// f / 2 for a positive normal float f (exact)
NSDG_FF_HD double widenHalfPos(float f)
{
    return doubleOf((static_cast<uint64_t>(bitsOf(f)) << 29) + (895ull << 52));
}
// non-negative float -> double; subnormal floats become 0
NSDG_FF_HD double widenNonneg(float f)
{
    return bitsOf(f) >= 0x00800000u ? widenPos(f) : 0.0;
}
// 0 <= d < 2^128 -> nearest float (ties away from zero); 0 below the
// smallest normal float
NSDG_FF_HD float narrowPos(double d)
{
    const int64_t b = static_cast<int64_t>(bitsOf(d));
    const int64_t r = (b - (896ll << 52) + (1ll << 28)) >> 29;
    return b >= (897ll << 52) ? floatOf(static_cast<uint32_t>(r)) : 0.f;
}
// any double -> nearest float (ties away from zero); magnitudes below the
// smallest normal float become a signed zero, beyond the largest an infinity
NSDG_FF_HD float narrowAny(double d)
{
    const uint64_t b = bitsOf(d);
    const uint64_t mag = b & 0x7fffffffffffffffull;
    const uint32_t sign = static_cast<uint32_t>(b >> 32) & 0x80000000u;
    if (mag < (897ull << 52))
        return floatOf(sign);
    if (mag >= 0x47effffff0000000ull)
        return floatOf(sign | (mag > 0x7ff0000000000000ull ? 0x7fc00000u : 0x7f800000u));
    return floatOf(sign | static_cast<uint32_t>((mag - (896ull << 52) + (1ull << 28)) >> 29));
}

// The FP64 form: t = inv + DeltaMin^2 with one rounding (FMA), one Newton
// step from the seed y0 (a positive normal float), z = Pa y1 rounded to FP32.
// Host only: the device kernels carry their own copy of these operations.
inline float viscNewton64(float inv, double Pa, double dmin, float y0)
{
    const double td = widenNonneg(inv);
    const double t = std::fma(dmin, dmin, td);
    const double yd = widenPos(y0);
    const double yh = widenHalfPos(y0);
    const double h = t * yd;
    const double e2 = std::fma(-h, yh, 0.5); // (1 - t y0^2) / 2
    const double z = Pa * yd;
    const double z8 = std::fma(z, e2, z);
    return narrowPos(z8);
}

// The float-float form.  d2h + d2l: DeltaMin^2 as a pair of floats (d2h the
// nearest float, d2l the nearest float to the rest); y0 the same seed.
NSDG_FF_HD float viscFloatFloat(float inv, double Pa, float d2h, float d2l, float y0)
{
    // t = th + tl: TwoSum of inv and d2h, then the low part of DeltaMin^2
    const float th = add(inv, d2h);
    const float bv = sub(th, inv);
    const float av = sub(th, bv);
    const float tl = add(add(sub(inv, av), sub(d2h, bv)), d2l);
    // r = 1 - t y0^2 from y0^2 = p + pe and th p = q + qe (both exact);
    // 1 - q is exact (q is within 2^-20 of 1)
    const float p = mul(y0, y0);
    const float pe = fma(y0, y0, -p);
    const float q = mul(th, p);
    const float qe = fma(th, p, -q);
    const float r = fma(-tl, p, fma(-th, pe, sub(sub(1.f, q), qe)));
    // y1 = y0 + yl
    const float yl = mul(mul(y0, r), 0.5f);
    // Pa = ph + pl (the difference is exact in FP64), Pa below 2^-100 scaled
    // by 2^64 first so that pl stays a normal float (FP64 subnormals count
    // as 0); then (ph + pl)(y0 + yl) with ph y0 = m + me exactly
    const uint64_t pb = bitsOf(Pa);
    const bool tiny = pb < (923ull << 52);
    const double ps = !tiny ? Pa : (pb >= (1ull << 52) ? doubleOf(pb + (64ull << 52)) : 0.0);
    const float ph = narrowPos(ps);
    const float pl = narrowAny(ps - widenNonneg(ph));
    const float m = mul(ph, y0);
    const float me = fma(ph, y0, -m);
    float z = add(m, fma(ph, yl, fma(pl, y0, me)));
    if (tiny)
        z = mul(z, 0x1p-64f);
    // results below the smallest normal float are 0, as the FP64 form's
    // conversion to float makes them
    return z >= 0x1p-126f ? z : 0.f;
}

// The float-float form with a check that its result is bitwise the FP64
// form's (viscNewton64 with the same seed).  Error bounds, relative to z, for
// a seed with |r| = |1 - t y0^2| <= 2^-19 (rsqrtf's seed: about 2^-21):
//   the pair m + s (before its last rounding) is within 2^-41 of the exact
//   Newton value Pa y0 (1 + r / 2): r carries three roundings of at most
//   2^-43 (its terms are below 2^-19) and the dropped tl pe (2^-48), which
//   reach y1 halved (2^-42.4); y0 r / 2 one rounding of 2^-44; s one of
//   2^-43.8; the dropped pl yl at most 2^-44; the pair splits of Pa and
//   DeltaMin^2 at most 2^-48 each (for Pa >= 2^-76: below, pl could be
//   flushed to 0);
//   the FP64 form's z8 is within 2^-51 of the same value (four FP64
//   roundings; the seed's widening is exact).
// Hence if m + s = z + err (exact, Fast2Sum) lies farther than 2^-39 |z|
// inside the interval of reals that round to z, z8 rounds to z as well:
// `exact` is true and z is the FP64 form's result.  Otherwise `exact` is
// false and the caller evaluates the FP64 form: z within 2^-39 of a
// rounding boundary (about 2^-15 of random cases), z a power of two, z below
// 2^-80 or not finite, Pa below 2^-76 and not zero, or a seed outside the
// bound.  Pa = 0 gives +0, as the FP64 form does.
NSDG_FF_HD float viscFloatFloatChecked(float inv, double Pa, float d2h, float d2l, float y0, bool& exact)
{
    exact = false;
    const uint64_t pb = bitsOf(Pa);
    if (pb == 0) {
        exact = true;
        return 0.f;
    }
    // Pa >= 2^-76: then the low part pl, flushed to 0 below 2^-126, loses at
    // most 2^-50 of Pa
    if (pb < (947ull << 52) || pb >= (1ull << 63))
        return 0.f;
    const float th = add(inv, d2h);
    const float bv = sub(th, inv);
    const float av = sub(th, bv);
    const float tl = add(add(sub(inv, av), sub(d2h, bv)), d2l);
    const float p = mul(y0, y0);
    const float pe = fma(y0, y0, -p);
    const float q = mul(th, p);
    const float qe = fma(th, p, -q);
    const float r = fma(-tl, p, fma(-th, pe, sub(sub(1.f, q), qe)));
    if (!(r <= 0x1p-19f && r >= -0x1p-19f))
        return 0.f;
    const float yl = mul(mul(y0, r), 0.5f);
    const float ph = narrowPos(Pa);
    const float pl = narrowAny(Pa - widenNonneg(ph));
    const float m = mul(ph, y0);
    const float me = fma(ph, y0, -m);
    const float s = fma(ph, yl, fma(pl, y0, me));
    const float z = add(m, s);
    const float err = sub(s, sub(z, m)); // m + s = z + err exactly: |s| < 2^-18 |m|
    const uint32_t zb = bitsOf(z);
    const uint32_t ex = zb & 0x7f800000u;
    if (ex < (47u << 23) || ex == 0x7f800000u || (zb & 0x007fffffu) == 0u)
        return z;
    // z in (2^e, 2^(e+1)): the reals that round to z lie within 2^(e-24) of
    // it; the margin 2^(e-38) is at least 2^-39 |z|
    const float half = floatOf(ex - (24u << 23));
    const float margin = floatOf(ex - (38u << 23));
    const float aerr = err < 0.f ? -err : err;
    exact = aerr < sub(half, margin);
    return z;
}

// DeltaMin^2 as the pair (d2h, d2l) viscFloatFloat takes: d2h the float the
// kernels' launch parameters hold (DeltaMin^2 rounded to nearest even), d2l
// the rest, DeltaMin^2 - d2h formed exactly by one FMA.  Host only; the
// device forms d2l from the same operations.
inline void splitSquare(double dmin, float& d2h, float& d2l)
{
    d2h = static_cast<float>(dmin * dmin);
    d2l = narrowAny(std::fma(dmin, dmin, -widenPos(d2h)));
}

} // namespace nsdg_ff
