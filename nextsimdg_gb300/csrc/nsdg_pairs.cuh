// nsdg_pairs.cuh — float-pair ("double-float") arithmetic on the FP32 pipe,
// for kernels of the FP64 path whose FP64 work would otherwise bound them.
//
// GB300 issues FP64 at about 1/64 of the FP32 rate (about 2 FP64 FMA per SM
// per clock), so a kernel that applies 9 x 9 operators in FP64 is FP64-issue
// bound long before it is HBM bound.  Here a value is carried as an
// unevaluated sum hi + lo of two floats (about 48 significant bits) and
// products and sums are formed with error-free transformations: the
// FMA-based exact product (TwoProduct, as in Dekker's double-float
// arithmetic) and Knuth's TwoSum.  Every FP32 operation is an explicit
// round-to-nearest intrinsic (__fadd_rn, __fmul_rn, __fmaf_rn), which the
// compiler never contracts or reassociates, so the transformations stay
// error-free.
//
// Conversions between double and float pairs work on the bit patterns (the
// INT pipe), not through FP64 conversion instructions.
#pragma once

#include <cuda_runtime.h>

namespace nsdg {
namespace pairs {

struct F2 {
    float hi, lo;
};

// x = hi + lo: hi the leading 24 significant bits of x (truncated), lo the
// next 24 (the integer remainder rounded once): |x - (hi + lo)| <= 2^-47 |x|.
// Magnitudes below 2^-126 (and zero) give hi = lo = 0; the remainder of
// values below 2^-74 is dropped (its size is below 2^-97).  Non-finite values
// give a non-finite hi.
__device__ __forceinline__ F2 split(double x)
{
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    const unsigned hw = static_cast<unsigned>(b >> 32), lw = static_cast<unsigned>(b);
    const unsigned e = (hw >> 20) & 0x7ffu;
    const unsigned sign = hw & 0x80000000u;
    F2 r;
    if (e < 897u) {
        r.hi = __uint_as_float(sign);
        r.lo = r.hi;
        return r;
    }
    if (e > 1150u) { // beyond the float range, or inf / nan
        r.hi = __uint_as_float(sign | 0x7f800000u | ((hw & 0xfffffu) << 3) | (lw >> 29));
        r.lo = 0.0f;
        return r;
    }
    r.hi = __uint_as_float(sign | ((e - 896u) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29));
    const unsigned rest = lw & 0x1fffffffu; // remainder: rest * 2^(e - 1075)
    const unsigned se = e - 948u;           // exponent field of 2^(e - 1075) as a float
    const float scale = (e > 948u) ? __uint_as_float(se << 23) : 0.0f;
    r.lo = __uint_as_float(__float_as_uint(__fmul_rn(__uint2float_rn(rest), scale)) | sign);
    return r;
}

// The exact double value of a float (zero and subnormals give a signed zero).
__device__ __forceinline__ double widen(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned sign = u & 0x80000000u;
    const unsigned ex = e == 0xffu ? 0x7ffu : e + 896u;
    const unsigned hw = e == 0u ? sign : (sign | (ex << 20) | ((u & 0x7fffffu) >> 3));
    const unsigned lw = e == 0u ? 0u : (u << 29);
    return __hiloint2double(static_cast<int>(hw), static_cast<int>(lw));
}

// hi + lo as one double (one FP64 addition)
__device__ __forceinline__ double value(F2 a) { return widen(a.hi) + widen(a.lo); }

__device__ __forceinline__ F2 pairOf(float2 v) { return F2 { v.x, v.y }; }

// Fast2Sum: a + b = s + t exactly, |a| >= |b| or a == 0
__device__ __forceinline__ F2 renorm(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return F2 { s, __fsub_rn(b, __fsub_rn(s, a)) };
}

// Accumulator of a dot product: s += a x with the leading products and the
// running sum of leading parts kept error-free, the low-order terms summed
// in a second float.
struct Acc {
    float hi = 0.0f, lo = 0.0f;
};
__device__ __forceinline__ void madd(Acc& s, F2 a, F2 x)
{
    const float p = __fmul_rn(a.hi, x.hi);
    const float pe = __fmaf_rn(a.hi, x.hi, -p);
    const float t = __fadd_rn(s.hi, p);
    const float z = __fsub_rn(t, s.hi);
    const float te = __fadd_rn(__fsub_rn(s.hi, __fsub_rn(t, z)), __fsub_rn(p, z));
    const float cross = __fmaf_rn(a.hi, x.lo, __fmul_rn(a.lo, x.hi));
    s.lo = __fadd_rn(s.lo, __fadd_rn(__fadd_rn(te, pe), cross));
    s.hi = t;
}
__device__ __forceinline__ F2 result(const Acc& s) { return renorm(s.hi, s.lo); }

// a + b (TwoSum of the leading parts)
__device__ __forceinline__ F2 add(F2 a, F2 b)
{
    const float t = __fadd_rn(a.hi, b.hi);
    const float z = __fsub_rn(t, a.hi);
    const float te = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(t, z)), __fsub_rn(b.hi, z));
    return renorm(t, __fadd_rn(te, __fadd_rn(a.lo, b.lo)));
}
// a b (TwoProduct of the leading parts)
__device__ __forceinline__ F2 mul(F2 a, F2 b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    const float pe = __fmaf_rn(a.hi, b.hi, -p);
    return renorm(p, __fadd_rn(pe, __fmaf_rn(a.hi, b.lo, __fmul_rn(a.lo, b.hi))));
}
// a c for a float c
__device__ __forceinline__ F2 mul(F2 a, float c)
{
    const float p = __fmul_rn(a.hi, c);
    const float pe = __fmaf_rn(a.hi, c, -p);
    return renorm(p, __fmaf_rn(a.lo, c, pe));
}
// a c for a power of two c (exact)
__device__ __forceinline__ F2 scale2(F2 a, float c) { return F2 { __fmul_rn(a.hi, c), __fmul_rn(a.lo, c) }; }

} // namespace pairs
} // namespace nsdg
