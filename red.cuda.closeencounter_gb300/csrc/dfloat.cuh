// dfloat.cuh -- double-float arithmetic on GB300's FP32 pipes (unevaluated sums of two
// floats: Knuth's two-sum, the FMA two-product, and the double-double add / multiply of
// Hida, Li and Bailey (2001) carried out in float), and exact FP64 <-> FP32 conversions done
// on the bit patterns with integer operations (a conversion on the FP64 pipe would cost as
// much issue as about 64 FP32 operations).  Used by the mixed-precision gravity kernels.
#pragma once

#include <cuda_runtime.h>

namespace redgb {

// The split is done on the bit patterns, with integer operations only (a conversion
// FP64 -> FP32 runs on GB300's scarce FP64 pipe): hi = v rounded to 24 significant bits
// (round half up on the dropped 29 bits; a carry into the exponent is the correct next
// value, up to infinity), lo = the signed remainder rounded to FP32, so |v - (hi + lo)| <=
// 2^-48 |v| and hi carries no bias.  |v| < 2^-74 gives lo = 0 and |v| < 2^-126 gives
// hi = lo = 0; |v| >= 2^128 gives an infinite hi.
__device__ __forceinline__ void split_bits(double v, float& hi, float& lo)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7ffu);
    const int ef = e - 896;  // FP32 biased exponent
    if (ef <= 0) {
        hi = lo = 0.0f;
        return;
    }
    const unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
    if (ef >= 255) {  // beyond FP32's range, or inf / NaN: built from bits (a hardware
                      // conversion here would be evaluated for every call, on the FP64 pipe)
        hi = __uint_as_float(sign | 0x7f800000u | (e == 2047 && mant != 0 ? 0x400000u : 0u));
        lo = 0.0f;
        return;
    }
    unsigned hb = sign | ((unsigned)ef << 23) | (unsigned)(mant >> 29);
    int r = (int)(mant & 0x1FFFFFFFu);  // the dropped bits, in units of 2^(e - 1075)
    if (r >= (1 << 28)) {
        hb += 1u;
        r -= 1 << 29;
    }
    hi = __uint_as_float(hb);
    const int es = e - 948;  // FP32 biased exponent of 2^(e - 1075)
    const float l = es > 0 ? __int2float_rn(r) * __uint_as_float((unsigned)es << 23) : 0.0f;
    lo = sign ? -l : l;
}

struct DF {
    float hi, lo;
};

__device__ __forceinline__ DF df_two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    return DF{s, (a - (s - bb)) + (b - bb)};
}

// |a| >= |b| (or a == 0)
__device__ __forceinline__ DF df_fast_sum(float a, float b)
{
    const float s = a + b;
    return DF{s, b - (s - a)};
}

__device__ __forceinline__ DF df_two_prod(float a, float b)
{
    const float p = a * b;
    return DF{p, fmaf(a, b, -p)};
}

__device__ __forceinline__ DF df_add(DF a, DF b)
{
    DF s = df_two_sum(a.hi, b.hi);
    const DF t = df_two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = df_fast_sum(s.hi, s.lo);
    s.lo += t.lo;
    return df_fast_sum(s.hi, s.lo);
}

// a + b for operands of one sign (no cancellation): the "sloppy" addition of Hida, Li and
// Bailey, whose relative error stays near 2^-46 when the operands cannot cancel
__device__ __forceinline__ DF df_add_same_sign(DF a, DF b)
{
    DF s = df_two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return df_fast_sum(s.hi, s.lo);
}

__device__ __forceinline__ DF df_mul(DF a, DF b)
{
    DF p = df_two_prod(a.hi, b.hi);
    p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
    return df_fast_sum(p.hi, p.lo);
}

// (ah + al) - (bh + bl) of two split coordinates
__device__ __forceinline__ DF df_diff(float ah, float al, float bh, float bl)
{
    const DF s = df_two_sum(ah, -bh);
    return df_two_sum(s.hi, (al - bl) + s.lo);
}

// FP32 -> FP64 on the bit pattern (exact; no FP64-pipe conversion); FP32 denormals -> 0.
// Infinities and NaNs are built from their bits too: a hardware conversion in that branch is
// evaluated for every call (a select, not a branch) and runs on GB300's FP64 pipe.
__device__ __forceinline__ double f2d_bits(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned ef = (u >> 23) & 0xffu;
    const unsigned long long e = ef == 255u ? 0x7ffull : (unsigned long long)(ef + 896u);
    const unsigned long long b = ((unsigned long long)(u & 0x80000000u) << 32) | (e << 52) |
                                 ((unsigned long long)(u & 0x7fffffu) << 29);
    return __longlong_as_double(ef == 0u ? 0ll : (long long)b);
}

__device__ __forceinline__ double df_to_double(DF a) { return f2d_bits(a.hi) + f2d_bits(a.lo); }

__device__ __forceinline__ DF split_df(double v)
{
    DF d;
    split_bits(v, d.hi, d.lo);
    return d;
}

// compensated accumulation: s + c tracks the exact sum of the added terms to ~2^-46
struct Acc2 {
    float s, c;
};

__device__ __forceinline__ void two_sum_add(Acc2& a, float t)
{
    const float s = a.s + t;
    const float bp = s - a.s;
    const float err = (a.s - (s - bp)) + (t - bp);
    a.s = s;
    a.c += err;
}

// a double-float term into a compensated FP32 accumulator
__device__ __forceinline__ void acc_df(Acc2& acc, DF t)
{
    two_sum_add(acc, t.hi);
    acc.c += t.lo;
}

// a stage-vector element stored as a double-float pair (float2: hi, lo)
__device__ __forceinline__ float2 to_f2(double v)
{
    float h, l;
    split_bits(v, h, l);
    return make_float2(h, l);
}

__device__ __forceinline__ double f2_to_double(float2 f) { return f2d_bits(f.x) + f2d_bits(f.y); }

// a coordinate split for the mixed gravity kernels' 32-byte body records (x, y, z, m as
// float2 pairs #0..#3).  Coordinates beyond 1e15 AU are clamped there (a merged body is
// parked at 1e20 AU, pp_disk.cu:1184, and a hit-star merger stays active with m = 0 until
// the next ejection check): |r|^2 then stays finite in FP32, so the pair loops need no clamp,
// and such a body's zero mass gives a zero term.
__device__ __forceinline__ void split_coord(double v, float& hi, float& lo)
{
    split_bits(v, hi, lo);
    if (fabsf(hi) > 1.0e15f) {
        hi = copysignf(1.0e15f, hi);
        lo = 0.0f;
    }
}


}  // namespace redgb
