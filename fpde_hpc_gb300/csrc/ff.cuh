// Float-float ("double-single") arithmetic for sums that are too heavy for GB300's FP64 pipe
// (2 DFMA/clk/SM): a value is an unevaluated pair hi + lo of floats. Products use the exact
// FMA error of hi*hi; sums use the error-free TwoSum (Knuth), so a pair carries ~48 bits.
// Every operation is written with the _rn intrinsics so the compiler cannot contract the
// error terms away.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fpde {

// double -> (hi, lo) from the bits, integer instructions only: hi is x truncated to 24
// significant bits, lo the remainder truncated to 24 bits, so |x - hi - lo| < 2^-47 |x|.
// |x| < 2^-126 gives (0, 0); lo flushes to zero below the float normal range; |x| >= 2^128
// gives +-inf (NaN stays NaN).
__device__ __forceinline__ float2 d2ff(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7FF) - 1023;
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    if (e < -126) return make_float2(0.f, 0.f);
    if (e > 127) return make_float2(__int_as_float((int)(sign | 0x7F800000u | (e == 1024 && m ? 0x400000u : 0u))), 0.f);
    const float hi = __int_as_float((int)(sign | ((uint32_t)(e + 127) << 23) | (uint32_t)(m >> 29)));
    const uint32_t rem = (uint32_t)(m & 0x1FFFFFFFull);           // the 29 bits below hi
    float lo = 0.f;
    if (rem) {
        const int pos = 31 - __clz(rem);                            // its leading bit, 0..28
        const int el = e - 52 + pos;
        if (el >= -126) {
            const uint32_t mant = pos >= 23 ? rem >> (pos - 23) : rem << (23 - pos);
            lo = __int_as_float((int)(sign | ((uint32_t)(el + 127) << 23) | (mant & 0x7FFFFFu)));
        }
    }
    return make_float2(hi, lo);
}

// (ah, al) += (bh, bl): TwoSum of the high parts, the low parts and the error added in float.
__device__ __forceinline__ void ff_add(float &ah, float &al, float bh, float bl)
{
    const float s = __fadd_rn(ah, bh);
    const float bb = __fsub_rn(s, ah);
    const float err = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
    al = __fadd_rn(al, __fadd_rn(err, bl));
    ah = s;
}

// (ah, al) += w * d for pairs w, d: w.hi*d.hi exactly (product and its FMA error), the cross
// terms w.hi*d.lo + w.lo*d.hi rounded, w.lo*d.lo (below 2^-48 of the product) dropped.
__device__ __forceinline__ void ff_fma(float &ah, float &al, float2 w, float2 d)
{
    const float ph = __fmul_rn(w.x, d.x);
    float pe = __fmaf_rn(w.x, d.x, -ph);
    pe = __fmaf_rn(w.x, d.y, pe);
    pe = __fmaf_rn(w.y, d.x, pe);
    ff_add(ah, al, ph, pe);
}

// Renormalise (ah, al) so that al is below half an ulp of ah (TwoSum of the two parts).
__device__ __forceinline__ void ff_renorm(float &ah, float &al)
{
    const float s = __fadd_rn(ah, al);
    const float bb = __fsub_rn(s, ah);
    al = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(al, bb));
    ah = s;
}

}  // namespace fpde
