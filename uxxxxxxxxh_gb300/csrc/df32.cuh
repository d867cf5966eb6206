// Float-pair ("df32") arithmetic for FP64 grids on GB300.
//
// GB300's FP64 pipe issues about 2 operations per clock per SM (measured:
// 600 G DFMA/s on 152 SMs), while its FP32 pipes issue 128 FFMA and its
// integer pipes 64 operations per clock per SM.  A 7-point FP64 sweep done
// in native DFMA is therefore capped near 86 GStencil/s, a fifth of what HBM
// could feed.  This header keeps FP64 values as an unevaluated sum of two
// floats, value = h + l, and does all arithmetic on the FP32 pipes:
//
//   * split_f64: double -> (h, l) with integer bit operations and one
//     integer-to-float conversion (the double-to-float conversion runs on
//     the FP64 pipe, so it is avoided).  h holds the top 24 significant bits
//     (truncated), l the remaining 29 rounded to 24, so
//     |x - (h + l)| <= 2^-48 |x| for 2^-74 <= |x| < 2^128.  Below 2^-74 the
//     low part is dropped and below 2^-126 the value flushes to zero
//     (absolute error under 2^-74, about 5e-23); 2^128 and above sets the
//     range flag.
//   * Scaling: a pair may hold x * 2^s instead of x.  The split then
//     rebiases the exponent by 896 - s instead of 896 (1023 - 127) and the
//     join by the same amount back, so the window above applies to x * 2^s:
//     a run can place any 2^202 range of FP64 magnitudes inside it.  A
//     linear sweep commutes with the power-of-two scale exactly (every
//     product and sum of scaled values is the scaled product or sum, as long
//     as nothing leaves the window), so results do not depend on s.
//   * df_fma: acc += c * x with the product's rounding error recovered by an
//     FMA (Dekker/Veltkamp product via fused multiply-add) and the running
//     sum's by Knuth's TwoSum; error terms are gathered in acc.l.
//   * join_f64: (h, l) -> the double nearest h + l: each float is widened
//     exactly by bit construction and the two are added by one DADD, the
//     only FP64 instruction per point (the FP64 pipe is otherwise idle).
// Every operation is written with the _rn intrinsics so the compiler cannot
// contract or reassociate it; the error-free transformations depend on each
// product and sum being rounded exactly once.
#pragma once
#include <cstdint>

namespace uhs {

struct df {
    float h, l;
};

// Exponent rebias between a double x and the float pair of x * 2^shift.
__host__ __device__ constexpr int pair_bias(int shift) { return 896 - shift; }

// x -> the pair of x * 2^shift (bias = pair_bias(shift)).
__device__ __forceinline__ float2 split_f64(double x, unsigned &range_err, int bias = 896) {
    const unsigned hi = static_cast<unsigned>(__double2hiint(x)), lo = static_cast<unsigned>(__double2loint(x));
    const unsigned sign = hi & 0x80000000u;
    // biased float exponent of x * 2^shift (E + 127 + shift, E = eb - 1023)
    const int fe = static_cast<int>((hi >> 20) & 0x7ffu) - bias;
    // h: exponent rebiased and the top 23 fraction bits funnel-shifted in
    // from both words.
    const unsigned f = __funnelshift_l(lo, hi - (static_cast<unsigned>(bias) << 20), 3);
    const unsigned hb = (f & 0x7fffffffu) | sign;
    // l: the remaining 29 fraction bits (weight 2^(fe-127-52)), rounded to 24
    // bits by the integer-to-float conversion and scaled by that weight.
    const float lm = __uint2float_rn(lo & 0x1fffffffu);
    const float sc = __uint_as_float((hb & 0x7f800000u) - (52u << 23));
    float l = __uint_as_float(__float_as_uint(__fmul_rn(lm, sc)) | sign);
    float h = __uint_as_float(hb);
    if (static_cast<unsigned>(fe - 1) >= 254u) {  // scaled exponent outside [-126, 127] (or x zero)
        if (fe > 254) range_err = 1u;
        h = __uint_as_float(sign);
    }
    if (fe < 53) l = 0.0f;  // the low part's weight below the float range: drop it
    return make_float2(h, l);
}

// Exact float -> double of v * 2^-shift by bit construction (normal floats
// and zero; a subnormal float becomes zero).  No FP64 instruction.
__device__ __forceinline__ double f2d_bits(float v, int bias = 896) {
    const unsigned b = __float_as_uint(v);
    const unsigned s = b & 0x80000000u;
    const unsigned hi = s | (((b & 0x7fffffffu) >> 3) + (static_cast<unsigned>(bias) << 20));
    const unsigned lo = b << 29;
    return (b & 0x7f800000u) ? __hiloint2double(static_cast<int>(hi), static_cast<int>(lo))
                             : __hiloint2double(static_cast<int>(s), 0);
}

// The pair of x * 2^shift -> the double nearest x = (h + l) * 2^-shift: both
// halves converted exactly, then one correctly rounded FP64 addition (the
// only FP64 instruction per point).
__device__ __forceinline__ double join_f64(float h, float l, int bias = 896) {
    return __dadd_rn(f2d_bits(h, bias), f2d_bits(l, bias));
}

// acc = c * x  (first term)
__device__ __forceinline__ void df_mul(df &acc, float ch, float cl, float2 x) {
    const float p = __fmul_rn(ch, x.x);
    float e = __fmaf_rn(ch, x.x, -p);
    e = __fmaf_rn(ch, x.y, e);
    e = __fmaf_rn(cl, x.x, e);
    acc.h = p;
    acc.l = e;
}

// acc += c * x
__device__ __forceinline__ void df_fma(df &acc, float ch, float cl, float2 x) {
    const float p = __fmul_rn(ch, x.x);
    float e = __fmaf_rn(ch, x.x, -p);
    e = __fmaf_rn(ch, x.y, e);
    e = __fmaf_rn(cl, x.x, e);
    const float s = __fadd_rn(acc.h, p);
    const float v = __fsub_rn(s, acc.h);
    const float t = __fadd_rn(__fsub_rn(acc.h, __fsub_rn(s, v)), __fsub_rn(p, v));
    acc.h = s;
    acc.l = __fadd_rn(acc.l, __fadd_rn(t, e));
}

// (h, l) -> the same value with |l| <= ulp(h) / 2 (TwoSum).
__device__ __forceinline__ float2 renorm(df a) {
    const float s = __fadd_rn(a.h, a.l);
    const float v = __fsub_rn(s, a.h);
    const float t = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, v)), __fsub_rn(a.l, v));
    return make_float2(s, t);
}

}  // namespace uhs
