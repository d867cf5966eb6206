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

// ---- packed float pairs: two points' sums per instruction ----------------
// sm_100-family GPUs issue FP32 add/mul/fma on register pairs (.f32x2): one
// instruction per two lanes' worth of operations, at the same pipe rate.  A
// sweep bound by instruction issue sums two points (two rows of a thread's
// column) in packed accumulators.  The products stay scalar: a packed
// instruction takes no constant-bank operand, so packed products would move
// every coefficient into a register pair at each use, while the scalar ones
// read it where it lies.  Products and their errors are formed per point
// (8 scalar operations for the two points of a term), the two points' results
// are paired by the register allocator (they come from separate
// instructions), and the error-free sum runs packed (8 operations): 16
// instructions per term for two points instead of 24.  Each operation is the
// scalar one of df_mul / df_fma / renorm in the same order with the same
// rounding, so the results are bit-identical to the scalar sweep's.
// A u64 holds {point 0, point 1}; df2 holds the pairs' hi and lo parts.
typedef unsigned long long u64;

struct df2 {
    u64 h, l;
};

__device__ __forceinline__ u64 pk2(float a, float b) {
    u64 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk2(u64 v, float &a, float &b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ u64 add2(u64 a, u64 b) {
    u64 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ u64 sub2(u64 a, u64 b) {
    u64 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}

// c * x of one point: the product's hi and its error with the cross terms
// (as in df_mul / df_fma).
__device__ __forceinline__ void df_prod(float ch, float cl, float2 x, float &p, float &e) {
    p = __fmul_rn(ch, x.x);
    e = __fmaf_rn(ch, x.x, -p);
    e = __fmaf_rn(ch, x.y, e);
    e = __fmaf_rn(cl, x.x, e);
}

// acc = c * {x0, x1} (df_mul of both points).
__device__ __forceinline__ void df2_mul_s(df2 &acc, float ch, float cl, float2 x0, float2 x1) {
    float p0, p1, e0, e1;
    df_prod(ch, cl, x0, p0, e0);
    df_prod(ch, cl, x1, p1, e1);
    acc.h = pk2(p0, p1);
    acc.l = pk2(e0, e1);
}

// acc += c * {x0, x1} (df_fma of both points; TwoSum and the low-part
// accumulation packed).
__device__ __forceinline__ void df2_fma_s(df2 &acc, float ch, float cl, float2 x0, float2 x1) {
    float p0, p1, e0, e1;
    df_prod(ch, cl, x0, p0, e0);
    df_prod(ch, cl, x1, p1, e1);
    const u64 p = pk2(p0, p1), e = pk2(e0, e1);
    const u64 s = add2(acc.h, p);
    const u64 v = sub2(s, acc.h);
    const u64 t = add2(sub2(acc.h, sub2(s, v)), sub2(p, v));
    acc.h = s;
    acc.l = add2(acc.l, add2(t, e));
}

// renorm of both points: {hi, lo} pairs with |lo| <= ulp(hi) / 2.
__device__ __forceinline__ void renorm2(const df2 &a, u64 &h, u64 &l) {
    const u64 s = add2(a.h, a.l);
    const u64 v = sub2(s, a.h);
    l = add2(sub2(a.h, sub2(s, v)), sub2(a.l, v));
    h = s;
}

}  // namespace uhs

namespace uhs {

// ---- bounded sums: one stencil point's sum with an extraction bound ---------
// A point's sum  s = sum_k c_k * x_k  (float pairs c = ch + cl, x = xh + xl)
// in fewer FP32 operations than df_fma's TwoSum per term, by extracting each
// product's high part on a fixed grid (Rump, Ogita and Oishi, "Accurate
// floating-point summation", ExtractScalar):
//   B = sum_k |ch_k| |xh_k| (one FMA per term, bound_add);
//   sigma = 2^m, B (1 + 2^-16) < sigma <= 2 B (1 + 2^-16) (sigma_of);
//   p = ch * xh;  q = (sigma + p) - sigma;  r = fma(ch, xh, -q)
// With |p| <= sigma, q is p on the grid of multiples of 2^-24 sigma and
// p - q is exact (ExtractScalar's lemma), so every partial sum of the q's --
// multiples of 2^-24 sigma below sigma in magnitude, as sum |p| and the n
// roundings to the grid stay below B (1 + (2n + 1) 2^-24) < sigma for up to
// 127 terms -- is exact in a float: tau = sum q_k carries no error.  r is
// the rest of the exact product, ch * xh - q, rounded once (|r| <= 2^-23
// sigma, so its error is below 2^-47 sigma), and the low-order parts go into
// lo:
//   lo += r;  lo = fma(ch, xl, lo);  lo = fma(cl, xh, lo)
// 9 FP32 operations per term with the bound, against df_fma's 12.  The
// point's value is tau + lo, renormalised by one TwoSum (renorm) as before.
// The error is relative to sum |c_k x_k| of the point itself, as with
// df_fma's errors relative to its partial sums: lo sums n terms of at most
// 2^-23 sigma <= 2^-22 (1 + 2^-16) B, so its roundings stay below about
// n^2 2^-46 B, in practice (random signs) near n^1.5 2^-47 B; for a field of
// one sign, B is the point's value.
//
// The bound's exponent is clamped so sigma stays a normal float (inputs
// beyond 2^125 overflow the grid: the range flag catches them).
__device__ __forceinline__ float bound_add(float b, float cabs, float2 x) {  // cabs = |ch|
    return __fmaf_rn(cabs, fabsf(x.x), b);
}
__device__ __forceinline__ float sigma_of(float b) {
    const float bb = __fmul_ru(b, 1.0000152587890625f);  // 1 + 2^-16
    const int e = min(static_cast<int>(__float_as_uint(bb) & 0x7f800000u), 253 << 23);
    return __int_as_float(e + (1 << 23));
}

// acc = c * x (first term of a bounded sum)
__device__ __forceinline__ void dfs_mul(df &acc, float sigma, float ch, float cl, float2 x) {
    const float p = __fmul_rn(ch, x.x);
    const float q = __fsub_rn(__fadd_rn(sigma, p), sigma);
    const float r = __fmaf_rn(ch, x.x, -q);
    acc.h = q;
    acc.l = __fmaf_rn(cl, x.x, __fmaf_rn(ch, x.y, r));
}

// acc += c * x (bounded sum)
__device__ __forceinline__ void dfs_fma(df &acc, float sigma, float ch, float cl, float2 x) {
    const float p = __fmul_rn(ch, x.x);
    const float q = __fsub_rn(__fadd_rn(sigma, p), sigma);
    const float r = __fmaf_rn(ch, x.x, -q);
    acc.h = __fadd_rn(acc.h, q);
    acc.l = __fmaf_rn(cl, x.x, __fmaf_rn(ch, x.y, __fadd_rn(acc.l, r)));
}

// The same for two points at once: the extraction and the two additions
// packed (.f32x2), the products and the low-order terms per point.  Per
// point the same operations as dfs_mul / dfs_fma, so bit-identical to them.
// sig holds {sigma of point 0, sigma of point 1}.
__device__ __forceinline__ void dfs2_mul_s(df2 &acc, u64 sig, float ch, float cl, float2 x0, float2 x1) {
    const u64 p = pk2(__fmul_rn(ch, x0.x), __fmul_rn(ch, x1.x));
    const u64 q = sub2(add2(sig, p), sig);
    float q0, q1;
    upk2(q, q0, q1);
    const float r0 = __fmaf_rn(ch, x0.x, -q0), r1 = __fmaf_rn(ch, x1.x, -q1);
    acc.h = q;
    acc.l = pk2(__fmaf_rn(cl, x0.x, __fmaf_rn(ch, x0.y, r0)), __fmaf_rn(cl, x1.x, __fmaf_rn(ch, x1.y, r1)));
}

__device__ __forceinline__ void dfs2_fma_s(df2 &acc, u64 sig, float ch, float cl, float2 x0, float2 x1) {
    const u64 p = pk2(__fmul_rn(ch, x0.x), __fmul_rn(ch, x1.x));
    const u64 q = sub2(add2(sig, p), sig);
    float q0, q1;
    upk2(q, q0, q1);
    const float r0 = __fmaf_rn(ch, x0.x, -q0), r1 = __fmaf_rn(ch, x1.x, -q1);
    acc.h = add2(acc.h, q);
    float l0, l1;
    upk2(add2(acc.l, pk2(r0, r1)), l0, l1);
    acc.l = pk2(__fmaf_rn(cl, x0.x, __fmaf_rn(ch, x0.y, l0)), __fmaf_rn(cl, x1.x, __fmaf_rn(ch, x1.y, l1)));
}

}  // namespace uhs
