// Double-float arithmetic (Dekker 1971; Knuth, TAOCP vol. 2, 4.2.2): a value carried as an
// unevaluated sum of two floats hi + lo with about 48 significant bits, computed at FP32
// throughput (GB300's FP64 rate is a small fraction of its FP32 rate).  Used for the
// reference's float64 coordinate chain and for exact re-scoring of distances.
#pragma once

#include <cuda_runtime.h>

namespace cmt {

struct DF {
    float hi, lo;
};

__device__ __forceinline__ DF df_from(double v)
{
    float h = __double2float_rn(v);
    return DF{h, __double2float_rn(v - (double)h)};
}

__device__ __forceinline__ DF df_fast_two_sum(float a, float b)
{
    float s = __fadd_rn(a, b);
    return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ DF df_add(DF a, DF b)
{
    float s = __fadd_rn(a.hi, b.hi);
    float bb = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    return df_fast_two_sum(s, e);
}

__device__ __forceinline__ DF df_mul(DF a, DF b)
{
    float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return df_fast_two_sum(p, e);
}

// float32 of a double-float (hi is already the nearest float of hi + lo unless lo sits on
// half an ulp, which __fadd_rn resolves)
__device__ __forceinline__ float df_to_float(DF a) { return __fadd_rn(a.hi, a.lo); }

// hi + lo of a product of two floats (exact)
__device__ __forceinline__ DF df_prod(float a, float b)
{
    float p = __fmul_rn(a, b);
    return DF{p, __fmaf_rn(a, b, -p)};
}

// a * b for a double-float a and a float b
__device__ __forceinline__ DF df_mul_f(DF a, float b)
{
    float p = __fmul_rn(a.hi, b);
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    return df_fast_two_sum(p, e);
}

// a + b for a double-float a and a float b
__device__ __forceinline__ DF df_add_f(DF a, float b)
{
    float s = __fadd_rn(a.hi, b);
    float bb = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return df_fast_two_sum(s, __fadd_rn(e, a.lo));
}

__device__ __forceinline__ double df_to_double(DF a) { return (double)a.hi + (double)a.lo; }

// float32 of the dot product of three double-float pairs (x = hi, y = lo), sum_c a_c b_c
// (Ogita, Rump & Oishi 2005, "Accurate sum and dot product", algorithm Dot2 with the exact
// product by FMA).  The products' leading parts p_c = fl(a.hi b.hi) are summed with TwoSum
// (Knuth); their exact rounding errors, the cross terms a.hi b.lo + a.lo b.hi (a.lo b.lo,
// below 2^-48 of the product, is dropped) and the two sums' errors are gathered in floats
// and added last, so the one final rounding sees the dot product to about 2^-46 of the
// products' size.
__device__ __forceinline__ float df_dot3_to_float(float2 a0, float2 b0, float2 a1, float2 b1, float2 a2, float2 b2)
{
    const float p0 = __fmul_rn(a0.x, b0.x), p1 = __fmul_rn(a1.x, b1.x), p2 = __fmul_rn(a2.x, b2.x);
    float e0 = __fmaf_rn(a0.x, b0.x, -p0);
    e0 = __fmaf_rn(a0.x, b0.y, e0);
    e0 = __fmaf_rn(a0.y, b0.x, e0);
    float e1 = __fmaf_rn(a1.x, b1.x, -p1);
    e1 = __fmaf_rn(a1.x, b1.y, e1);
    e1 = __fmaf_rn(a1.y, b1.x, e1);
    float e2 = __fmaf_rn(a2.x, b2.x, -p2);
    e2 = __fmaf_rn(a2.x, b2.y, e2);
    e2 = __fmaf_rn(a2.y, b2.x, e2);
    const float s = __fadd_rn(p0, p1), bs = __fsub_rn(s, p0);
    float err = __fadd_rn(__fsub_rn(p0, __fsub_rn(s, bs)), __fsub_rn(p1, bs));
    const float s2 = __fadd_rn(s, p2), bs2 = __fsub_rn(s2, s);
    err = __fadd_rn(err, __fadd_rn(__fsub_rn(s, __fsub_rn(s2, bs2)), __fsub_rn(p2, bs2)));
    return __fadd_rn(s2, __fadd_rn(err, __fadd_rn(__fadd_rn(e0, e1), e2)));
}

// float32 of x (s.x + s.y) for a float x and a double-float s: the exact product's leading
// part plus its rounding error and the low-part term, rounded once
__device__ __forceinline__ float df_scale_to_float(float x, float2 s)
{
    const float p = __fmul_rn(x, s.x);
    float e = __fmaf_rn(x, s.x, -p);
    e = __fmaf_rn(x, s.y, e);
    return __fadd_rn(p, e);
}

// fl32(x + (ah + al) y) for floats x, y and a double-float a: the product ah y split
// exactly (FMA), x + ah y by TwoSum, the low parts added, one final rounding.  Equal to the
// FP64 value x + a y rounded to float except within ~2^-46 of a rounding boundary.
__device__ __forceinline__ float axpy_rn(float x, float ah, float al, float y)
{
    const float ph = __fmul_rn(ah, y);
    float pe = __fmaf_rn(ah, y, -ph);
    pe = __fmaf_rn(al, y, pe);
    const float s = __fadd_rn(x, ph), bs = __fsub_rn(s, x);
    const float se = __fadd_rn(__fsub_rn(x, __fsub_rn(s, bs)), __fsub_rn(ph, bs));
    return __fadd_rn(s, __fadd_rn(se, pe));
}

// Compensated sum of float products (Ogita, Rump & Oishi 2005, algorithm Dot2): s carries
// the rounded running sum, c the exact errors of the products (FMA) and of the additions
// (TwoSum); s + c is the sum as if accumulated in twice the working precision.
struct Dot2 {
    float s, c;
};

__device__ __forceinline__ void dot2_add(Dot2 &d, float a, float b)
{
    const float h = __fmul_rn(a, b);
    const float l = __fmaf_rn(a, b, -h);
    const float s = __fadd_rn(d.s, h), bs = __fsub_rn(s, d.s);
    const float e = __fadd_rn(__fsub_rn(d.s, __fsub_rn(s, bs)), __fsub_rn(h, bs));
    d.s = s;
    d.c = __fadd_rn(d.c, __fadd_rn(e, l));
}

// d += x (the sum's TwoSum error into c)
__device__ __forceinline__ void dot2_add1(Dot2 &d, float x)
{
    const float s = __fadd_rn(d.s, x), bs = __fsub_rn(s, d.s);
    d.c = __fadd_rn(d.c, __fadd_rn(__fsub_rn(d.s, __fsub_rn(s, bs)), __fsub_rn(x, bs)));
    d.s = s;
}

__device__ __forceinline__ double dot2_value(const Dot2 &d) { return (double)d.s + (double)d.c; }

}  // namespace cmt
