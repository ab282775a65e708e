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

}  // namespace cmt
