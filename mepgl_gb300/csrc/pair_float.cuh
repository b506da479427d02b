// pair_float.cuh -- float-float arithmetic for the paired FP64 mode.
//
// GB300 runs FP32 on its FMA pipes at tens of times the FP64 rate.  A value
// is kept as an unevaluated sum hi + lo of two floats (|lo| <= ulp(hi) / 2,
// about 48 significant bits), and every operation is built from exact
// float transformations: Knuth's two-sum for addition and the FMA
// two-product for multiplication, each followed by a renormalising
// fast-two-sum (the double-double algorithms of Dekker, 1971, and of Hida,
// Li and Bailey, "Algorithms for quad-double precision floating point
// arithmetic", 2001, here on floats).  Relative error per operation is a
// few units of 2^-48, i.e. about 1e-14, against 1.1e-16 for double: fields
// stay double in memory, and every reduction past the warp is double.
//
// All float operations use the _rn intrinsics so that the compiler neither
// contracts nor reorders them; the transformations depend on their order.
#pragma once

#include <cuda_runtime.h>

namespace mepgl {

struct ff {
    float hi, lo;
    ff() = default;
    __host__ __device__ constexpr ff(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ constexpr ff(float f) : hi(f), lo(0.0f) {}
    __host__ __device__ constexpr ff(int i) : hi((float)i), lo(0.0f) {}
    // nearest float, then the float nearest to the remainder (exact for the
    // constants used here; two FP64 operations at run time)
    __host__ __device__ constexpr ff(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
    __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

struct ff2 {
    ff x, y;
};

// s + e = a + b exactly (Knuth)
__device__ __forceinline__ ff two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return ff(s, e);
}

// s + e = a + b exactly when |a| >= |b| (Dekker)
__device__ __forceinline__ ff fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return ff(s, __fsub_rn(b, __fsub_rn(s, a)));
}

// Addition.  MEPGL_FF_ACCURATE_ADD = 1: the IEEE-style sum (error a few
// units of 2^-48 of the result); 0 (default): the cheaper sum of Hida, Li
// and Bailey (error a few units of 2^-48 of |a| + |b|), measured 1.2x faster
// on the NLCG passes and within every paired-mode tolerance.
#ifndef MEPGL_FF_ACCURATE_ADD
#define MEPGL_FF_ACCURATE_ADD 0
#endif
__device__ __forceinline__ ff operator+(ff a, ff b)
{
    const ff s = two_sum(a.hi, b.hi);
#if MEPGL_FF_ACCURATE_ADD
    const ff t = two_sum(a.lo, b.lo);
    ff u = fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
    return fast_two_sum(u.hi, __fadd_rn(u.lo, t.lo));
#else
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
#endif
}

__device__ __forceinline__ ff operator-(ff a) { return ff(-a.hi, -a.lo); }
__device__ __forceinline__ ff operator-(ff a, ff b) { return a + (-b); }

__device__ __forceinline__ ff operator*(ff a, ff b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);          // exact error of the product
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}

__device__ __forceinline__ ff &operator+=(ff &a, ff b) { return a = a + b; }
__device__ __forceinline__ ff &operator-=(ff &a, ff b) { return a = a - b; }
__device__ __forceinline__ ff &operator*=(ff &a, ff b) { return a = a * b; }
__device__ __forceinline__ bool operator==(ff a, ff b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(ff a, ff b) { return !(a == b); }

// mixed forms with plain numbers (literals in the stencil code)
__device__ __forceinline__ ff operator*(int i, ff a) { return ff(i) * a; }
__device__ __forceinline__ ff operator*(ff a, int i) { return a * ff(i); }

// warp shuffle of any lattice number type (float, double, float-float)
__device__ __forceinline__ float shfl_down(float v, int o) { return __shfl_down_sync(0xffffffffu, v, o); }
__device__ __forceinline__ double shfl_down(double v, int o) { return __shfl_down_sync(0xffffffffu, v, o); }
__device__ __forceinline__ ff shfl_down(ff v, int o)
{
    return ff(__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o));
}

// ------------------------------------------------ packed pairs of float-floats
// Two independent float-float numbers (one per lane of an FP32x2 register
// pair: the two components of a two-component string), hi = (hi_0, hi_1),
// lo = (lo_0, lo_1).  Every operation is the scalar one above, lane by lane,
// on the packed FP32x2 instructions (same rounding, half the instructions).
struct ffp {
    float2 hi, lo;
};

__device__ __forceinline__ float2 neg2f(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 addf2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 subf2(float2 a, float2 b) { return __fadd2_rn(a, neg2f(b)); }

__device__ __forceinline__ ffp two_sum(float2 a, float2 b)
{
    const float2 s = addf2(a, b);
    const float2 bb = subf2(s, a);
    return ffp{s, addf2(subf2(a, subf2(s, bb)), subf2(b, bb))};
}

__device__ __forceinline__ ffp fast_two_sum(float2 a, float2 b)
{
    const float2 s = addf2(a, b);
    return ffp{s, subf2(b, subf2(s, a))};
}

__device__ __forceinline__ ffp operator+(ffp a, ffp b)
{
    const ffp s = two_sum(a.hi, b.hi);
#if MEPGL_FF_ACCURATE_ADD
    const ffp t = two_sum(a.lo, b.lo);
    const ffp u = fast_two_sum(s.hi, addf2(s.lo, t.hi));
    return fast_two_sum(u.hi, addf2(u.lo, t.lo));
#else
    return fast_two_sum(s.hi, addf2(s.lo, addf2(a.lo, b.lo)));
#endif
}

__device__ __forceinline__ ffp operator-(ffp a) { return ffp{neg2f(a.hi), neg2f(a.lo)}; }
__device__ __forceinline__ ffp operator-(ffp a, ffp b) { return a + (-b); }

__device__ __forceinline__ ffp operator*(ffp a, ffp b)
{
    const float2 p = __fmul2_rn(a.hi, b.hi);
    float2 e = __ffma2_rn(a.hi, b.hi, neg2f(p));   // exact error of the products
    e = __ffma2_rn(a.hi, b.lo, e);
    e = __ffma2_rn(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}

// double <-> float-float at the memory boundary (two and three FP64-pipe
// operations; integer-only splitting was measured slower on GB300, where
// these kernels are bound by instruction issue rather than by the FP64 pipe)
__device__ __forceinline__ ff to_ff(double d)
{
    const float h = __double2float_rn(d);
    return ff(h, __double2float_rn(d - (double)h));
}

__device__ __forceinline__ double to_double(ff a) { return (double)a.hi + (double)a.lo; }

}  // namespace mepgl
