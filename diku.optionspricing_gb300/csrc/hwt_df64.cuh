// Double-float ("df64") numbers for the FP32 pipes: a value is an unevaluated
// sum hi + lo of two floats with |lo| <= ulp(hi) / 2, about 48 significand bits.
//
// GB300 issues FP32 arithmetic at 64 times its FP64 rate, so a row update kept in
// df64 (about 30 float operations per node and pass) runs faster than the same
// update in native double (3 DFMA per node) while staying within the 1e-10
// relative bound of the FP64 results.  The building blocks are the classical
// error-free transformations: Knuth's TwoSum and Dekker's FastTwoSum for sums,
// and the FMA-based exact product (the rounding error of a*b is fma(a, b, -a*b));
// the double-word sum and product follow the "sloppy" sum and the FMA product of
// Joldes, Muller and Popescu (ACM TOMS 2017), and the three-term dot product is a
// compensated one in the manner of Ogita, Rump and Oishi (SIAM J. Sci. Comput.
// 2005): the products' and sums' rounding errors are gathered in one float and
// added back once.  The sloppy sum is accurate for terms of one sign, which is all
// the tree's sweeps ever add (probabilities, discount factors and values are
// non-negative).  Every operation uses the _rn intrinsics, so the compiler cannot
// contract or reassociate them.  The float exponent range limits magnitudes to
// about 1e-38 .. 3e38; Arrow-Debreu values below that flush to zero, which moves
// prices by less than 1e-30.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace hwt {

struct df64 {
    float hi, lo;
    df64() = default;
    __host__ __device__ df64(double x)
    {
        hi = (float)x;
        lo = (float)(x - (double)hi);
    }
    __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ df64 df64_make(float hi, float lo)
{
    df64 r;
    r.hi = hi;
    r.lo = lo;
    return r;
}

// s + e = a + b exactly (|a| >= |b| not required)
__device__ __forceinline__ float two_sum(float a, float b, float &e)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return s;
}

// s + e = a + b exactly when |a| >= |b| (or a == 0)
__device__ __forceinline__ df64 fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return df64_make(s, __fsub_rn(b, __fsub_rn(s, a)));
}

// x * y, both double-word, with the low parts' cross terms; error ~ 5 u^2
__device__ __forceinline__ df64 operator*(df64 x, df64 y)
{
    const float ch = __fmul_rn(x.hi, y.hi);
    float cl = __fmaf_rn(x.hi, y.hi, -ch);
    cl = __fmaf_rn(x.hi, y.lo, cl);
    cl = __fmaf_rn(x.lo, y.hi, cl);
    return fast_two_sum(ch, cl);
}

// x + y for terms of one sign ("sloppy" double-word sum)
__device__ __forceinline__ df64 operator+(df64 x, df64 y)
{
    float e;
    const float s = two_sum(x.hi, y.hi, e);
    return fast_two_sum(s, __fadd_rn(e, __fadd_rn(x.lo, y.lo)));
}

__device__ __forceinline__ df64 operator-(df64 x) { return df64_make(-x.hi, -x.lo); }
__device__ __forceinline__ df64 operator-(df64 x, df64 y) { return x + (-y); }
__device__ __forceinline__ df64 &operator+=(df64 &x, df64 y)
{
    x = x + y;
    return x;
}

// a + b of two floats, exactly
__device__ __forceinline__ df64 exact_sum(float a, float b)
{
    float e;
    const float s = two_sum(a, b, e);
    return df64_make(s, e);
}

// x / y: a float quotient, its remainder x - q1 y from the exact product and a
// difference that keeps the cancelled bits, and one correction term (relative
// error a few u^2, u = 2^-24)
__device__ __forceinline__ df64 operator/(df64 x, df64 y)
{
    const float q1 = __fdiv_rn(x.hi, y.hi);
    const float ph = __fmul_rn(q1, y.hi);
    const float pl = __fmaf_rn(q1, y.lo, __fmaf_rn(q1, y.hi, -ph));
    float e;
    const float s = two_sum(x.hi, -ph, e);
    const float rem = __fadd_rn(s, __fadd_rn(e, __fsub_rn(x.lo, pl)));
    return fast_two_sum(q1, __fdiv_rn(rem, y.hi));
}

// fma for every row type.  Declaring the df64 overload in this namespace hides the
// global fma from unqualified calls here, so the float and double ones are
// restated as exact-match overloads that forward to the C functions.
__host__ __device__ __forceinline__ float fma(float a, float b, float c) { return ::fmaf(a, b, c); }
__host__ __device__ __forceinline__ double fma(double a, double b, double c) { return ::fma(a, b, c); }

// a * b + c with one renormalisation
__device__ __forceinline__ df64 fma(df64 a, df64 b, df64 c)
{
    const float ph = __fmul_rn(a.hi, b.hi);
    float pl = __fmaf_rn(a.hi, b.hi, -ph);
    pl = __fmaf_rn(a.hi, b.lo, pl);
    pl = __fmaf_rn(a.lo, b.hi, pl);
    float e;
    const float s = two_sum(ph, c.hi, e);
    return fast_two_sum(s, __fadd_rn(__fadd_rn(e, pl), c.lo));
}

// a x + b y + c z, compensated: three exact products, two TwoSums, one
// renormalisation (31 float operations)
__device__ __forceinline__ df64 dot3(df64 a, df64 x, df64 b, df64 y, df64 c, df64 z)
{
    const float p1 = __fmul_rn(a.hi, x.hi);
    float e1 = __fmaf_rn(a.hi, x.hi, -p1);
    e1 = __fmaf_rn(a.hi, x.lo, e1);
    e1 = __fmaf_rn(a.lo, x.hi, e1);
    const float p2 = __fmul_rn(b.hi, y.hi);
    float e2 = __fmaf_rn(b.hi, y.hi, -p2);
    e2 = __fmaf_rn(b.hi, y.lo, e2);
    e2 = __fmaf_rn(b.lo, y.hi, e2);
    const float p3 = __fmul_rn(c.hi, z.hi);
    float e3 = __fmaf_rn(c.hi, z.hi, -p3);
    e3 = __fmaf_rn(c.hi, z.lo, e3);
    e3 = __fmaf_rn(c.lo, z.hi, e3);
    float t1, t2;
    float s = two_sum(p1, p2, t1);
    s = two_sum(s, p3, t2);
    const float lo = __fadd_rn(__fadd_rn(e1, e2), __fadd_rn(e3, __fadd_rn(t1, t2)));
    return fast_two_sum(s, lo);
}

// Two double-float numbers side by side (lanes .x and .y) for the paired FP32
// instructions (__fadd2_rn, __fmul2_rn, __ffma2_rn: two operations per issue slot).
// a - b is issued as fma(b, -1, a), which rounds as the subtraction, so every lane
// of these functions gives bitwise the result of its scalar counterpart above.
struct df64x2 {
    float2 hi, lo;
};

__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

__device__ __forceinline__ float2 two_sum2(float2 a, float2 b, float2 &e)
{
    const float2 s = __fadd2_rn(a, b);
    const float2 bb = sub2(s, a);
    e = __fadd2_rn(sub2(a, sub2(s, bb)), sub2(b, bb));
    return s;
}

__device__ __forceinline__ df64x2 fast_two_sum2(float2 a, float2 b)
{
    const float2 s = __fadd2_rn(a, b);
    df64x2 r;
    r.hi = s;
    r.lo = sub2(b, sub2(s, a));
    return r;
}

// dot3 on two lanes, in an order that retires each product's terms early (the
// operations and their operands are dot3's, so the results are bitwise the same)
__device__ __forceinline__ float2 prod_err2(const df64x2 &a, const df64x2 &x, float2 &p)
{
    p = __fmul2_rn(a.hi, x.hi);
    float2 e = __ffma2_rn(a.hi, x.hi, make_float2(-p.x, -p.y));
    e = __ffma2_rn(a.hi, x.lo, e);
    return __ffma2_rn(a.lo, x.hi, e);
}

__device__ __forceinline__ df64x2 dot3x2(const df64x2 &a, const df64x2 &x, const df64x2 &b, const df64x2 &y,
                                         const df64x2 &c, const df64x2 &z)
{
    float2 p1, p2, p3, t1, t2;
    const float2 e1 = prod_err2(a, x, p1);
    const float2 e2 = prod_err2(b, y, p2);
    float2 s = two_sum2(p1, p2, t1);
    const float2 e12 = __fadd2_rn(e1, e2);
    const float2 e3 = prod_err2(c, z, p3);
    s = two_sum2(s, p3, t2);
    const float2 lo = __fadd2_rn(e12, __fadd2_rn(e3, __fadd2_rn(t1, t2)));
    return fast_two_sum2(s, lo);
}

}  // namespace hwt
