// Float-float arithmetic: a value is the unevaluated sum hi + lo of two binary32
// numbers with |lo| <= ulp(hi)/2 — 48 significant bits over the exponent range
// of binary32.
//
// Why: on GB300 a warp's binary64 instruction holds its sub-partition for 64
// cycles, a binary32 one for one, so a residual whose every operation costs
// 7-20 binary32 instructions still runs several times faster than its binary64
// build while keeping a rounding floor near 1e-14 relative (binary32: 1e-7) —
// far below the 1e-8 residual fall the mixed forms iterate to.
//
// Building blocks, all error-free transformations of binary32 operations:
//   two_sum       Knuth, TAOCP vol. 2, sec. 4.2.2 (6 operations, any a, b)
//   fast_two_sum  Dekker, Numer. Math. 18 (1971) (3 operations, |a| >= |b|)
//   two_prod      a*b = p + e exactly, e from one fused multiply-add
// Pair operations follow Joldes, Muller & Popescu, "Tight and rigorous error
// bounds for basic building blocks of double-word arithmetic", ACM TOMS 44(2),
// 2017: the "sloppy" pair sum (their Algorithm 5: error below 2^-46 of
// |x| + |y|; relative to the result only when no cancellation occurs, which is
// what binary64 operands carrying earlier roundings give as well) and the pair
// product with fused multiply-adds (their Algorithm 11 shape, relative error
// below 2^-46).  Quotient and square root take a correctly rounded binary32
// first approximation and one correction whose remainder is formed exactly
// (Karp & Markstein, "High-precision division and square root", ACM TOMS
// 23(4), 1997): relative error below 2^-44 and 2^-46.  (Bounds as measured on
// random operands by tests/test_ff_arith.py.)
//
// Compiles as plain C++ (host tests) and as CUDA device code.  The unit that
// instantiates these for the GPU is compiled with -fmad=false so that no a*b+c
// written here is contracted behind the transformations' backs; the fused
// multiply-adds they need are explicit fmaf calls.
#pragma once
#include <math.h>

#if defined(__CUDACC__)
#define FF_HD __host__ __device__ __forceinline__
#else
#define FF_HD inline
#endif

namespace cfdgb {

struct alignas(8) ff {
    float hi, lo;
    ff() = default;
    FF_HD constexpr ff(float h, float l) : hi(h), lo(l) {}
    FF_HD constexpr ff(int v) : hi((float)v), lo(0.f) {}
    // nearest binary32 plus the nearest binary32 of the remainder: exact to 2^-48
    FF_HD constexpr ff(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
    FF_HD explicit operator double() const { return (double)hi + (double)lo; }
    FF_HD explicit operator float() const { return hi; }
};

FF_HD ff ff_fast_two_sum(float a, float b) {
    const float s = a + b;
    const float e = b - (s - a);
    return ff(s, e);
}
FF_HD ff ff_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return ff(s, e);
}

FF_HD ff operator-(ff x) { return ff(-x.hi, -x.lo); }

FF_HD ff operator+(ff x, ff y) {
    const ff s = ff_two_sum(x.hi, y.hi);
    const float v = x.lo + y.lo;
    const float w = s.lo + v;
    return ff_fast_two_sum(s.hi, w);
}
FF_HD ff operator-(ff x, ff y) { return x + (-y); }

FF_HD ff operator*(ff x, ff y) {
    const float p = x.hi * y.hi;
    float e = fmaf(x.hi, y.hi, -p);  // x.hi*y.hi - p, exactly
    e = fmaf(x.hi, y.lo, e);
    e = fmaf(x.lo, y.hi, e);
    return ff_fast_two_sum(p, e);
}

FF_HD float ff_recip_seed(float y) {
#if defined(__CUDA_ARCH__)
    return __frcp_rn(y);
#else
    return 1.0f / y;
#endif
}

FF_HD ff operator/(ff x, ff y) {
    const float r = ff_recip_seed(y.hi);
    const float q1 = x.hi * r;
    // remainder x - q1*y: q1*y.hi = p + pe exactly; x.hi - p is exact (p is
    // within a few ulps of x.hi); the remaining terms are of order ulp(x)
    const float p = q1 * y.hi;
    const float pe = fmaf(q1, y.hi, -p);
    float rem = (x.hi - p) - pe;
    rem = rem + x.lo;
    rem = fmaf(-q1, y.lo, rem);
    const float q2 = rem * r;
    return ff_fast_two_sum(q1, q2);
}

FF_HD ff ff_sqrt(ff x) {
    if (!(x.hi > 0.f)) return ff(sqrtf(x.hi), 0.f);  // 0, or NaN for negative input
    const float s = sqrtf(x.hi);                      // correctly rounded
#if defined(__CUDA_ARCH__)
    const float t = rsqrtf(x.hi);                     // 1/sqrt, only scales the correction
#else
    const float t = 1.0f / s;
#endif
    const float p = s * s;
    const float pe = fmaf(s, s, -p);  // s*s = p + pe exactly
    float rem = (x.hi - p) - pe;
    rem = rem + x.lo;                 // x - s*s
    const float c = rem * (0.5f * t);
    return ff_fast_two_sum(s, c);
}

FF_HD ff& operator+=(ff& a, ff b) { a = a + b; return a; }
FF_HD ff& operator-=(ff& a, ff b) { a = a - b; return a; }
FF_HD ff& operator*=(ff& a, ff b) { a = a * b; return a; }
FF_HD ff& operator/=(ff& a, ff b) { a = a / b; return a; }

// Ordering of normalised pairs: by the high part, ties by the low part.
FF_HD bool operator<(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
FF_HD bool operator>(ff a, ff b) { return b < a; }
FF_HD bool operator<=(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo); }
FF_HD bool operator>=(ff a, ff b) { return b <= a; }
FF_HD bool operator==(ff a, ff b) { return a.hi == b.hi && a.lo == b.lo; }
FF_HD bool operator!=(ff a, ff b) { return !(a == b); }

FF_HD ff ff_abs(ff x) { return x.hi < 0.f ? -x : x; }

}  // namespace cfdgb
