// Float-float instantiation support for the residual kernels (the mixed-ff
// form): record types, loads/stores, constants and the two device functions
// whose generic forms would call pow() — Sutherland's law, whose exponent 1.5
// is T*sqrt(T) here, and the far-field boundary state, evaluated in binary64
// on the few boundary faces and rounded back.
#pragma once
#include "ff_arith.h"

namespace cfdgb {

struct alignas(16) q4 { ff x, y, z, w; };
struct alignas(16) q2 { ff x, y; };
template <> struct V4<ff> { typedef q4 type; };
template <> struct V2<ff> { typedef q2 type; };

// accumulator of the residual gather: float-float for float-float fluxes
template <> struct Acc<ff> { typedef ff type; };
FF_HD ff acc_widen(ff x) { return x; }

__device__ __forceinline__ q4 ld4(const q4* p) {
    const float4* q = reinterpret_cast<const float4*>(p);
    const float4 a = q[0], b = q[1];
    return q4{ff(a.x, a.y), ff(a.z, a.w), ff(b.x, b.y), ff(b.z, b.w)};
}
__device__ __forceinline__ void st4(q4* p, const q4& v) {
    float4* q = reinterpret_cast<float4*>(p);
    q[0] = make_float4(v.x.hi, v.x.lo, v.y.hi, v.y.lo);
    q[1] = make_float4(v.z.hi, v.z.lo, v.w.hi, v.w.lo);
}

// Constants as binary64 literals, split into pairs where they are used.
template <> struct C<ff> {
    static constexpr double gamma = 1.4;
    static constexpr double gm1 = 1.4 - 1.0;
    static constexpr double pr = 0.72;
    static constexpr double omega = 1.5;
};

__device__ __forceinline__ ff dsqrt(ff x) { return ff_sqrt(x); }
__device__ __forceinline__ ff dabs(ff x) { return ff_abs(x); }
__device__ __forceinline__ ff dpow(ff x, ff y) { return ff(pow((double)x, (double)y)); }

// mu = (1+cc)/(T+cc) * T^1.5 * sqrt(Gamma) * Ma / Re as K * T*sqrt(T) / (T+cc),
// with K = (1+cc)*sqrt(Gamma)*Ma/Re and cc held per mesh as pairs (ffk).
template <> __device__ __forceinline__ ff sutherland<ff>(ff temp, const MeshPrm& m) {
    const ff cc(m.ffk[0], m.ffk[1]), k(m.ffk[2], m.ffk[3]);
    return k * (temp * ff_sqrt(temp)) / (temp + cc);
}

template <>
__device__ __forceinline__ unsigned boundary_state<ff>(int bc, bool viscous, const ff* ul, ff nx, ff ny,
                                                       const MeshPrm& m, ff* ue) {
    double a[4], e[4];
#pragma unroll
    for (int j = 0; j < 4; j++) a[j] = (double)ul[j];
    const unsigned err = boundary_state<double>(bc, viscous, a, (double)nx, (double)ny, m, e);
#pragma unroll
    for (int j = 0; j < 4; j++) ue[j] = ff(e[j]);
    return err;
}

}  // namespace cfdgb
