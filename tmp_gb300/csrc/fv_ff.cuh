// Float-float instantiation support for the residual kernels (the MIXFF form):
// record types, loads/stores, constants and the two device functions whose
// generic forms call pow() — Sutherland's law (T^1.5 = T*sqrt(T)) and the
// far-field boundary state (rho^1.4 and t^2.5) — written without it, so that
// no warp of the float-float residual waits on the binary64 pipe.
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
// (no dpow for pairs: the two generic functions that call pow() are specialised
// below, so a new use fails to compile instead of reaching the binary64 pipe)

// mu = (1+cc)/(T+cc) * T^1.5 * sqrt(Gamma) * Ma / Re as K * T*sqrt(T) / (T+cc),
// with K = (1+cc)*sqrt(Gamma)*Ma/Re and cc held per mesh as pairs (ffk).
template <> __device__ __forceinline__ ff sutherland<ff>(ff temp, const MeshPrm& m) {
    const ff cc(m.ffk[0], m.ffk[1]), k(m.ffk[2], m.ffk[3]);
    return k * (temp * ff_sqrt(temp)) / (temp + cc);
}

// x^0.4 for x > 0: a binary32 seed refined by two Newton steps on y^5 = x^2,
// y <- (4y + x^2/y^4)/5, each of which squares the seed's relative error.
__device__ __forceinline__ ff ff_pow04(ff x) {
    ff y(powf(x.hi, 0.4f), 0.f);
    const ff x2 = x * x;
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const ff y2 = y * y;
        y = (ff(4) * y + x2 / (y2 * y2)) / ff(5);
    }
    return y;
}

// Face state of a boundary face in pairs: the generic expressions
// (HandleViscousBoundary / HandleInvicidBoundary, BoundaryStrategy.h:73-335)
// with the reference's pow() calls rewritten for Gamma = 1.4 — rho^Gamma as
// rho * rho^0.4 and t^(1/(Gamma-1)) = t^2.5 as t*t*sqrt(t) — and the
// freestream values and entropy taken as per-mesh pairs.
template <>
__device__ __forceinline__ unsigned boundary_state<ff>(int bc, bool viscous, const ff* ul, ff nx, ff ny,
                                                       const MeshPrm& m, ff* ue) {
    const ff G = ff(C<ff>::gamma), GM1 = ff(C<ff>::gm1);
    unsigned err = 0;
    if (bc == BC_WALL) {
        if (viscous) {
            ue[0] = ul[0]; ue[1] = ul[1]; ue[2] = ff(0); ue[3] = ff(0);
        } else {
            const ff vnl = dot2(ul[2], ul[3], nx, ny);
            const ff t0 = ul[2] - nx * vnl, t1 = ul[3] - ny * vnl;
            if (dot2(t0, t1, nx, ny) > ff(1.0e-7)) err |= ERR_WALLTAN;  // the reference's binary64 bound
            ue[0] = ul[0]; ue[1] = ul[1]; ue[2] = t0; ue[3] = t1;
        }
        return err;
    }
    const ff rinf(m.fff[0], m.fff[1]), pinf(m.fff[2], m.fff[3]), uinf(m.fff[4], m.fff[5]),
        vinf(m.fff[6], m.fff[7]), cinf(m.fff[8], m.fff[9]), s_inf(m.fff[10], m.fff[11]);
    const ff vnl = dot2(ul[2], ul[3], nx, ny);
    const ff tl0 = ul[2] - nx * vnl, tl1 = ul[3] - ny * vnl;
    const ff vnr = dot2(uinf, vinf, nx, ny);
    const ff tr0 = uinf - nx * vnr, tr1 = vinf - ny * vnr;
    const ff rl = ul[0], pl = ul[1];
    if (ff_abs(vnr) < cinf) {
        const ff cl = ff_sqrt(G * pl / rl);
        const ff vnb = (vnl + vnr + ff(2) * (cl - cinf) / GM1) / ff(2);
        const ff cb = (vnl - vnr + ff(2) * (cinf + cl) / GM1) * GM1 / ff(4);
        ff sb, e0, e1;
        if (vnr >= ff(0)) {
            sb = pl / (rl * ff_pow04(rl));
            e0 = tl0 + nx * vnb; e1 = tl1 + ny * vnb;
        } else {
            sb = s_inf;
            e0 = tr0 + nx * vnb; e1 = tr1 + ny * vnb;
        }
        const ff t = cb * cb / (G * sb);
        ue[0] = t * t * ff_sqrt(t);
        ue[1] = ue[0] * cb * cb / G;
        ue[2] = e0; ue[3] = e1;
    } else if (vnr >= ff(0)) {
        ue[0] = ul[0]; ue[1] = ul[1]; ue[2] = ul[2]; ue[3] = ul[3];
    } else {
        ue[0] = rinf; ue[1] = pinf; ue[2] = uinf; ue[3] = vinf;
    }
    return err;
}

}  // namespace cfdgb
