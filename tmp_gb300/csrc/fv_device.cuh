// Device-side arithmetic of the unstructured finite-volume path.
//
// Each function restates one piece of the reference solver with the same
// operation order (left-to-right C++ evaluation, "result = 0; result += ..."
// dot products), so that the binary64 instantiation compiled with -fmad=false
// produces the reference's values bit for bit wherever only +,-,*,/ and sqrt are
// involved (all correctly rounded on both sides).  pow() is the only libm call
// on the path (far-field Riemann state and Sutherland's law) and may differ in
// the last bit.  The binary32 instantiation is the fast form.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cfdgb {

struct alignas(32) d4 { double x, y, z, w; };
struct alignas(16) d2 { double x, y; };

template <class T> struct V4;
template <> struct V4<double> { typedef d4 type; };
template <> struct V4<float> { typedef float4 type; };
template <class T> struct V2;
template <> struct V2<double> { typedef d2 type; };
template <> struct V2<float> { typedef float2 type; };

// Error bits raised by kernels (OR-ed into a device word, read by the host).
enum : unsigned {
    ERR_PSTAR = 1u,        // HLLCFluxStrategy.cpp:79-86 consistency check
    ERR_NONPHYS = 2u,      // NaN / non-positive rho or p
    ERR_WALLTAN = 4u,      // BoundaryStrategy.h:250-256 check
    ERR_TIMEOUT = 8u,      // bounded device wait gave up
    ERR_SCHED = 16u,       // a sweep schedule launched on a grid it was not built for
};

// Boundary codes (edge3d<2>::BoundaryType).
constexpr int BC_WALL = -2;
constexpr int BC_FAR = -3;

// Per-mesh constants (freestream in the reference's nondimensional form,
// TopologyHolderStrategy.cpp:325-396, and Sutherland constants,
// LaminarFluxStrategy.h:76-96).
struct MeshPrm {
    double rho_inf, p_inf, u_inf, v_inf, c_inf;  // fs_primVar[0..3], fsnd_soundSpeed
    double mach, re, cc;                         // fs_mach, fs_Re, 110.5 / fs_Temperature
    double sqrt_gamma;                           // sqrtf64(Gamma)
    int viscous;
    int pad;
    double sst_k, sst_w, sst_mut;                // SST freestream k, omega, mu_t (nondimensional)
    float ffk[4];                                // float-float cc and (1+cc)*sqrt(Gamma)*Ma/Re (hi, lo each)
    float fff[12];                               // float-float rho, p, u, v, c at infinity and p/rho^Gamma there
};

template <class T> struct C {
    static constexpr T gamma = T(1.4);
    static constexpr T gm1 = T(1.4) - T(1);  // (Gamma - 1) in the working precision
    static constexpr T pr = T(0.72);          // fs_Pr
    static constexpr T omega = T(1.5);        // OMEGAN
};

// ---- loads / stores --------------------------------------------------------
__device__ __forceinline__ d4 ld4(const d4* p) {
    const double2* q = reinterpret_cast<const double2*>(p);
    double2 a = q[0], b = q[1];
    return d4{a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ void st4(d4* p, const d4& v) {
    double2* q = reinterpret_cast<double2*>(p);
    q[0] = make_double2(v.x, v.y);
    q[1] = make_double2(v.z, v.w);
}
__device__ __forceinline__ float4 ld4(const float4* p) { return *p; }
__device__ __forceinline__ void st4(float4* p, const float4& v) { *p = v; }

// Accumulator type of the residual gather and the widening into it: binary64
// for binary64 and binary32 fluxes (the float-float one is in fv_ff.cuh).
template <class T> struct Acc { typedef double type; };
__device__ __forceinline__ double acc_widen(double x) { return x; }
__device__ __forceinline__ double acc_widen(float x) { return (double)x; }

template <class T, class Q> __device__ __forceinline__ void to_arr(const Q& v, T* a) {
    a[0] = v.x; a[1] = v.y; a[2] = v.z; a[3] = v.w;
}

// "result = 0; result += a0*b0; result += a1*b1" (vector3d::dot_product).
template <class T> __device__ __forceinline__ T dot2(T a0, T a1, T b0, T b1) {
    T r = T(0);
    r += a0 * b0;
    r += a1 * b1;
    return r;
}
template <class T> __device__ __forceinline__ T sq2(T a0, T a1) { return dot2(a0, a1, a0, a1); }
template <class T> __device__ __forceinline__ T smax(T a, T b) { return (a < b) ? b : a; }  // std::max
template <class T> __device__ __forceinline__ T smin(T a, T b) { return (b < a) ? b : a; }  // std::min

__device__ __forceinline__ double dsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float dsqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double dpow(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float dpow(float x, float y) { return powf(x, y); }
__device__ __forceinline__ double dabs(double x) { return fabs(x); }
__device__ __forceinline__ float dabs(float x) { return fabsf(x); }

// Sutherland viscosity, LaminarFluxStrategy::computeMu (LaminarFluxStrategy.h:76-96):
// (1.0+cc)/(T+cc)*powf64(T,1.5)*sqrtf64(Gamma)*fs_Ma/fs_Re, evaluated left to right.
template <class T> __device__ __forceinline__ T sutherland(T temp, const MeshPrm& m) {
    T cc = T(m.cc);
    T a = (T(1.0) + cc) / (temp + cc);
    a = a * dpow(temp, T(1.5));
    a = a * T(m.sqrt_gamma);
    a = a * T(m.mach);
    a = a / T(m.re);
    return a;
}

// Primitive <-> conservative, TopologyHolderStrategy.cpp:48-109.
template <class T> __device__ __forceinline__ void cons_from_prim(const T* u, T* w) {
    T vm = T(0);
    vm += u[2] * u[2];
    w[2] = u[0] * u[2];
    vm += u[3] * u[3];
    w[3] = u[0] * u[3];
    w[0] = u[0];
    w[1] = u[1] / C<T>::gm1 + T(0.5) * u[0] * vm;
}
template <class T> __device__ __forceinline__ void prim_from_cons(const T* w, T* u) {
    u[0] = w[0];
    T vm = T(0);
    u[2] = w[2] / u[0];
    vm += u[2] * u[2];
    u[3] = w[3] / u[0];
    vm += u[3] * u[3];
    u[1] = C<T>::gm1 * (w[1] - T(0.5) * u[0] * vm);
}

// Face state of a boundary face.  Inviscid: HandleInvicidBoundary
// (BoundaryStrategy.h:197-335); viscous: HandleViscousBoundary (:73-195).
// ul: left-cell primitive.  Returns the error bits it raises.
template <class T>
__device__ __forceinline__ unsigned boundary_state(int bc, bool viscous, const T* ul, T nx, T ny,
                                                   const MeshPrm& m, T* ue) {
    const T G = C<T>::gamma, GM1 = C<T>::gm1;
    unsigned err = 0;
    if (bc == BC_WALL) {
        if (viscous) {
            ue[0] = ul[0]; ue[1] = ul[1]; ue[2] = T(0); ue[3] = T(0);
        } else {
            T vnl = dot2(ul[2], ul[3], nx, ny);
            T t0 = ul[2] - nx * vnl, t1 = ul[3] - ny * vnl;
            // binary64: the reference's absolute bound; binary32: scaled to its rounding
            T wtol = sizeof(T) == 8 ? T(1.0e-7) : T(1.0e-4) * (dabs(t0) + dabs(t1) + T(1));
            if (dot2(t0, t1, nx, ny) > wtol) err |= ERR_WALLTAN;
            ue[0] = ul[0]; ue[1] = ul[1]; ue[2] = t0; ue[3] = t1;
        }
        return err;
    }
    // far field (Riemann invariants)
    const T rinf = T(m.rho_inf), pinf = T(m.p_inf), uinf = T(m.u_inf), vinf = T(m.v_inf), cinf = T(m.c_inf);
    T vnl = dot2(ul[2], ul[3], nx, ny);
    T tl0 = ul[2] - nx * vnl, tl1 = ul[3] - ny * vnl;
    T vnr = dot2(uinf, vinf, nx, ny);
    T tr0 = uinf - nx * vnr, tr1 = vinf - ny * vnr;
    T rl = ul[0], pl = ul[1];
    if (dabs(vnr) < cinf) {
        T cl = dsqrt(G * pl / rl);
        T vnb = (vnl + vnr + T(2) * (cl - cinf) / GM1) / T(2);
        T cb = (vnl - vnr + T(2) * (cinf + cl) / GM1) * GM1 / T(4);
        T sb, e0, e1;
        if (vnr >= T(0)) {
            sb = (pl / dpow(rl, G));
            e0 = tl0 + nx * vnb; e1 = tl1 + ny * vnb;
        } else {
            sb = (pinf / dpow(rinf, G));
            e0 = tr0 + nx * vnb; e1 = tr1 + ny * vnb;
        }
        ue[0] = dpow((cb * cb / (G * sb)), (T(1.0) / (G - T(1))));
        ue[1] = ue[0] * cb * cb / G;
        ue[2] = e0; ue[3] = e1;
    } else if (vnr >= T(0)) {
        ue[0] = ul[0]; ue[1] = ul[1]; ue[2] = ul[2]; ue[3] = ul[3];
    } else {
        ue[0] = rinf; ue[1] = pinf; ue[2] = uinf; ue[3] = vinf;
    }
    return err;
}

// Venkatakrishnan limiter value for one face (Vankatakrishnan_Limiter.hpp:99-111).
template <class T> __device__ __forceinline__ T venkat(T d2, T d1max, T d1min, T eps2) {
    if (d2 > T(0))
        return (d1max * d1max + eps2 + T(2) * d2 * d1max) / (d1max * d1max + T(2) * d2 * d2 + d1max * d2 + eps2);
    if (d2 < T(0))
        return (d1min * d1min + eps2 + T(2) * d2 * d1min) / (d1min * d1min + T(2) * d2 * d2 + d1min * d2 + eps2);
    return T(1);
}

// HLLC flux of an interior face (HLLCFluxStrategy.cpp:40-133), F already
// multiplied by the face length.  Returns ERR_PSTAR when |p*_R - p*_L| >= 1e-10.
template <class T>
__device__ __forceinline__ unsigned hllc(const T* ql, const T* qr, T nx, T ny, T area, T* F) {
    const T G = C<T>::gamma, GM1 = C<T>::gm1;
    T dl = ql[0], pl = ql[1], ul = ql[2], vl = ql[3];
    T vnl = dot2(ul, vl, nx, ny);
    T cl = dsqrt(G * pl / dl);
    T hl = pl * G / (GM1 * dl) + T(0.5) * sq2(ul, vl);
    T dr = qr[0], pr = qr[1], ur = qr[2], vr = qr[3];
    T vnr = dot2(ur, vr, nx, ny);
    T cr = dsqrt(G * pr / dr);
    T hr = pr * G / (GM1 * dr) + T(0.5) * sq2(ur, vr);
    T el = dsqrt(dl) / (dsqrt(dl) + dsqrt(dr));
    T er = T(1) - el;
    T ht = el * hl + er * hr;
    T vnt = el * vnl + er * vnr;
    T ct = dsqrt(GM1 * (ht - T(0.5) * (vnt * vnt)));
    T sl = smin(vnl - cl, vnt - ct);
    T sr = smax(vnt + ct, vnr + cr);
    T sm = (dr * vnr * (sr - vnr) - dl * vnl * (sl - vnl) + pl - pr) / (dr * (sr - vnr) - dl * (sl - vnl));
    T ps = dl * (vnl - sl) * (vnl - sm) + pl;
    T ps2 = dr * (vnr - sr) * (vnr - sm) + pr;
    // The reference's absolute 1e-10 bound assumes binary64; binary32 rounding of
    // the same expression is ~1e-7 relative, so that form checks 1e-4 relative.
    T ptol = sizeof(T) == 8 ? T(1e-10) : T(1e-4) * smax(dabs(ps), T(1));
    unsigned err = (dabs(ps2 - ps) < ptol) ? 0u : ERR_PSTAR;
    if (sl > T(0)) {
        T re = pl / GM1 + T(0.5) * dl * sq2(ul, vl);
        F[0] = vnl * dl * area;
        F[1] = vnl * (re + pl) * area;
        F[2] = (vnl * dl * ul + pl * nx) * area;
        F[3] = (vnl * dl * vl + pl * ny) * area;
    } else if (sr < T(0)) {
        T re = pr / GM1 + T(0.5) * dr * sq2(ur, vr);
        F[0] = vnr * dr * area;
        F[1] = vnr * (re + pr) * area;
        F[2] = (vnr * dr * ur + pr * nx) * area;
        F[3] = (vnr * dr * vr + pr * ny) * area;
    } else {
        T s, vn, d, p, u, v;
        if (sm < T(0)) { s = sr; vn = vnr; d = dr; p = pr; u = ur; v = vr; }
        else { s = sl; vn = vnl; d = dl; p = pl; u = ul; v = vl; }
        T re = p / GM1 + T(0.5) * d * sq2(u, v);
        T f0 = (s - vn) * d / (s - sm);
        T f1 = ((s - vn) * re - p * vn + ps * sm) / (s - sm);
        T f2 = ((s - vn) * d * u + (ps - p) * nx) / (s - sm);
        T f3 = ((s - vn) * d * v + (ps - p) * ny) / (s - sm);
        F[0] = f0 * sm * area;
        F[1] = (f1 + ps) * sm * area;
        F[2] = (f2 * sm + ps * nx) * area;
        F[3] = (f3 * sm + ps * ny) * area;
    }
    return err;
}

// Wall (pressure only) and far-field (Euler flux of the face state) fluxes
// (HLLCFluxStrategy.cpp:22-48).
template <class T> __device__ __forceinline__ void wall_flux(const T* q, T nx, T ny, T area, T* F) {
    F[0] = T(0) * area;
    F[1] = T(0) * area;
    F[2] = q[1] * nx * area;
    F[3] = q[1] * ny * area;
}
template <class T> __device__ __forceinline__ void euler_flux(const T* q, T nx, T ny, T area, T* F) {
    const T GM1 = C<T>::gm1;
    T d = q[0], p = q[1], u = q[2], v = q[3];
    T re = p / GM1 + T(0.5) * d * sq2(u, v);
    T vn = dot2(u, v, nx, ny);
    F[0] = vn * d * area;
    F[1] = vn * (re + p) * area;
    F[2] = (vn * d * u + p * nx) * area;
    F[3] = (vn * d * v + p * ny) * area;
}

// Convective flux of a conservative state, ConservativeParam2ConvectiveFlux
// (TopologyHolderStrategy.cpp:129-141).
template <class T> __device__ __forceinline__ void conv_flux_w(const T* w, T nx, T ny, T* F) {
    const T GM1 = C<T>::gm1;
    T u = w[2] / w[0], v = w[3] / w[0];
    T vn = dot2(u, v, nx, ny);
    T d = w[0];
    T p = GM1 * (w[1] - T(0.5) * d * sq2(u, v));
    F[0] = w[0] * vn;
    F[1] = (w[1] + p) * vn;
    F[2] = w[2] * vn + p * nx;
    F[3] = w[3] * vn + p * ny;
}

}  // namespace cfdgb

#include "fv_ff.cuh"
