// Kernels of one residual evaluation and of the time integrators.
//
// Data layout in HBM (all meshes of a case concatenated; cell and face indices
// are global):
//   faces  lr[f] = (left, right|BC)             int2
//          fg0[f] = (nx, ny, length, 125*vol_left)   fg1[f] = (xf-xl, yf-yl, xf-xr, yf-yr)
//          fvis[f] = (xr-xl, yr-yl, |xr-xl|^2, 0)    (boundary: xf-xl)
//   cells  cgeo[c] = (vol, xc, yc, 0); cface[c] = 4 signed face codes in ascending
//          face order: +(f+1) if c is the left cell of f, -(f+1) if right, 0 = none.
//   state  U (primitive) / W (conservative) / R as 32-byte records per cell.
//
// A residual is four passes, none of which scatters:
//   face_state   (face-centric)  face value U_edge, convective/viscous spectral
//                                contributions, mu at faces
//   cell_grad    (cell-centric)  Green-Gauss gradients, spectral radii, min/max
//                                over neighbours and the Venkatakrishnan limiter
//   face_flux    (face-centric)  limited reconstruction + HLLC (+ laminar flux)
//   cell_update  (cell-centric)  residual gather in ascending face order, then the
//                                integrator's per-cell work (RK stage / LU-SGS D)
// Every per-cell sum visits the cell's faces in ascending face index, the order
// in which the reference's face loops reach that cell, so sums round the same.
#pragma once
#include <type_traits>

#include "fv_device.cuh"

namespace cfdgb {

template <class T> using v4 = typename V4<T>::type;
template <class T> using v2 = typename V2<T>::type;

__device__ __forceinline__ int code_face(int code) { return (code > 0 ? code : -code) - 1; }

// ---------------------------------------------------------------------------
// face_state: BoundaryStrategy::HandleBoundary + the per-edge part of
// solveSpectralRadius (Euler2D.cpp:242-267, ViscousFlow2D.cpp:220-253) and of
// LaminarFluxStrategy::computeMu for edges.
//
// With the SST model coupled (mutc != null; binary64 and float-float forms:
// ViscousFlow2D with isLaminar() false, ViscousFlow2D.h:118-154) the face also
// gets its eddy viscosity (ComputeTurbulenceViscousCoefficient's face loop,
// SSTKWStrategy.h:749-777) into mutf, and the viscous spectral radius uses
// mu/Pr + mu_t/Prt.
template <class T, bool VISC, int CONTRACT = 0>
__global__ void __launch_bounds__(256) k_face_state(int nf, const int2* __restrict__ lr, const int* __restrict__ fmesh,
                                                    const MeshPrm* __restrict__ prm, const v4<T>* __restrict__ fg0,
                                                    const v4<T>* __restrict__ U, v4<T>* __restrict__ Ue,
                                                    v2<T>* __restrict__ fspec, T* __restrict__ mue,
                                                    unsigned* __restrict__ err, const double* __restrict__ mutc,
                                                    double* __restrict__ mutf) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const T G = C<T>::gamma;
    int2 e = lr[f];
    v4<T> g = ld4(fg0 + f);
    T nx = g.x, ny = g.y, A = g.z;
    T ue[4];
    if (e.y >= 0) {
        T a[4], b[4];
        to_arr(ld4(U + e.x), a);
        to_arr(ld4(U + e.y), b);
#pragma unroll
        for (int j = 0; j < 4; j++) ue[j] = (a[j] + b[j]) / T(2);
    } else {
        T a[4];
        to_arr(ld4(U + e.x), a);
        MeshPrm m = prm[fmesh[f]];
        unsigned bad = boundary_state<T>(e.y, VISC, a, nx, ny, m, ue);
        if (bad) atomicOr(err, bad);
    }
    v4<T> o;
    o.x = ue[0]; o.y = ue[1]; o.z = ue[2]; o.w = ue[3];
    st4(Ue + f, o);
    T c = dsqrt(G * ue[1] / ue[0]);
    T vn = dot2(ue[2], ue[3], nx, ny);
    v2<T> s;
    s.x = (dabs(vn) + c) * A;
    s.y = T(0);
    if (VISC) {
        MeshPrm m = prm[fmesh[f]];
        T mu = sutherland<T>(ue[1] / ue[0], m);
        mue[f] = mu;
        T mpr = mu / C<T>::pr;
        if constexpr (!std::is_same<T, float>::value) {
            if (mutc) {
                double mf;
                if (e.y >= 0) mf = 0.5 * (mutc[e.x] + mutc[e.y]);
                else if (e.y == BC_WALL) mf = 0.0;
                else mf = (double)dot2(ue[2], ue[3], nx, ny) > 0.0 ? mutc[e.x] : m.sst_mut;
                mutf[f] = mf;
                mpr = mu / C<T>::pr + T(mf) / T(0.9);
            }
        }
        s.y = smax(T(4) / (T(3.0) * ue[0]), G / ue[0]) * mpr * A * A;
    }
    fspec[f] = s;
}

// ---------------------------------------------------------------------------
// cell_grad: solveGradient (Euler2D.cpp:209-240 / ViscousFlow2D.cpp:181-218),
// the per-cell sums of solveSpectralRadius, computeMu for cells, and the
// Venkatakrishnan limiter (Vankatakrishnan_Limiter.hpp:69-177,186-200).
template <class T, bool VISC, int CONTRACT = 0>
__global__ void __launch_bounds__(256) k_cell_grad(
    int nc, const int4* __restrict__ cface, const int2* __restrict__ lr, const int* __restrict__ cmesh,
    const MeshPrm* __restrict__ prm, const v4<T>* __restrict__ cgeo, const v4<T>* __restrict__ fg0,
    const v4<T>* __restrict__ fg1, const v4<T>* __restrict__ U, const v4<T>* __restrict__ Ue,
    const v2<T>* __restrict__ fspec, int first_order, v4<T>* __restrict__ grad, v4<T>* __restrict__ phi,
    T* __restrict__ specc, T* __restrict__ specv, v2<T>* __restrict__ gradT, T* __restrict__ mu) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    int4 cf = cface[c];
    int codes[4] = {cf.x, cf.y, cf.z, cf.w};
    T uc[4];
    to_arr(ld4(U + c), uc);
    T vol = ld4(cgeo + c).x;
    T gx[4] = {T(0), T(0), T(0), T(0)}, gy[4] = {T(0), T(0), T(0), T(0)};
    T gtx = T(0), gty = T(0);
    T sc = T(0), sv = T(0);
    T umax[4], umin[4];
#pragma unroll
    for (int j = 0; j < 4; j++) { umax[j] = uc[j]; umin[j] = uc[j]; }
#pragma unroll
    for (int s = 0; s < 4; s++) {
        int code = codes[s];
        if (code == 0) break;
        int f = code_face(code);
        bool left = code > 0;
        v4<T> g = ld4(fg0 + f);
        T nx = g.x, ny = g.y, A = g.z;
        T ue[4];
        to_arr(ld4(Ue + f), ue);
#pragma unroll
        for (int j = 0; j < 4; j++) {
            T tx = nx * (A * ue[j]), ty = ny * (A * ue[j]);
            if (left) { gx[j] = gx[j] + tx; gy[j] = gy[j] + ty; }
            else { gx[j] = gx[j] - tx; gy[j] = gy[j] - ty; }
        }
        v2<T> sp = fspec[f];
        sc += sp.x;
        if (VISC) {
            T et = ue[1] / ue[0];
            T tx = nx * (A * et), ty = ny * (A * et);
            if (left) { gtx = gtx + tx; gty = gty + ty; }
            else { gtx = gtx - tx; gty = gty - ty; }
            sv += sp.y / vol;
        }
        int2 e = lr[f];
        int other = left ? e.y : e.x;
        if (other >= 0) {
            T uo[4];
            to_arr(ld4(U + other), uo);
#pragma unroll
            for (int j = 0; j < 4; j++) { umax[j] = smax(umax[j], uo[j]); umin[j] = smin(umin[j], uo[j]); }
        }
    }
#pragma unroll
    for (int j = 0; j < 4; j++) { gx[j] = gx[j] / vol; gy[j] = gy[j] / vol; }
    T lim[4] = {T(1), T(1), T(1), T(1)};
    T d1max[4], d1min[4];
#pragma unroll
    for (int j = 0; j < 4; j++) { d1max[j] = umax[j] - uc[j]; d1min[j] = umin[j] - uc[j]; }
#pragma unroll
    for (int s = 0; s < 4; s++) {
        int code = codes[s];
        if (code == 0) break;
        int f = code_face(code);
        T eps2 = ld4(fg0 + f).w;
        v4<T> d = ld4(fg1 + f);
        T dx = code > 0 ? d.x : d.z, dy = code > 0 ? d.y : d.w;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            T d2 = dot2(gx[j], gy[j], dx, dy);
            lim[j] = smin(lim[j], venkat(d2, d1max[j], d1min[j], eps2));
        }
    }
    if (first_order) {
#pragma unroll
        for (int j = 0; j < 4; j++) lim[j] = T(0);
    }
    v4<T> g0, g1, p;
    g0.x = gx[0]; g0.y = gy[0]; g0.z = gx[1]; g0.w = gy[1];
    g1.x = gx[2]; g1.y = gy[2]; g1.z = gx[3]; g1.w = gy[3];
    p.x = lim[0]; p.y = lim[1]; p.z = lim[2]; p.w = lim[3];
    st4(grad + 2 * (size_t)c, g0);
    st4(grad + 2 * (size_t)c + 1, g1);
    st4(phi + c, p);
    specc[c] = sc;
    if (VISC) {
        v2<T> t;
        t.x = gtx / vol;
        t.y = gty / vol;
        gradT[c] = t;
        specv[c] = sv;
        MeshPrm m = prm[cmesh[c]];
        mu[c] = sutherland<T>(uc[1] / uc[0], m);
    }
}

// ---------------------------------------------------------------------------
// face_flux: HLLCFluxStrategy::updateLeftRight + computeFlux
// (HLLCFluxStrategy.h:35-100, HLLCFluxStrategy.cpp:4-170) and
// LaminarFluxStrategy::computeFlux(int) (LaminarFluxStrategy.h:110-216).
// Writes the convective and the viscous flux of each face separately so the
// gather can add them in the reference's two-loop order.  With the SST model
// coupled (mutf != null; binary64 and float-float forms) the viscous flux uses
// mu + mu_t and mu/Pr + mu_t/Prt (getMuEdge / getMuOverPrEdge,
// ViscousFlow2D.h:128-145).
template <class T, bool VISC, int CONTRACT = 0>
__global__ void __launch_bounds__(256) k_face_flux(
    int nf, const int2* __restrict__ lr, const v4<T>* __restrict__ fg0, const v4<T>* __restrict__ fg1,
    const v4<T>* __restrict__ fvis, const v4<T>* __restrict__ U, const v4<T>* __restrict__ grad,
    const v4<T>* __restrict__ phi, const v4<T>* __restrict__ Ue, const T* __restrict__ mue,
    const v2<T>* __restrict__ gradT, v4<T>* __restrict__ Fc, v4<T>* __restrict__ Fv, unsigned* __restrict__ err,
    const double* __restrict__ mutf) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const T G = C<T>::gamma, GM1 = C<T>::gm1;
    int2 e = lr[f];
    v4<T> g = ld4(fg0 + f);
    T nx = g.x, ny = g.y, A = g.z;
    T F[4];
    T ul[4], ur[4];
    v4<T> gl0, gl1, gr0, gr1;
    if (e.y >= 0) {
        v4<T> d = ld4(fg1 + f);
        T pl[4], pr[4];
        to_arr(ld4(U + e.x), ul);
        to_arr(ld4(U + e.y), ur);
        to_arr(ld4(phi + e.x), pl);
        to_arr(ld4(phi + e.y), pr);
        gl0 = ld4(grad + 2 * (size_t)e.x);
        gl1 = ld4(grad + 2 * (size_t)e.x + 1);
        gr0 = ld4(grad + 2 * (size_t)e.y);
        gr1 = ld4(grad + 2 * (size_t)e.y + 1);
        T glx[4] = {gl0.x, gl0.z, gl1.x, gl1.z}, gly[4] = {gl0.y, gl0.w, gl1.y, gl1.w};
        T grx[4] = {gr0.x, gr0.z, gr1.x, gr1.z}, gry[4] = {gr0.y, gr0.w, gr1.y, gr1.w};
        T ql[4], qr[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            ql[j] = dot2(glx[j], gly[j], d.x, d.y) * pl[j] + ul[j];
            qr[j] = dot2(grx[j], gry[j], d.z, d.w) * pr[j] + ur[j];
        }
        unsigned bad = hllc<T>(ql, qr, nx, ny, A, F);
        if (bad) atomicOr(err, bad);
    } else {
        T q[4];
        to_arr(ld4(Ue + f), q);
        if (e.y == BC_WALL) wall_flux<T>(q, nx, ny, A, F);
        else euler_flux<T>(q, nx, ny, A, F);
    }
    v4<T> o;
    o.x = F[0]; o.y = F[1]; o.z = F[2]; o.w = F[3];
    st4(Fc + f, o);
    if (!VISC) return;
    // viscous flux
    T mu = mue[f];
    T mpr = mu / C<T>::pr;
    if constexpr (!std::is_same<T, float>::value) {
        if (mutf) {
            const T mt = T(mutf[f]);
            mpr = mu / C<T>::pr + mt / T(0.9);
            mu = mu + mt;
        }
    }
    T eff = T(2.0) / T(3.0) * mu;
    T g0x, g0y, g1x, g1y, gtx, gty;  // d(u)/dx,dy ; d(v)/dx,dy ; dT/dx,dy at the face
    if (e.y >= 0) {
        v4<T> lv = ld4(fvis + f);
        T lx = lv.x, ly = lv.y, l2 = lv.z;
        // u component (gradU[2]) and v component (gradU[3])
        T ax = (gl1.x + gr1.x) * T(0.5), ay = (gl1.y + gr1.y) * T(0.5);
        T k = (ur[2] - ul[2] - dot2(ax, ay, lx, ly)) / l2;
        g0x = ax + lx * k; g0y = ay + ly * k;
        ax = (gl1.z + gr1.z) * T(0.5); ay = (gl1.w + gr1.w) * T(0.5);
        k = (ur[3] - ul[3] - dot2(ax, ay, lx, ly)) / l2;
        g1x = ax + lx * k; g1y = ay + ly * k;
        v2<T> tl = gradT[e.x], tr = gradT[e.y];
        ax = (tl.x + tr.x) * T(0.5); ay = (tl.y + tr.y) * T(0.5);
        T rt = ur[1] / ur[0];
        T lt = ul[1] / ul[0];
        k = (rt - lt - dot2(ax, ay, lx, ly)) / l2;
        gtx = ax + lx * k; gty = ay + ly * k;
    } else {
        v4<T> q1 = ld4(grad + 2 * (size_t)e.x + 1);
        g0x = q1.x; g0y = q1.y; g1x = q1.z; g1y = q1.w;
        if (e.y == BC_WALL) { gtx = T(0); gty = T(0); }
        else { v2<T> t = gradT[e.x]; gtx = t.x; gty = t.y; }
    }
    v4<T> qe = ld4(Ue + f);
    T ve0 = qe.z, ve1 = qe.w;
    T txx = eff * (T(2.0) * g0x - g1y);
    T tyy = eff * (T(2.0) * g1y - g0x);
    T txy = mu * (g0y + g1x);
    T qx = -G / GM1 * mpr * gtx;
    T qy = -G / GM1 * mpr * gty;
    v4<T> v;
    v.x = T(0.0);
    v.y = ((ve0 * txx + ve1 * txy - qx) * nx + (ve0 * txy + ve1 * tyy - qy) * ny) * A;
    v.z = (txx * nx + txy * ny) * A;
    v.w = (txy * nx + tyy * ny) * A;
    st4(Fv + f, v);
}

// (CONTRACT only names the instantiation: the binary64 residual is built twice,
// in k_fp64.cu without multiply-add contraction (the reference's bits) and in
// k_fp64fma.cu with it (the mixed form, whose residual need not equal the
// reference's bits), and distinct template arguments keep the two apart.)

// ---------------------------------------------------------------------------
// cell_update: residual gather (R[lC] += F, R[rC] -= F in HLLCFluxStrategy.cpp:
// 150-168, then R[lC] -= Fv, R[rC] += Fv in LaminarFluxStrategy.h:192-210),
// followed by the integrator's per-cell work.  The residual is always summed in
// binary64 (the fast form's fluxes are widened here).
enum UpdMode { UPD_RESID = 0, UPD_RK = 1, UPD_LUSGS = 2 };

template <class T, bool VISC, int MODE>
__global__ void __launch_bounds__(256) k_cell_update(
    int nc, const int4* __restrict__ cface, const d4* __restrict__ cgeo64, const v4<T>* __restrict__ Fc,
    const v4<T>* __restrict__ Fv, const T* __restrict__ specc, const T* __restrict__ specv, double cfl,
    int stage, double alpha, d4* __restrict__ R, d4* __restrict__ U64, d4* __restrict__ W, d4* __restrict__ W0,
    double* __restrict__ dt, double* __restrict__ diag, v4<T>* __restrict__ Ulow, const float* __restrict__ cflmul,
    int turb) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    int4 cf = cface[c];
    int codes[4] = {cf.x, cf.y, cf.z, cf.w};
    typedef typename Acc<T>::type A;  // binary64, or float-float for float-float fluxes
    A ra[4] = {A(0.0), A(0.0), A(0.0), A(0.0)};
#pragma unroll
    for (int s = 0; s < 4; s++) {
        int code = codes[s];
        if (code == 0) break;
        T fl[4];
        to_arr(ld4(Fc + code_face(code)), fl);
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (code > 0) ra[j] += acc_widen(fl[j]);
            else ra[j] -= acc_widen(fl[j]);
        }
    }
    if (VISC) {
#pragma unroll
        for (int s = 0; s < 4; s++) {
            int code = codes[s];
            if (code == 0) break;
            T fl[4];
            to_arr(ld4(Fv + code_face(code)), fl);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                if (code > 0) ra[j] -= acc_widen(fl[j]);
                else ra[j] += acc_widen(fl[j]);
            }
        }
    }
    const double r[4] = {(double)ra[0], (double)ra[1], (double)ra[2], (double)ra[3]};
    st4(R + c, d4{r[0], r[1], r[2], r[3]});
    if (MODE == UPD_RESID) return;
    double vol = cgeo64[c].x;
    double sc = (double)specc[c];
    if (MODE == UPD_RK) {
        // RungeKuttaStrategy::UpdateSerial (RungeKuttaStrategy.h:39-72): dt frozen at
        // stage 0 (SolveTime), W_now = W0 + a*dt*(-R)/vol, then initializePrimData.
        double w0[4], dtc;
        if (stage == 0) {
            double u[4];
            to_arr(ld4(U64 + c), u);
            cons_from_prim<double>(u, w0);
            st4(W0 + c, d4{w0[0], w0[1], w0[2], w0[3]});
            dtc = cfl * vol / sc;
            dt[c] = dtc;
        } else {
            to_arr(ld4(W0 + c), w0);
            dtc = dt[c];
        }
        double wn[4], un[4];
#pragma unroll
        for (int j = 0; j < 4; j++) wn[j] = w0[j] + alpha * dtc * (-r[j]) / vol;
        prim_from_cons<double>(wn, un);
        st4(W + c, d4{wn[0], wn[1], wn[2], wn[3]});
        st4(U64 + c, d4{un[0], un[1], un[2], un[3]});
        if (Ulow) {
            v4<T> q;
            q.x = (T)un[0]; q.y = (T)un[1]; q.z = (T)un[2]; q.w = (T)un[3];
            st4(Ulow + c, q);
        }
    } else {
        // SolveTime + TopologyHolderStrategy::SolveDiag (TopologyHolderStrategy.cpp:190-215);
        // an optional per-cell CFL multiplier (local CFL controller) scales the CFL.
        // With the SST model coupled, SolveTime's turbulent branch (ViscousFlow2D.h:223-242):
        // dt = CFL vol / (spec_c + 4 spec_v).
        double cl = cflmul ? cfl * (double)cflmul[c] : cfl;
        double dtc = turb ? cl * vol / (sc + 4.0 * (double)specv[c]) : cl * vol / sc;
        dt[c] = dtc;
        double OMEGAN = 1.5;
        double d = vol / dtc + 0.5 * OMEGAN * sc;
        if (VISC) d += (double)specv[c];
        diag[c] = d;
    }
}

}  // namespace cfdgb
