// SST k-omega turbulence residual of the reference (SSTKWStrategy.h:615-1013)
// on the device: face values and eddy viscosity, Green-Gauss gradients of k
// and omega with the blending functions F1 / F2, upwind convective and
// corrected-gradient viscous face fluxes, the production / destruction /
// cross-diffusion sources, the two-equation LU-SGS diagonal (SolveDiag,
// :170-192) and the eddy-viscosity update (UpdatePrimitiveVariables, :194-223).
//
// Compiled with -fmad=false and written with the reference's operation order,
// so that everything except tanh (F1, F2) reproduces it bit for bit.  As in
// the flow residual there is no scatter: faces compute face quantities, cells
// gather their faces in ascending face order, which is the order of the
// reference's edge loops.
#include <cuda_runtime.h>

#include <type_traits>

#include "case.hpp"
#include "sweep_flow.cuh"
#include "fv_ff.cuh"

namespace cfdgb {
namespace {

// SSTkomegaModel constants (SSTKWStrategy.h:14-30)
constexpr double beta1 = 0.075, beta2 = 0.0828, sigma_k1 = 0.85, sigma_k2 = 1.0, sigma_w1 = 0.5,
                 sigma_w2 = 0.856, Cw1 = 0.533, Cw2 = 0.440, a1 = 0.31, beta_star = 0.09;

__device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }  // std::max
__device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }  // std::min

// Where the model's passes read the flow's intermediates and the model's own
// state.  T = double: the binary64 arrays (the plain and MIXED forms; with
// -fmad=false and the reference's operation order this reproduces its SST
// functions).  T = ff (MIXFF): the float-float residual's own arrays and
// float-float copies of k, omega, mu_t and the wall distance made at the start
// of the model's passes, so the model runs on the FP32 pipe like the flow's
// residual; its intermediates (face k and omega, gradients, F1 / F2, face
// fluxes) are stored as pairs in the same 8-byte slots, and the residual and
// diagonal are written back in binary64.  tanh (F1, F2) is evaluated in
// binary64 in both.
template <class T> struct SstIo;
template <> struct SstIo<double> {
    typedef d4 V;
    static __device__ __forceinline__ double rho(const DevArrays& d, int c) { return d.U[c].x; }
    static __device__ __forceinline__ d4 ue(const DevArrays& d, int f) { return d.Ue[f]; }
    static __device__ __forceinline__ double mue(const DevArrays& d, int f) { return d.mue[f]; }
    static __device__ __forceinline__ double mu(const DevArrays& d, int c) { return d.mu[c]; }
    static __device__ __forceinline__ d4 fgeo(const DevArrays& d, int f) { return d.fgeo[f]; }
    static __device__ __forceinline__ d4 cgeo(const DevArrays& d, int c) { return d.cgeo[c]; }
    static __device__ __forceinline__ double kw(const DevArrays& d, int i) { return d.sstT[i]; }
    static __device__ __forceinline__ double mut(const DevArrays& d, int c) { return d.sstMut[c]; }
    static __device__ __forceinline__ double walld(const DevArrays& d, int c) { return d.walld[c]; }
    static __device__ __forceinline__ d4 gradu(const DevArrays& d, int c) { return d.grad[2 * c + 1]; }
    static __device__ __forceinline__ double specc(const DevArrays& d, int c) { return d.specc[c]; }
    static __device__ __forceinline__ double specv(const DevArrays& d, int c) { return d.specv[c]; }
    static __device__ __forceinline__ double mutf(const DevArrays& d, int f) { return d.sstMutf[f]; }
    static __device__ __forceinline__ double dt(const DevArrays& d, int c) { return d.dt[c]; }
    static __device__ __forceinline__ double abs_(double x) { return fabs(x); }
    static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
    static __device__ __forceinline__ double tanh_(double x) { return tanh(x); }
};
template <> struct SstIo<ff> {
    typedef q4 V;
    static __device__ __forceinline__ ff rho(const DevArrays& d, int c) { return reinterpret_cast<const ff*>(d.Uq)[4 * (size_t)c]; }
    static __device__ __forceinline__ q4 ue(const DevArrays& d, int f) { return ld4(d.Ueq + f); }
    static __device__ __forceinline__ ff mue(const DevArrays& d, int f) { return d.mueq[f]; }
    static __device__ __forceinline__ ff mu(const DevArrays& d, int c) { return d.muq[c]; }
    static __device__ __forceinline__ q4 fgeo(const DevArrays& d, int f) { return ld4(d.fg0q + f); }  // nx, ny, length
    static __device__ __forceinline__ q4 cgeo(const DevArrays& d, int c) { return ld4(d.cgeoq + c); }
    static __device__ __forceinline__ ff kw(const DevArrays& d, int i) { return d.sstTq[i]; }
    static __device__ __forceinline__ ff mut(const DevArrays& d, int c) { return d.sstMutq[c]; }
    static __device__ __forceinline__ ff walld(const DevArrays& d, int c) { return d.walldq[c]; }
    static __device__ __forceinline__ q4 gradu(const DevArrays& d, int c) { return ld4(d.gradq + 2 * (size_t)c + 1); }
    static __device__ __forceinline__ ff specc(const DevArrays& d, int c) { return d.speccq[c]; }
    static __device__ __forceinline__ ff specv(const DevArrays& d, int c) { return d.specvq[c]; }
    static __device__ __forceinline__ ff mutf(const DevArrays& d, int f) { return ff(d.sstMutf[f]); }
    static __device__ __forceinline__ ff dt(const DevArrays& d, int c) { return ff(d.dt[c]); }
    static __device__ __forceinline__ ff abs_(ff x) { return ff_abs(x); }
    static __device__ __forceinline__ ff sqrt_(ff x) { return ff_sqrt(x); }
    static __device__ __forceinline__ ff tanh_(ff x) { return ff(tanh((double)x)); }
};
template <class T> __device__ __forceinline__ T tmax(T a, T b) { return (a < b) ? b : a; }  // std::max
template <class T> __device__ __forceinline__ T tmin(T a, T b) { return (b < a) ? b : a; }  // std::min
template <class T> __device__ __forceinline__ T* as(double* p) { return reinterpret_cast<T*>(p); }
template <class T> __device__ __forceinline__ const T* as(const double* p) { return reinterpret_cast<const T*>(p); }

// The float-float copies of the model's state the MIXFF passes read.
__global__ void k_sst_to_ff(DevArrays d) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.nc) return;
    d.sstTq[2 * c] = ff(d.sstT[2 * c]);
    d.sstTq[2 * c + 1] = ff(d.sstT[2 * c + 1]);
    d.sstMutq[c] = ff(d.sstMut[c]);
    d.walldq[c] = ff(d.walld[c]);
}

// ComputeFaceTValue (:615-659) and the face loop of
// ComputeTurbulenceViscousCoefficient (:749-777).
template <class T>
__global__ void k_sst_face(DevArrays d) {
    typedef SstIo<T> IO;
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= d.nf) return;
    const int2 lr = d.lr[f];
    const auto g = IO::fgeo(d, f);
    const MeshPrm& P = d.prm[d.fmesh[f]];
    const int l = lr.x, r = lr.y;
    T t0, t1, mf;
    if (r >= 0) {
        t0 = T(0.5) * (IO::kw(d, 2 * l) + IO::kw(d, 2 * r));
        t1 = T(0.5) * (IO::kw(d, 2 * l + 1) + IO::kw(d, 2 * r + 1));
        mf = T(0.5) * (IO::mut(d, l) + IO::mut(d, r));
    } else if (r == BC_WALL) {
        const T dis = IO::walld(d, l);
        t0 = T(0.0);
        t1 = T(10.0) * T(6.0) * IO::mue(d, f) / (IO::ue(d, f).x * T(beta1) * dis * dis);
        mf = T(0.0);
    } else {
        const auto ue = IO::ue(d, f);
        T vn = T(0);
        vn += ue.z * g.x;
        vn += ue.w * g.y;
        if (vn > T(0.0)) {
            t0 = IO::kw(d, 2 * l);
            t1 = IO::kw(d, 2 * l + 1);
        } else {
            t0 = T(P.sst_k);
            t1 = T(P.sst_w);
        }
        mf = vn > T(0.0) ? IO::mut(d, l) : T(P.sst_mut);
    }
    T* Tf = as<T>(d.sstTf);
    Tf[2 * f] = t0;
    Tf[2 * f + 1] = t1;
    if (!d.turb) d.sstMutf[f] = (double)mf;  // coupled, the flow's face_state pass has formed it (for the viscous radius)
}

// ComputeCellTGradient (:662-692) and ComputeSSTf1f2 (:695-722).
template <class T>
__global__ void k_sst_cell(DevArrays d) {
    typedef SstIo<T> IO;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.nc) return;
    const int4 cf = d.cface[c];
    const int codes[4] = {cf.x, cf.y, cf.z, cf.w};
    const T* Tf = as<T>(d.sstTf);
    T gk0 = T(0), gk1 = T(0), gw0 = T(0), gw1 = T(0);
    for (int s = 0; s < 4; s++) {
        const int code = codes[s];
        if (code == 0) continue;
        const int f = code > 0 ? code - 1 : -code - 1;
        const auto g = IO::fgeo(d, f);
        const T ak = g.z * Tf[2 * f], aw = g.z * Tf[2 * f + 1];
        const T vk0 = g.x * ak, vk1 = g.y * ak, vw0 = g.x * aw, vw1 = g.y * aw;
        if (code > 0) {
            gk0 = gk0 + vk0; gk1 = gk1 + vk1; gw0 = gw0 + vw0; gw1 = gw1 + vw1;
        } else {
            gk0 = gk0 - vk0; gk1 = gk1 - vk1; gw0 = gw0 - vw0; gw1 = gw1 - vw1;
        }
    }
    const T vol = IO::cgeo(d, c).x;
    gk0 = gk0 / vol; gk1 = gk1 / vol; gw0 = gw0 / vol; gw1 = gw1 / vol;
    T* G = as<T>(d.sstG);
    G[4 * c] = gk0; G[4 * c + 1] = gk1; G[4 * c + 2] = gw0; G[4 * c + 3] = gw1;
    T gradVal = T(0);
    gradVal += gk0 * gw0;
    gradVal += gk1 * gw1;
    const T rho = IO::rho(d, c), dis = IO::walld(d, c), K = IO::kw(d, 2 * c), w = IO::kw(d, 2 * c + 1),
            muL = IO::mu(d, c);
    const T CD_kw = tmax(T(2.0) * rho * T(sigma_w2) / w * gradVal, T(1.0e-20));
    T arg1 = tmax(IO::sqrt_(K) / (T(0.09) * w * dis), T(500.0) * muL / (rho * w * dis * dis));
    arg1 = tmin(arg1, T(4.0) * rho * T(sigma_w2) * K / (CD_kw * dis * dis));
    const T arg2 = tmax(T(2.0) * IO::sqrt_(K) / (T(0.09) * w * dis), T(500.0) * muL / (rho * w * dis * dis));
    as<T>(d.sstF1)[c] = IO::tanh_(arg1 * arg1 * arg1 * arg1);
    as<T>(d.sstF2)[c] = IO::tanh_(arg2 * arg2);
}

// SolveConvectiveTFlux (:783-831) and SolveViscousTFlux (:834-920).  The
// interior face gradient is corrected along the centre line one component
// after the other, the y component using the already corrected x component,
// as the reference does.
template <class T>
__global__ void k_sst_flux(DevArrays d) {
    typedef SstIo<T> IO;
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= d.nf) return;
    const int2 lr = d.lr[f];
    const int l = lr.x, r = lr.y;
    const auto g = IO::fgeo(d, f);
    const T nx = g.x, ny = g.y, A = g.z;
    const auto ue = IO::ue(d, f);
    const T* Tf = as<T>(d.sstTf);
    const T* F1 = as<T>(d.sstF1);
    const T* G = as<T>(d.sstG);
    T vn = T(0);
    vn += ue.z * nx;
    vn += ue.w * ny;
    T fc0, fc1;
    if (r >= 0) {
        const T vp = T(0.5) * (vn + IO::abs_(vn)), vs = T(0.5) * (vn - IO::abs_(vn));
        const T rl = IO::rho(d, l), rr = IO::rho(d, r);
        fc0 = IO::kw(d, 2 * l) * rl * vp * A + IO::kw(d, 2 * r) * rr * vs * A;
        fc1 = IO::kw(d, 2 * l + 1) * rl * vp * A + IO::kw(d, 2 * r + 1) * rr * vs * A;
    } else {
        fc0 = vn * ue.x * Tf[2 * f] * A;
        fc1 = vn * ue.x * Tf[2 * f + 1] * A;
    }
    T face_f1, g00, g01, g10, g11;
    if (r >= 0) {
        const auto cl = IO::cgeo(d, l), cr = IO::cgeo(d, r);
        const T l0 = cr.y - cl.y, l1 = cr.z - cl.z;
        T L2 = T(0);
        L2 += l0 * l0;
        L2 += l1 * l1;
        face_f1 = T(0.5) * (F1[l] + F1[r]);
        const T* Gl = G + 4 * l;
        const T* Gr = G + 4 * r;
        g00 = (Gl[0] + Gr[0]) * T(0.5);
        g01 = (Gl[1] + Gr[1]) * T(0.5);
        g10 = (Gl[2] + Gr[2]) * T(0.5);
        g11 = (Gl[3] + Gr[3]) * T(0.5);
        const T dk = IO::kw(d, 2 * r) - IO::kw(d, 2 * l), dw = IO::kw(d, 2 * r + 1) - IO::kw(d, 2 * l + 1);
        g00 = g00 + ((dk) - (g00 * l0 + g01 * l1)) * l0 / L2;
        g01 = g01 + ((dk) - (g00 * l0 + g01 * l1)) * l1 / L2;
        g10 = g10 + ((dw) - (g10 * l0 + g11 * l1)) * l0 / L2;
        g11 = g11 + ((dw) - (g10 * l0 + g11 * l1)) * l1 / L2;
    } else {
        face_f1 = F1[l];
        g00 = G[4 * l];
        g01 = G[4 * l + 1];
        g10 = G[4 * l + 2];
        g11 = G[4 * l + 3];
    }
    const T sigma_k = face_f1 * T(sigma_k1) + (T(1) - face_f1) * T(sigma_k2);
    const T sigma_w = face_f1 * T(sigma_w1) + (T(1) - face_f1) * T(sigma_w2);
    const T faceMul = IO::mue(d, f), faceMut = IO::mutf(d, f);
    const T txx_k = (faceMul + sigma_k * faceMut) * g00;
    const T tyy_k = (faceMul + sigma_k * faceMut) * g01;
    const T txx_w = (faceMul + sigma_w * faceMut) * g10;
    const T tyy_w = (faceMul + sigma_w * faceMut) * g11;
    T fv0 = txx_k * nx + tyy_k * ny;
    T fv1 = txx_w * nx + tyy_w * ny;
    fv0 *= A;
    fv1 *= A;
    T* Fc = as<T>(d.sstFc);
    T* Fv = as<T>(d.sstFv);
    Fc[2 * f] = fc0;
    Fc[2 * f + 1] = fc1;
    Fv[2 * f] = fv0;
    Fv[2 * f + 1] = fv1;
}

// rans_P_Solver (:923-966), SolveTotalTFlux (:969-1013) and SolveDiag (:170-192).
// coupled = 0: the residual as written, Q vol + sum(Fc - Fv); coupled = 1 (the
// model inside every LU-SGS step): sum(Fc - Fv) - Q vol, the sign that
// dW = -R / D needs for the sources (the written sign turns production into
// destruction).
template <class T>
__global__ void k_sst_total(DevArrays d, int coupled) {
    typedef SstIo<T> IO;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.nc) return;
    const T f1 = as<T>(d.sstF1)[c];
    const T* G = as<T>(d.sstG) + 4 * c;
    T rdiv = T(0);
    rdiv += G[0] * G[2];
    rdiv += G[1] * G[3];
    const T Cw = f1 * T(Cw1) + (T(1.0) - f1) * T(Cw2);
    const T beta = f1 * T(beta1) + (T(1.0) - f1) * T(beta2);
    const T rho = IO::rho(d, c);
    const T k = IO::kw(d, 2 * c), w = IO::kw(d, 2 * c + 1), mut = IO::mut(d, c);
    const auto gu = IO::gradu(d, c);  // (du/dx, du/dy, dv/dx, dv/dy)
    const T ux = gu.x, uy = gu.y, vx = gu.z, vy = gu.w;
    const T ddls0 = T(2.0 / 3.0) * ((ux - vy) * (ux - vy));
    const T ddls1 = (uy + vx) * (uy + vx);
    const T ddls2 = T(2.0 / 3.0) * rho * k * (ux + vy);
    const T P = (ddls0 + ddls1) * mut - ddls2;
    const T q0 = P - T(beta_star) * rho * k * w;
    const T q1 = Cw * rho * P / mut - beta * rho * w * w + T(2) * (T(1) - f1) * rho * T(sigma_w2) / w * rdiv;
    const T vol = IO::cgeo(d, c).x;
    T r0 = coupled ? -(q0 * vol) : q0 * vol, r1 = coupled ? -(q1 * vol) : q1 * vol;
    const int4 cf = d.cface[c];
    const int codes[4] = {cf.x, cf.y, cf.z, cf.w};
    const T* Fc = as<T>(d.sstFc);
    const T* Fv = as<T>(d.sstFv);
    for (int s = 0; s < 4; s++) {
        const int code = codes[s];
        if (code == 0) continue;
        const int f = code > 0 ? code - 1 : -code - 1;
        const T e0 = Fc[2 * f] - Fv[2 * f], e1 = Fc[2 * f + 1] - Fv[2 * f + 1];
        if (code > 0) {
            r0 += e0;
            r1 += e1;
        } else {
            r0 -= e0;
            r1 -= e1;
        }
    }
    d.sstR[2 * c] = (double)r0;
    d.sstR[2 * c + 1] = (double)r1;
    const T OMEGAN = T(1.5);
    const T diag = vol / IO::dt(d, c) + T(0.5) * OMEGAN * IO::specc(d, c) + IO::specv(d, c);
    d.sstD[2 * c] = (double)(diag + T(2.0) * T(beta_star) * w * vol);  // omega, as the reference (:183)
    d.sstD[2 * c + 1] = (double)(diag + vol * IO::abs_(T(2.0) * beta * w + T(2.0) * T(sigma_w2) * (T(1) - f1) * rdiv / (w * w)));
}

// initializeConsData then UpdatePrimitiveVariables: W = rho (k, omega),
// (k, omega) = W / rho, mu_t = a1 W_k / max(a1 W_omega / rho, F2 |dv/dx - du/dy|).
// |dv/dx - du/dy| and F2 of cell c for the eddy-viscosity update, from the
// binary64 arrays or (MIXFF) the float-float ones the model's passes used.
__device__ __forceinline__ void model_curl_f2(const DevArrays& d, int c, double& curl, double& f2) {
    if (d.ffsst) {
        const q4 gu = ld4(d.gradq + 2 * (size_t)c + 1);
        curl = fabs((double)(gu.z - gu.y));
        f2 = (double)as<ff>(d.sstF2)[c];
    } else {
        const d4 gu = d.grad[2 * c + 1];
        curl = fabs(gu.z - gu.y);
        f2 = d.sstF2[c];
    }
}

__global__ void k_sst_mut(DevArrays d) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.nc) return;
    const double rho = d.U[c].x;
    const double W0 = d.sstT[2 * c] * rho, W1 = d.sstT[2 * c + 1] * rho;
    d.sstT[2 * c] = W0 / rho;
    d.sstT[2 * c + 1] = W1 / rho;
    double curl, f2;
    model_curl_f2(d, c, curl, f2);
    const double h = dmax(a1 * W1 / rho, f2 * curl);
    d.sstMut[c] = a1 * W0 / h;
}

// ---------------------------------------------------------------------------
// Coupled turbulence LU-SGS (CFD_FLOW_SST).  The reference's SSTkomegaModel
// would run LUSGSIntegrator over its two equations (turbModelTimeStrategy,
// ViscousFlow2D.cpp:62-63) with SolveDF (:251-474); as written that SolveDF
// reads the neighbour's k, omega pair past the cell's own, passes the current
// cell as the neighbour in its right-cell branch (a zero centre line) and
// reads flow arrays no caller sets.  These kernels run the intended step: for
// neighbour j across face f of cell i, with the flow's W_j (before the update)
// and its increment dW_j of the same sweep direction,
//   DF = 0.5 (+-(W_t,j + dW_t,j) Vn(W_j + dW_j) -+ W_t,j Vn(W_j) - r_A dW_t,j) A,
// r_A as the flow's (SolveViscousFlux with mu/Pr + mu_t/Prt of cell i),
// forward dW_t1,i = (-R_t,i - sum DF) / D_t,i, backward dW_t,i = dW_t1,i -
// sum DF / D_t,i, in the reference's cell order (same levels as the flow).
constexpr unsigned long long kSentT = 0x7ff4c0ffee5eed22ULL;  // signalling-NaN "not yet computed"
constexpr unsigned kSentTf = 0x7fa0c0dfu;
constexpr long long kSpinT = 1LL << 22;

__device__ __forceinline__ bool sent_t(double x) { return (unsigned long long)__double_as_longlong(x) == kSentT; }
__device__ __forceinline__ bool sent_tf(float x) { return __float_as_uint(x) == kSentTf; }

// Per (cell i, face slot s): the increment-free terms of the turbulence SolveDF
// - W_t,j Vn(W_j), r_A, and Vn(W_j + dW_j) with the flow increment of the
// direction that uses this slot (forward if j < i, backward if j > i) - then
// the "not yet computed" sentinels and 1/D_t.  After the flow's sweeps; or,
// `coupled`, before them: Vn(W_j + dW_j) then comes from the flow's sweep of
// the same launch (its sentinel is set here).
__global__ void __launch_bounds__(256) k_sst_sweep_prep(DevArrays d, int coupled) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 4 * d.nc) return;
    const int i = t >> 2, s = t & 3;
    if (s < 2) {
        d.sstDW1[2 * i + s] = __longlong_as_double((long long)kSentT);
        d.sstDW[2 * i + s] = __longlong_as_double((long long)kSentT);
        d.sstDinv[2 * i + s] = 1.0 / d.sstD[2 * i + s];
    }
    if (s == 0 && d.sstDW1f) {
        const float sf = __uint_as_float(kSentTf);
        d.sstDW1f[i] = make_float2(sf, sf);
        d.sstDWf[i] = make_float2(sf, sf);
    }
    const int code = (&d.cface[i].x)[s];
    double fc0 = 0.0, fc1 = 0.0, rA = 0.0, vnp = 0.0;
    if (code != 0) {
        const int f = code > 0 ? code - 1 : -code - 1;
        const int2 e = d.lr[f];
        const int j = code > 0 ? e.y : e.x;
        if (j >= 0) {
            const d4 g = d.fg0[f];
            const d4 w0 = ld4(d.W + j);
            const double vn0 = dot2(w0.z / w0.x, w0.w / w0.x, g.x, g.y);
            if (coupled) {
                vnp = __longlong_as_double((long long)kSentT);
            } else {
                // as the flow's binary64 sweep forms Vn on this face
                const d4 dw = ld4((j < i ? d.dW1 : d.dW) + j);
                const d4 wp = d4{w0.x + dw.x, w0.y + dw.y, w0.z + dw.z, w0.w + dw.w};
                vnp = dot2(wp.z / wp.x, wp.w / wp.x, g.x, g.y);
            }
            fc0 = d.sstW[2 * j] * vn0;
            fc1 = d.sstW[2 * j + 1] * vn0;
            const d4 uj = ld4(d.U + j);
            const double G = 1.4;
            const double vn = dot2(uj.z, uj.w, g.x, g.y);
            const double c = sqrt(G * uj.y / uj.x);
            rA = 1.5 * (fabs(vn) + c);
            rA += dmax(4 / (3 * uj.x), G / uj.x) * (d.mu[i] / 0.72 + d.sstMut[i] / 0.9) / sqrt(d.fvis[f].z);
        }
    }
    d.sstFcs[2 * t] = fc0;
    d.sstFcs[2 * t + 1] = fc1;
    d.sstRA[t] = rA;
    d.sstVnp[t] = vnp;
}

// The fast forms' prep: the same per-slot terms formed in binary32 from the
// binary32 copies of the flow's state and increments (Wf, dW1f / dWf, as the
// flow's binary32 sweep polls them), packed per slot for the binary32 sweep,
// with a binary32 copy of W_t; the sentinels and 1/D as above.  Only the
// sweep operator is rounded differently: the update and the residual that
// fix the converged state stay as they are.
__global__ void __launch_bounds__(256) k_sst_sweep_prep32(DevArrays d, int coupled) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 4 * d.nc) return;
    const int i = t >> 2, s = t & 3;
    if (s < 2) {
        d.sstDW1[2 * i + s] = __longlong_as_double((long long)kSentT);
        d.sstDW[2 * i + s] = __longlong_as_double((long long)kSentT);
        d.sstDinv[2 * i + s] = 1.0 / d.sstD[2 * i + s];
    }
    if (s == 0) {
        const float sf = __uint_as_float(kSentTf);
        d.sstDW1f[i] = make_float2(sf, sf);
        d.sstDWf[i] = make_float2(sf, sf);
        d.sstWf[i] = make_float2((float)d.sstW[2 * i], (float)d.sstW[2 * i + 1]);
    }
    const int code = (&d.cface[i].x)[s];
    float rA = 0.f, vnp = 0.f, dvn = 0.f, A = 0.f;
    if (code != 0) {
        const int f = code > 0 ? code - 1 : -code - 1;
        const int2 e = d.lr[f];
        const int j = code > 0 ? e.y : e.x;
        if (j >= 0) {
            const float4 g = d.fg0f[f];
            A = g.z;
            if (coupled) {
                vnp = dvn = __uint_as_float(kSentTf);
            } else {
                // Vn(W_j + dW_j) and its change as the flow's binary32 sweep forms them (base velocity
                // plus the exact difference)
                const float4 w0 = d.Wf[j];
                const float u = w0.z / w0.x, v = w0.w / w0.x;
                const float vn0 = u * g.x + v * g.y;
                const float4 dw = (j < i ? d.dW1f : d.dWf)[j];
                const float rp = 1.f / (w0.x + dw.x);
                const float du = (dw.z - u * dw.x) * rp, dv = (dw.w - v * dw.x) * rp;
                dvn = du * g.x + dv * g.y;
                vnp = vn0 + dvn;
            }
            const d4 ud = ld4(d.U + j);
            const float rho = (float)ud.x, p = (float)ud.y;
            const float vn = (float)ud.z * g.x + (float)ud.w * g.y;
            rA = 1.5f * (fabsf(vn) + sqrtf(1.4f * p / rho));
            const float mui = d.ffsst ? d.muq[i].hi : (float)d.mu[i];
            rA += fmaxf(4.f / (3.f * rho), 1.4f / rho) * (mui / 0.72f + (float)d.sstMut[i] / 0.9f) /
                  sqrtf(d.fvisf[f].z);
        }
    }
    d.sstSlotf[t] = make_float4(0.f, 0.f, rA, A);
    d.sstVnpf[t] = make_float2(vnp, dvn);
}

// One dataflow launch per direction: one warp per cell, taken in level order
// (positions p = block + B*q, as the flow's dataflow sweep), lanes 2s+m for
// face slot s and equation m.  A neighbour's increment is final once its
// words are no longer the sentinel; every wait is bounded (ERR_TIMEOUT).
// T = double: the plain form (every operation in binary64, as the C
// restatement); T = float: the slot terms in binary32 and the published copy
// polled in binary32, the increment itself formed in binary64 from them.
// CPL: the flow's sweep runs in the same grid and writes Vn(W_j + dW_j) per
// slot as it goes; the slot's value is then awaited like an increment.  bid, B:
// this block's number among the B blocks that run the turbulence sweep.
template <bool FWD, class T, bool PF, bool CPL>
__device__ __forceinline__ void sst_sweep_body(const DevArrays& d, const int* __restrict__ order, int bid, int B) {
    const int lane = threadIdx.x & 31;
    const int s = (lane >> 1) & 3, m = lane & 1;
    const int warp = threadIdx.x >> 5;
    const int NW = blockDim.x >> 5;
    double* dst = FWD ? d.sstDW1 : d.sstDW;
    float2* dstf = FWD ? d.sstDW1f : d.sstDWf;
    const int q0 = ((warp - (int)(bid % NW)) % NW + NW) % NW;
    // PF: the inputs of a position that do not depend on a neighbour's
    // increment (its cell, face slot, neighbour and the per-slot constants) are
    // loaded one position ahead, while the warp waits for the current
    // position's neighbour: their chain of dependent loads (order, cell faces,
    // face cells, then the neighbour's records) stays off the sweep's critical
    // path, for more registers per thread.
    struct In {
        int i, j;
        int4 cf;
        bool use, left;
        T wt, fc, rA, vnp, A;
        float dvn;  // binary32 form: the exact change of Vn, so the flux change needs no cancelling difference
        double own, dd;
        float ownf, ddf;
    };
    auto load = [&](long long p, In& x) {
        x.i = order[p];
        x.cf = d.cface[x.i];
        const int code = lane < 8 ? (s == 0 ? x.cf.x : s == 1 ? x.cf.y : s == 2 ? x.cf.z : x.cf.w) : 0;
        x.use = false;
        x.left = false;
        x.j = 0;
        int f = 0;
        if (code != 0) {
            f = code > 0 ? code - 1 : -code - 1;
            x.left = code > 0;
            const int2 e = d.lr[f];
            x.j = x.left ? e.y : e.x;
            x.use = FWD ? (x.j >= 0 && x.j < x.i) : (x.j > x.i);
        }
        x.own = 0.0;
        x.dd = 1.0;
        if (lane < 2) {
            x.own = FWD ? d.sstR[2 * x.i + m] : d.sstDW1[2 * x.i + m];
            x.dd = std::is_same<T, double>::value ? d.sstD[2 * x.i + m] : d.sstDinv[2 * x.i + m];
        }
        x.ownf = (float)x.own;
        x.ddf = (float)x.dd;
        x.wt = x.fc = x.rA = x.vnp = x.A = T(0);
        x.dvn = 0.f;
        if (x.use) {
            const size_t t = (size_t)x.i * 4 + s;
            if constexpr (std::is_same<T, double>::value) {
                x.wt = d.sstW[2 * x.j + m];
                x.fc = d.sstFcs[2 * t + m];
                x.rA = d.sstRA[t];
                if (!CPL) x.vnp = d.sstVnp[t];
                x.A = d.fgeo[f].z;
            } else {
                const float4 sl = d.sstSlotf[t];
                const float2 wt = d.sstWf[x.j];
                x.wt = m ? wt.y : wt.x;
                x.rA = sl.z;
                if (!CPL) {
                    const float2 vv = d.sstVnpf[t];
                    x.vnp = vv.x;
                    x.dvn = vv.y;
                }
                x.A = sl.w;
            }
        }
    };
    long long p = (long long)bid + (long long)B * q0;
    if (p >= d.nc) return;
    In cur, nxt;
    load(p, cur);
    for (;;) {
        const long long pn = p + (long long)B * NW;
        const bool more = pn < d.nc;
        if (PF && more) load(pn, nxt);
        T DF = T(0);
        if (cur.use) {
            long long it = 0;
            T dt;
            if (CPL) {  // the flow's Vn(W_j + dW_j) of this slot, written once by the flow's sweep
                const size_t t = (size_t)cur.i * 4 + s;
                if constexpr (std::is_same<T, double>::value) {
                    double v;
                    while (true) {
                        v = __ldcv(d.sstVnp + t);
                        if (!sent_t(v)) break;
                        if (++it > kSpinT) { atomicOr(d.err, ERR_TIMEOUT); break; }
                        if (d.poll_ns > 0) __nanosleep(d.poll_ns);
                    }
                    cur.vnp = v;
                } else {
                    float2 v;
                    while (true) {
                        v = __ldcv(d.sstVnpf + t);
                        if (!sent_tf(v.x) && !sent_tf(v.y)) break;
                        if (++it > kSpinT) { atomicOr(d.err, ERR_TIMEOUT); break; }
                        if (d.poll_ns > 0) __nanosleep(d.poll_ns);
                    }
                    cur.vnp = v.x;
                    cur.dvn = v.y;
                }
                it = 0;
            }
            if (std::is_same<T, double>::value) {
                const double2* qd = reinterpret_cast<const double2*>((FWD ? d.sstDW1 : d.sstDW) + 2 * (size_t)cur.j);
                double2 a;
                while (true) {
                    a = __ldcv(qd);
                    if (!sent_t(a.x) && !sent_t(a.y)) break;
                    if (++it > kSpinT) { atomicOr(d.err, ERR_TIMEOUT); break; }
                    if (d.poll_ns > 0) __nanosleep(d.poll_ns);
                }
                dt = (T)(m ? a.y : a.x);
            } else {
                const float2* qf = (FWD ? d.sstDW1f : d.sstDWf) + cur.j;
                float2 a;
                while (true) {
                    a = __ldcv(qf);
                    if (!sent_tf(a.x) && !sent_tf(a.y)) break;
                    if (++it > kSpinT) { atomicOr(d.err, ERR_TIMEOUT); break; }
                    if (d.poll_ns > 0) __nanosleep(d.poll_ns);
                }
                dt = (T)(m ? a.y : a.x);
            }
            T dfc;
            if constexpr (std::is_same<T, double>::value) {
                const T fcp = (cur.wt + dt) * cur.vnp;
                dfc = cur.left ? (fcp - cur.fc) : (cur.fc - fcp);
            } else {
                // (W_t + dW_t) Vn' - W_t Vn = W_t dVn + dW_t Vn': no difference of nearly equal products
                const T ch = cur.wt * cur.dvn + dt * cur.vnp;
                dfc = cur.left ? ch : -ch;
            }
            DF = T(0.5) * (dfc - cur.rA * dt) * cur.A;
        }
        __syncwarp();
        // ordered sum over the face slots (lanes m, 2+m, 4+m, 6+m)
        const T v0 = __shfl_sync(0xffffffffu, DF, m);
        const T v1 = __shfl_sync(0xffffffffu, DF, 2 + m);
        const T v2 = __shfl_sync(0xffffffffu, DF, 4 + m);
        const T v3 = __shfl_sync(0xffffffffu, DF, 6 + m);
        T dF = T(0);
        if (cur.cf.x != 0) dF += v0;
        if (cur.cf.y != 0) dF += v1;
        if (cur.cf.z != 0) dF += v2;
        if (cur.cf.w != 0) dF += v3;
        if (std::is_same<T, double>::value) {
            double res = 0.0;
            if (lane < 2) res = FWD ? (-cur.own - (double)dF) / cur.dd : cur.own - (double)dF / cur.dd;
            const double r1 = __shfl_sync(0xffffffffu, res, 1);
            if (lane == 0) __stcg(reinterpret_cast<double2*>(dst + 2 * (size_t)cur.i), make_double2(res, r1));
        } else {
            // the binary32 copy the next levels wait for first, then the binary64 increment
            float resf = 0.f;
            if (lane < 2)
                resf = FWD ? (-cur.ownf - (float)dF) * cur.ddf : cur.ownf - (float)dF * cur.ddf;
            const float f1 = __shfl_sync(0xffffffffu, resf, 1);
            if (lane == 0) __stcg(dstf + cur.i, make_float2(resf, f1));
            double res = 0.0;
            if (lane < 2) res = FWD ? (-cur.own - (double)dF) * cur.dd : cur.own - (double)dF * cur.dd;
            const double r1 = __shfl_sync(0xffffffffu, res, 1);
            if (lane == 0) __stcg(reinterpret_cast<double2*>(dst + 2 * (size_t)cur.i), make_double2(res, r1));
        }
        if (!more) break;
        if (!PF) load(pn, nxt);
        cur = nxt;
        p = pn;
    }
}

template <bool FWD, class T, bool PF>
__global__ void __launch_bounds__(256) k_sst_sweep(DevArrays d, const int* __restrict__ order) {
    sst_sweep_body<FWD, T, PF, false>(d, order, blockIdx.x, gridDim.x);
}

// The flow's and the turbulence equations' sweeps of one direction in one
// cooperative grid: blocks [0, nflow) run the flow's round-robin sweep (F32:
// its binary32 form) and hand each slot's Vn(W_j + dW_j) to the turbulence
// sweep on the other blocks, which no longer waits for the whole flow sweep.
// Each part only depends on its own and the flow's earlier positions, and
// every block is resident, so both always progress; every wait is bounded.
template <bool FWD, bool F32, bool PF>
__global__ void __launch_bounds__(256) k_sweep_coupled(DevArrays d, int nflow) {
    if ((int)blockIdx.x < nflow) {
        if constexpr (F32) {
            sweep_flow32_body<FWD, false, PF>(blockIdx.x, nflow, FWD ? d.npos2_fwd : d.npos2_bwd,
                                              FWD ? d.fwd_order2 : d.bwd_order2, d.cface, d.lr, d.fg0f, d.Wf, d.swraf,
                                              d.R, d.invD, d.dW1, d.dW, d.dW1f, d.dWf, d.err, d.poll_ns, d.sstVnpf);
        } else {
            sweep_flow_body<FWD, PF>(blockIdx.x, nflow, d.nc, FWD ? d.fwd_order : d.bwd_order, d.cface, d.lr, d.fg0,
                                     d.W, d.swfc, d.swra, d.R, d.diag, d.invD, d.dW1, d.dW, d.err, d.poll_ns, d.sstVnp);
        }
    } else {
        sst_sweep_body<FWD, typename std::conditional<F32, float, double>::type, PF, true>(
            d, FWD ? d.fwd_order : d.bwd_order, blockIdx.x - nflow, gridDim.x - nflow);
    }
}

// W_t += dW_t; k, omega = W_t / rho with rho after the flow's update, kept at
// or above 1e-4 of the freestream values (the clip that SSTKWStrategy.h:206-215
// has commented out); mu_t = a1 W_k / max(a1 W_omega / rho, F2 |dv/dx - du/dy|)
// (UpdatePrimitiveVariables, :194-223).
__global__ void k_sst_update(DevArrays d) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.nc) return;
    const MeshPrm& P = d.prm[d.cmesh[c]];
    const double kmin = 1e-4 * P.sst_k, wmin = 1e-4 * P.sst_w;
    const double rho = d.U[c].x;
    double w0 = d.sstW[2 * c] + d.sstDW[2 * c], w1 = d.sstW[2 * c + 1] + d.sstDW[2 * c + 1];
    double k = w0 / rho, w = w1 / rho;
    if (!(k >= kmin)) { k = kmin; w0 = rho * kmin; }
    if (!(w >= wmin)) { w = wmin; w1 = rho * wmin; }
    d.sstW[2 * c] = w0;
    d.sstW[2 * c + 1] = w1;
    d.sstT[2 * c] = k;
    d.sstT[2 * c + 1] = w;
    double curl, f2;
    model_curl_f2(d, c, curl, f2);
    const double h = dmax(a1 * w1 / rho, f2 * curl);
    d.sstMut[c] = a1 * w0 / h;
}

// initializeConsData (:97-109): W_t = rho (k, omega)
__global__ void k_sst_cons(DevArrays d) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.nc) return;
    const double rho = d.U[c].x;
    d.sstW[2 * c] = d.sstT[2 * c] * rho;
    d.sstW[2 * c + 1] = d.sstT[2 * c + 1] * rho;
}

inline unsigned nb(int n, int bs) { return (unsigned)((n + bs - 1) / bs); }

}  // namespace

void launch_sst_residual(const DevArrays& d, const LaunchCfg& L) {
    k_sst_face<double><<<nb(d.nf, 256), 256, 0, L.stream>>>(d);
    k_sst_cell<double><<<nb(d.nc, 256), 256, 0, L.stream>>>(d);
    k_sst_flux<double><<<nb(d.nf, 256), 256, 0, L.stream>>>(d);
    k_sst_total<double><<<nb(d.nc, 256), 256, 0, L.stream>>>(d, 0);
    *L.counter += 4;
}

void launch_sst_stage(const DevArrays& d, const LaunchCfg& L, int stage) {
    if (d.ffsst) {  // MIXFF: the model in float-float on its copies of k, omega, mu_t and the wall distance
        if (stage == 0) {
            k_sst_to_ff<<<nb(d.nc, 256), 256, 0, L.stream>>>(d);
            *L.counter += 1;
        }
        if (stage == 0) k_sst_face<ff><<<nb(d.nf, 256), 256, 0, L.stream>>>(d);
        else if (stage == 1) k_sst_cell<ff><<<nb(d.nc, 256), 256, 0, L.stream>>>(d);
        else if (stage == 2) k_sst_flux<ff><<<nb(d.nf, 256), 256, 0, L.stream>>>(d);
        else k_sst_total<ff><<<nb(d.nc, 256), 256, 0, L.stream>>>(d, 1);
    } else {
        if (stage == 0) k_sst_face<double><<<nb(d.nf, 256), 256, 0, L.stream>>>(d);
        else if (stage == 1) k_sst_cell<double><<<nb(d.nc, 256), 256, 0, L.stream>>>(d);
        else if (stage == 2) k_sst_flux<double><<<nb(d.nf, 256), 256, 0, L.stream>>>(d);
        else k_sst_total<double><<<nb(d.nc, 256), 256, 0, L.stream>>>(d, 1);
    }
    *L.counter += 1;
}

void launch_sst_update_mut(const DevArrays& d, const LaunchCfg& L) {
    k_sst_mut<<<nb(d.nc, 256), 256, 0, L.stream>>>(d);
    *L.counter += 1;
}

}  // namespace cfdgb

namespace cfdgb {

int sst_sweep_max_grid(int blocks_per_sm, int threads, bool pf) {
    int dev = 0, sms = 0, a = 0, b = 0, c2 = 0, d2 = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &a, pf ? (void*)k_sst_sweep<true, double, true> : (void*)k_sst_sweep<true, double, false>, threads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &b, pf ? (void*)k_sst_sweep<false, double, true> : (void*)k_sst_sweep<false, double, false>, threads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &c2, pf ? (void*)k_sst_sweep<true, float, true> : (void*)k_sst_sweep<true, float, false>, threads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &d2, pf ? (void*)k_sst_sweep<false, float, true> : (void*)k_sst_sweep<false, float, false>, threads, 0);
    int per = a < b ? a : b;
    per = per < c2 ? per : c2;
    per = per < d2 ? per : d2;
    if (blocks_per_sm > 0 && blocks_per_sm < per) per = blocks_per_sm;
    return per * sms;
}

void launch_sst_sweep_prep(const DevArrays& d, const LaunchCfg& L, bool fp32, bool coupled) {
    const int cp = coupled ? 1 : 0;
    if (fp32)
        k_sst_sweep_prep32<<<nb(4 * d.nc, 256), 256, 0, L.stream>>>(d, cp);
    else
        k_sst_sweep_prep<<<nb(4 * d.nc, 256), 256, 0, L.stream>>>(d, cp);
    *L.counter += 1;
}

int sweep_coupled_max_grid(bool fp32, int blocks_per_sm, int threads, bool pf) {
    int dev = 0, sms = 0, a = 0, b = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    void* f1 = fp32 ? (pf ? (void*)k_sweep_coupled<true, true, true> : (void*)k_sweep_coupled<true, true, false>)
                    : (pf ? (void*)k_sweep_coupled<true, false, true> : (void*)k_sweep_coupled<true, false, false>);
    void* f2 = fp32 ? (pf ? (void*)k_sweep_coupled<false, true, true> : (void*)k_sweep_coupled<false, true, false>)
                    : (pf ? (void*)k_sweep_coupled<false, false, true> : (void*)k_sweep_coupled<false, false, false>);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, f1, threads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, f2, threads, 0);
    int per = a < b ? a : b;
    if (blocks_per_sm > 0 && blocks_per_sm < per) per = blocks_per_sm;
    return per * sms;
}

cudaError_t launch_sweep_coupled(const DevArrays& d, const LaunchCfg& L, bool forward, bool fp32, int grid,
                                 int nflow) {
    void* args[] = {(void*)&d, (void*)&nflow};
    void* fn;
    if (fp32)
        fn = d.flow_pf ? (forward ? (void*)k_sweep_coupled<true, true, true> : (void*)k_sweep_coupled<false, true, true>)
                       : (forward ? (void*)k_sweep_coupled<true, true, false> : (void*)k_sweep_coupled<false, true, false>);
    else
        fn = d.flow_pf ? (forward ? (void*)k_sweep_coupled<true, false, true> : (void*)k_sweep_coupled<false, false, true>)
                       : (forward ? (void*)k_sweep_coupled<true, false, false> : (void*)k_sweep_coupled<false, false, false>);
    cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(d.flow_threads), args, 0, L.stream);
    *L.counter += 1;
    return e;
}

cudaError_t launch_sst_sweeps(const DevArrays& d, const LaunchCfg& L, bool fp32) {
    if (fp32)
        k_sst_sweep_prep32<<<nb(4 * d.nc, 256), 256, 0, L.stream>>>(d, 0);
    else
        k_sst_sweep_prep<<<nb(4 * d.nc, 256), 256, 0, L.stream>>>(d, 0);
    *L.counter += 1;
    for (int dir = 0; dir < 2; dir++) {
        const int* order = dir == 0 ? d.fwd_order : d.bwd_order;
        void* args[] = {(void*)&d, (void*)&order};
        void* fn;
        if (d.flow_pf)
            fn = fp32 ? (dir == 0 ? (void*)k_sst_sweep<true, float, true> : (void*)k_sst_sweep<false, float, true>)
                      : (dir == 0 ? (void*)k_sst_sweep<true, double, true> : (void*)k_sst_sweep<false, double, true>);
        else
            fn = fp32 ? (dir == 0 ? (void*)k_sst_sweep<true, float, false> : (void*)k_sst_sweep<false, float, false>)
                      : (dir == 0 ? (void*)k_sst_sweep<true, double, false> : (void*)k_sst_sweep<false, double, false>);
        cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(d.sst_grid), dim3(d.flow_threads), args, 0, L.stream);
        *L.counter += 1;
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

void launch_sst_update(const DevArrays& d, const LaunchCfg& L) {
    k_sst_update<<<nb(d.nc, 256), 256, 0, L.stream>>>(d);
    *L.counter += 1;
}

void launch_sst_cons(const DevArrays& d, const LaunchCfg& L) {
    k_sst_cons<<<nb(d.nc, 256), 256, 0, L.stream>>>(d);
    *L.counter += 1;
}

}  // namespace cfdgb
