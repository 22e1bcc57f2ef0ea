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

#include "case.hpp"

namespace cfdgb {
namespace {

// SSTkomegaModel constants (SSTKWStrategy.h:14-30)
constexpr double beta1 = 0.075, beta2 = 0.0828, sigma_k1 = 0.85, sigma_k2 = 1.0, sigma_w1 = 0.5,
                 sigma_w2 = 0.856, Cw1 = 0.533, Cw2 = 0.440, a1 = 0.31, beta_star = 0.09;

__device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }  // std::max
__device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }  // std::min

// ComputeFaceTValue (:615-659) and the face loop of
// ComputeTurbulenceViscousCoefficient (:749-777).
__global__ void k_sst_face(DevArrays d) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= d.nf) return;
    const int2 lr = d.lr[f];
    const d4 g = d.fgeo[f];
    const MeshPrm& P = d.prm[d.fmesh[f]];
    const int l = lr.x, r = lr.y;
    double t0, t1, mf;
    if (r >= 0) {
        t0 = 0.5 * (d.sstT[2 * l] + d.sstT[2 * r]);
        t1 = 0.5 * (d.sstT[2 * l + 1] + d.sstT[2 * r + 1]);
        mf = 0.5 * (d.sstMut[l] + d.sstMut[r]);
    } else if (r == BC_WALL) {
        const double dis = d.walld[l];
        t0 = 0.0;
        t1 = 10.0 * 6.0 * d.mue[f] / (d.Ue[f].x * beta1 * dis * dis);
        mf = 0.0;
    } else {
        const d4 ue = d.Ue[f];
        double vn = 0;
        vn += ue.z * g.x;
        vn += ue.w * g.y;
        if (vn > 0.0) {
            t0 = d.sstT[2 * l];
            t1 = d.sstT[2 * l + 1];
        } else {
            t0 = P.sst_k;
            t1 = P.sst_w;
        }
        mf = vn > 0.0 ? d.sstMut[l] : P.sst_mut;
    }
    d.sstTf[2 * f] = t0;
    d.sstTf[2 * f + 1] = t1;
    d.sstMutf[f] = mf;
}

// ComputeCellTGradient (:662-692) and ComputeSSTf1f2 (:695-722).
__global__ void k_sst_cell(DevArrays d) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.nc) return;
    const int4 cf = d.cface[c];
    const int codes[4] = {cf.x, cf.y, cf.z, cf.w};
    double gk0 = 0, gk1 = 0, gw0 = 0, gw1 = 0;
    for (int s = 0; s < 4; s++) {
        const int code = codes[s];
        if (code == 0) continue;
        const int f = code > 0 ? code - 1 : -code - 1;
        const d4 g = d.fgeo[f];
        const double ak = g.z * d.sstTf[2 * f], aw = g.z * d.sstTf[2 * f + 1];
        const double vk0 = g.x * ak, vk1 = g.y * ak, vw0 = g.x * aw, vw1 = g.y * aw;
        if (code > 0) {
            gk0 = gk0 + vk0; gk1 = gk1 + vk1; gw0 = gw0 + vw0; gw1 = gw1 + vw1;
        } else {
            gk0 = gk0 - vk0; gk1 = gk1 - vk1; gw0 = gw0 - vw0; gw1 = gw1 - vw1;
        }
    }
    const double vol = d.cgeo[c].x;
    gk0 = gk0 / vol; gk1 = gk1 / vol; gw0 = gw0 / vol; gw1 = gw1 / vol;
    d.sstG[4 * c] = gk0; d.sstG[4 * c + 1] = gk1; d.sstG[4 * c + 2] = gw0; d.sstG[4 * c + 3] = gw1;
    double gradVal = 0;
    gradVal += gk0 * gw0;
    gradVal += gk1 * gw1;
    const double rho = d.U[c].x, dis = d.walld[c], K = d.sstT[2 * c], w = d.sstT[2 * c + 1], muL = d.mu[c];
    const double CD_kw = dmax(2.0 * rho * sigma_w2 / w * gradVal, 1.0e-20);
    double arg1 = dmax(sqrt(K) / (0.09 * w * dis), 500.0 * muL / (rho * w * dis * dis));
    arg1 = dmin(arg1, 4.0 * rho * sigma_w2 * K / (CD_kw * dis * dis));
    const double arg2 = dmax(2.0 * sqrt(K) / (0.09 * w * dis), 500.0 * muL / (rho * w * dis * dis));
    d.sstF1[c] = tanh(arg1 * arg1 * arg1 * arg1);
    d.sstF2[c] = tanh(arg2 * arg2);
}

// SolveConvectiveTFlux (:783-831) and SolveViscousTFlux (:834-920).  The
// interior face gradient is corrected along the centre line one component
// after the other, the y component using the already corrected x component,
// as the reference does.
__global__ void k_sst_flux(DevArrays d) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= d.nf) return;
    const int2 lr = d.lr[f];
    const int l = lr.x, r = lr.y;
    const d4 g = d.fgeo[f];
    const double nx = g.x, ny = g.y, A = g.z;
    const d4 ue = d.Ue[f];
    double vn = 0;
    vn += ue.z * nx;
    vn += ue.w * ny;
    double fc0, fc1;
    if (r >= 0) {
        const double vp = 0.5 * (vn + fabs(vn)), vs = 0.5 * (vn - fabs(vn));
        const double rl = d.U[l].x, rr = d.U[r].x;
        fc0 = d.sstT[2 * l] * rl * vp * A + d.sstT[2 * r] * rr * vs * A;
        fc1 = d.sstT[2 * l + 1] * rl * vp * A + d.sstT[2 * r + 1] * rr * vs * A;
    } else {
        fc0 = vn * ue.x * d.sstTf[2 * f] * A;
        fc1 = vn * ue.x * d.sstTf[2 * f + 1] * A;
    }
    double face_f1, g00, g01, g10, g11;
    if (r >= 0) {
        const double l0 = d.cgeo[r].y - d.cgeo[l].y, l1 = d.cgeo[r].z - d.cgeo[l].z;
        double L2 = 0;
        L2 += l0 * l0;
        L2 += l1 * l1;
        face_f1 = 0.5 * (d.sstF1[l] + d.sstF1[r]);
        const double* Gl = d.sstG + 4 * l;
        const double* Gr = d.sstG + 4 * r;
        g00 = (Gl[0] + Gr[0]) * 0.5;
        g01 = (Gl[1] + Gr[1]) * 0.5;
        g10 = (Gl[2] + Gr[2]) * 0.5;
        g11 = (Gl[3] + Gr[3]) * 0.5;
        const double dk = d.sstT[2 * r] - d.sstT[2 * l], dw = d.sstT[2 * r + 1] - d.sstT[2 * l + 1];
        g00 = g00 + ((dk) - (g00 * l0 + g01 * l1)) * l0 / L2;
        g01 = g01 + ((dk) - (g00 * l0 + g01 * l1)) * l1 / L2;
        g10 = g10 + ((dw) - (g10 * l0 + g11 * l1)) * l0 / L2;
        g11 = g11 + ((dw) - (g10 * l0 + g11 * l1)) * l1 / L2;
    } else {
        face_f1 = d.sstF1[l];
        g00 = d.sstG[4 * l];
        g01 = d.sstG[4 * l + 1];
        g10 = d.sstG[4 * l + 2];
        g11 = d.sstG[4 * l + 3];
    }
    const double sigma_k = face_f1 * sigma_k1 + (1 - face_f1) * sigma_k2;
    const double sigma_w = face_f1 * sigma_w1 + (1 - face_f1) * sigma_w2;
    const double faceMul = d.mue[f], faceMut = d.sstMutf[f];
    const double txx_k = (faceMul + sigma_k * faceMut) * g00;
    const double tyy_k = (faceMul + sigma_k * faceMut) * g01;
    const double txx_w = (faceMul + sigma_w * faceMut) * g10;
    const double tyy_w = (faceMul + sigma_w * faceMut) * g11;
    double fv0 = txx_k * nx + tyy_k * ny;
    double fv1 = txx_w * nx + tyy_w * ny;
    fv0 *= A;
    fv1 *= A;
    d.sstFc[2 * f] = fc0;
    d.sstFc[2 * f + 1] = fc1;
    d.sstFv[2 * f] = fv0;
    d.sstFv[2 * f + 1] = fv1;
}

// rans_P_Solver (:923-966), SolveTotalTFlux (:969-1013) and SolveDiag (:170-192).
__global__ void k_sst_total(DevArrays d) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.nc) return;
    const double f1 = d.sstF1[c];
    const double* G = d.sstG + 4 * c;
    double rdiv = 0;
    rdiv += G[0] * G[2];
    rdiv += G[1] * G[3];
    const double Cw = f1 * Cw1 + (1.0 - f1) * Cw2;
    const double beta = f1 * beta1 + (1.0 - f1) * beta2;
    const double rho = d.U[c].x;
    const double k = d.sstT[2 * c], w = d.sstT[2 * c + 1], mut = d.sstMut[c];
    const d4 gu = d.grad[2 * c + 1];  // (du/dx, du/dy, dv/dx, dv/dy)
    const double ux = gu.x, uy = gu.y, vx = gu.z, vy = gu.w;
    const double ddls0 = 2.0 / 3.0 * ((ux - vy) * (ux - vy));
    const double ddls1 = (uy + vx) * (uy + vx);
    const double ddls2 = 2.0 / 3.0 * rho * k * (ux + vy);
    const double P = (ddls0 + ddls1) * mut - ddls2;
    const double q0 = P - beta_star * rho * k * w;
    const double q1 = Cw * rho * P / mut - beta * rho * w * w + 2 * (1 - f1) * rho * sigma_w2 / w * rdiv;
    const double vol = d.cgeo[c].x;
    double r0 = q0 * vol, r1 = q1 * vol;
    const int4 cf = d.cface[c];
    const int codes[4] = {cf.x, cf.y, cf.z, cf.w};
    for (int s = 0; s < 4; s++) {
        const int code = codes[s];
        if (code == 0) continue;
        const int f = code > 0 ? code - 1 : -code - 1;
        const double e0 = d.sstFc[2 * f] - d.sstFv[2 * f], e1 = d.sstFc[2 * f + 1] - d.sstFv[2 * f + 1];
        if (code > 0) {
            r0 += e0;
            r1 += e1;
        } else {
            r0 -= e0;
            r1 -= e1;
        }
    }
    d.sstR[2 * c] = r0;
    d.sstR[2 * c + 1] = r1;
    const double OMEGAN = 1.5;
    const double diag = vol / d.dt[c] + 0.5 * OMEGAN * d.specc[c] + d.specv[c];
    d.sstD[2 * c] = diag + 2.0 * beta_star * w * vol;  // omega, as the reference (:183)
    d.sstD[2 * c + 1] = diag + vol * fabs(2.0 * beta * w + 2.0 * sigma_w2 * (1 - f1) * rdiv / (w * w));
}

// initializeConsData then UpdatePrimitiveVariables: W = rho (k, omega),
// (k, omega) = W / rho, mu_t = a1 W_k / max(a1 W_omega / rho, F2 |dv/dx - du/dy|).
__global__ void k_sst_mut(DevArrays d) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.nc) return;
    const double rho = d.U[c].x;
    const double W0 = d.sstT[2 * c] * rho, W1 = d.sstT[2 * c + 1] * rho;
    d.sstT[2 * c] = W0 / rho;
    d.sstT[2 * c + 1] = W1 / rho;
    const d4 gu = d.grad[2 * c + 1];
    const double curl = fabs(gu.z - gu.y);
    const double h = dmax(a1 * W1 / rho, d.sstF2[c] * curl);
    d.sstMut[c] = a1 * W0 / h;
}

inline unsigned nb(int n, int bs) { return (unsigned)((n + bs - 1) / bs); }

}  // namespace

void launch_sst_residual(const DevArrays& d, const LaunchCfg& L) {
    k_sst_face<<<nb(d.nf, 256), 256, 0, L.stream>>>(d);
    k_sst_cell<<<nb(d.nc, 256), 256, 0, L.stream>>>(d);
    k_sst_flux<<<nb(d.nf, 256), 256, 0, L.stream>>>(d);
    k_sst_total<<<nb(d.nc, 256), 256, 0, L.stream>>>(d);
    *L.counter += 4;
}

void launch_sst_update_mut(const DevArrays& d, const LaunchCfg& L) {
    k_sst_mut<<<nb(d.nc, 256), 256, 0, L.stream>>>(d);
    *L.counter += 1;
}

}  // namespace cfdgb
