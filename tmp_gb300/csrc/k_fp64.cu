// Binary64 kernels: geometry, the plain-form residual, RK/LU-SGS updates and the
// level-scheduled LU-SGS sweeps.  This translation unit is compiled with
// -fmad=false so that every a*b+c rounds twice, as in the reference's
// compiled code; together with the reference's operation order that makes the
// plain form reproduce the reference bit for bit (pow() aside).
#include "case.hpp"
#include "fv_kernels.cuh"
#include "sweep_flow.cuh"

namespace cfdgb {

static inline int nblk(int n, int bs) { return (n + bs - 1) / bs; }


// ---------------------------------------------------------------------------
// Geometry.  edge3d::find_area/find_normal/find_center (toolBox/edge3d_int.h:93-230)
__global__ void k_geom_faces(int nf, const int2* __restrict__ en, const d2* __restrict__ xy, d4* __restrict__ fgeo,
                             d2* __restrict__ fcen) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    int2 e = en[f];
    d2 p0 = xy[e.x], p1 = xy[e.y];
    double dx = p1.x - p0.x, dy = p1.y - p0.y;
    double l2 = 0;
    l2 += (dx * dx);
    l2 += (dy * dy);
    double A = sqrt(l2);
    fgeo[f] = d4{dy / A, -dx / A, A, 0.0};
    double cx = 0, cy = 0;
    cx = cx + p0.x; cy = cy + p0.y;
    cx = cx + p1.x; cy = cy + p1.y;
    fcen[f] = d2{cx / 2.0, cy / 2.0};
}

// triangle_area (mathTools/cellVolume.cpp:6-19)
__device__ __forceinline__ double tri_area(d2 p1, d2 p2, d2 p3) {
    double a = 0.5 * ((p1.x - p2.x) * (p1.y + p2.y) + (p2.x - p3.x) * (p2.y + p3.y) + (p3.x - p1.x) * (p3.y + p1.y));
    if (a < 0) a = -a;
    return a;
}

// computeCellVolume2D (mathTools/cellVolume.cpp:21-75) and cell3d::find_center
// (toolBox/cell3d_int.h:100-108).
__global__ void k_geom_cells(int nc, const int4* __restrict__ cv, const int* __restrict__ cnv, const d2* __restrict__ xy,
                             d4* __restrict__ cgeo) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    int4 v = cv[c];
    int n = cnv[c];
    d2 p[4];
    p[0] = xy[v.x]; p[1] = xy[v.y]; p[2] = xy[v.z];
    p[3] = n == 4 ? xy[v.w] : d2{0.0, 0.0};
    double area;
    if (n == 3) {
        area = tri_area(p[0], p[1], p[2]);
    } else {
        double abx = p[1].x - p[0].x, aby = p[1].y - p[0].y;
        double acx = p[2].x - p[0].x, acy = p[2].y - p[0].y;
        double adx = p[3].x - p[0].x, ady = p[3].y - p[0].y;
        // z components of AB x AC, AB x AD, AC x AD (the x,y components vanish in 2D)
        double abac = abx * acy - aby * acx;
        double abad = abx * ady - aby * adx;
        double acad = acx * ady - acy * adx;
        area = 0;
        if (abac * abad > 0) {
            if (acad * abad > 0) {
                area += tri_area(p[0], p[2], p[1]);
                area += tri_area(p[0], p[2], p[3]);
            } else {
                area += tri_area(p[0], p[3], p[1]);
                area += tri_area(p[0], p[3], p[2]);
            }
        } else {
            area += tri_area(p[0], p[1], p[2]);
            area += tri_area(p[0], p[1], p[3]);
        }
    }
    double cx = 0, cy = 0;
    for (int i = 0; i < n; i++) { cx = cx + p[i].x; cy = cy + p[i].y; }
    cgeo[c] = d4{area, cx / (double)n, cy / (double)n, 0.0};
}

// Per-face quantities the residual kernels read: 125*vol(left) for the limiter's
// epsilon^2 = K^3 * vol^(3/ndim) with K = 5 and the integer 3/2 = 1
// (Vankatakrishnan_Limiter.hpp:108,138 - both sides use the left cell's volume),
// the centre offsets of Vankatakrishnan_Limiter.hpp:107,137, and the centre line
// of LaminarFluxStrategy.h:136,149.
__global__ void k_geom_derived(int nf, const int2* __restrict__ lr, const d4* __restrict__ fgeo,
                               const d2* __restrict__ fcen, const d4* __restrict__ cgeo, d4* __restrict__ fg0,
                               d4* __restrict__ fg1, d4* __restrict__ fvis) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    int2 e = lr[f];
    d4 g = fgeo[f];
    d2 xf = fcen[f];
    d4 cl = cgeo[e.x];
    fg0[f] = d4{g.x, g.y, g.z, 125.0 * cl.x};
    double dlx = xf.x - cl.y, dly = xf.y - cl.z;
    double drx = 0, dry = 0, lx, ly;
    if (e.y >= 0) {
        d4 cr = cgeo[e.y];
        drx = xf.x - cr.y;
        dry = xf.y - cr.z;
        lx = cr.y - cl.y;
        ly = cr.z - cl.z;
    } else {
        lx = dlx;
        ly = dly;
    }
    fg1[f] = d4{dlx, dly, drx, dry};
    double l2 = 0;
    l2 += lx * lx;
    l2 += ly * ly;
    fvis[f] = d4{lx, ly, l2, 0.0};
}

void launch_geometry(const DevArrays& d, const LaunchCfg& L) {
    k_geom_faces<<<nblk(d.nf, 256), 256, 0, L.stream>>>(d.nf, d.enodes, d.xy, d.fgeo, d.fcen);
    k_geom_cells<<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.cverts, d.cnvert, d.xy, d.cgeo);
    k_geom_derived<<<nblk(d.nf, 256), 256, 0, L.stream>>>(d.nf, d.lr, d.fgeo, d.fcen, d.cgeo, d.fg0, d.fg1, d.fvis);
    *L.counter += 3;
}

// ---------------------------------------------------------------------------
// Residual, binary64.
template <bool V>
static void residual64(const DevArrays& d, const LaunchCfg& L, int first_order, int which) {
    if (which < 0 || which == 0) {
        k_face_state<double, V><<<nblk(d.nf, 256), 256, 0, L.stream>>>(d.nf, d.lr, d.fmesh, d.prm, d.fg0, d.U, d.Ue,
                                                                        d.fspec, d.mue, d.err,
                                                                        d.turb ? d.sstMut : nullptr,
                                                                        d.turb ? d.sstMutf : nullptr);
        *L.counter += 1;
    }
    if (which < 0 || which == 1) {
        k_cell_grad<double, V><<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.cface, d.lr, d.cmesh, d.prm, d.cgeo,
                                                                       d.fg0, d.fg1, d.U, d.Ue, d.fspec, first_order,
                                                                       d.grad, d.phi, d.specc, d.specv, d.gradT, d.mu);
        *L.counter += 1;
    }
    if (which < 0 || which == 2) {
        k_face_flux<double, V><<<nblk(d.nf, 256), 256, 0, L.stream>>>(d.nf, d.lr, d.fg0, d.fg1, d.fvis, d.U, d.grad,
                                                                       d.phi, d.Ue, d.mue, d.gradT, d.Fc, d.Fv, d.err,
                                                                       d.turb ? d.sstMutf : nullptr);
        *L.counter += 1;
    }
}
void launch_residual_fp64(const DevArrays& d, const LaunchCfg& L, bool viscous, int first_order, int which) {
    if (viscous) residual64<true>(d, L, first_order, which);
    else residual64<false>(d, L, first_order, which);
}

template <bool V, int M>
static void update64(const DevArrays& d, const LaunchCfg& L, double cfl, int stage, double alpha) {
    k_cell_update<double, V, M><<<nblk(d.nc, 256), 256, 0, L.stream>>>(
        d.nc, d.cface, d.cgeo, d.Fc, d.Fv, d.specc, d.specv, cfl, stage, alpha, d.R, d.U, d.W, d.W0, d.dt, d.diag,
        (d4*)nullptr, d.cflmul, d.turb);
    *L.counter += 1;
}
void launch_update_fp64(const DevArrays& d, const LaunchCfg& L, bool viscous, int mode, double cfl, int stage,
                        double alpha) {
    if (viscous) {
        if (mode == UPD_RESID) update64<true, UPD_RESID>(d, L, cfl, stage, alpha);
        else if (mode == UPD_RK) update64<true, UPD_RK>(d, L, cfl, stage, alpha);
        else update64<true, UPD_LUSGS>(d, L, cfl, stage, alpha);
    } else {
        if (mode == UPD_RESID) update64<false, UPD_RESID>(d, L, cfl, stage, alpha);
        else if (mode == UPD_RK) update64<false, UPD_RK>(d, L, cfl, stage, alpha);
        else update64<false, UPD_LUSGS>(d, L, cfl, stage, alpha);
    }
}

// ---------------------------------------------------------------------------
// LU-SGS sweeps.  For cell i of the current level, sum SolveDF over its faces in
// ascending order (TopologyHolderStrategy.cpp:217-323) taking only neighbours
// below i (forward) or above i (backward), then
//   forward:  dW1_i = (-R_i - sum) / D_i          (LUSGS_Integrator.cpp:492-523)
//   backward: dW_i  = dW1_i - sum / D_i           (LUSGS_Integrator.cpp:526-560)
// Cells of one level have no face between them, so they run in parallel and
// the result equals the reference's serial sweep.
// getMuOverPrCell (TopologyHolderStrategy.h:219-223; ViscousFlow2D.h:147-154):
// mu/Pr, plus mu_t/Prt when the SST model is coupled (mut != null)
template <class MuT>
__device__ __forceinline__ double mu_over_pr(const MuT* mu, const double* mut, int i) {
    return mut ? (double)mu[i] / 0.72 + mut[i] / 0.9 : (double)mu[i] / 0.72;
}
template <class MuT>
__device__ __forceinline__ float mu_over_pr_f(const MuT* mu, const double* mut, int i) {
    return mut ? (float)mu[i] / 0.72f + (float)mut[i] / 0.9f : (float)mu[i] / 0.72f;
}

template <bool VISC, bool FWD, class MuT>
__global__ void __launch_bounds__(128) k_sweep(int begin, int end, const int* __restrict__ order,
                                               const int4* __restrict__ cface, const int2* __restrict__ lr,
                                               const d4* __restrict__ fg0, const d4* __restrict__ fvis,
                                               const d4* __restrict__ W, const d4* __restrict__ U,
                                               const MuT* __restrict__ mu, const d4* __restrict__ R,
                                               const double* __restrict__ D, d4* dW1, d4* dW,
                                               const double* __restrict__ mut) {
    int idx = begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= end) return;
    const double G = 1.4;
    int i = order[idx];
    int4 cf = cface[i];
    int codes[4] = {cf.x, cf.y, cf.z, cf.w};
    double dF[4] = {0.0, 0.0, 0.0, 0.0};
    for (int s = 0; s < 4; s++) {
        int code = codes[s];
        if (code == 0) break;
        int f = code_face(code);
        bool left = code > 0;
        int2 e = lr[f];
        int j = left ? e.y : e.x;
        bool use = FWD ? (j >= 0 && j < i) : (j > i);
        double DF[4] = {0.0, 0.0, 0.0, 0.0};
        if (use) {
            double w0[4], dw[4], wp[4], fc[4], fcp[4], uj[4];
            to_arr(ld4(W + j), w0);
            to_arr(ld4((FWD ? dW1 : dW) + j), dw);
#pragma unroll
            for (int k = 0; k < 4; k++) wp[k] = w0[k] + dw[k];
            d4 g = fg0[f];
            double nx = g.x, ny = g.y, A = g.z;
            conv_flux_w<double>(w0, nx, ny, fc);
            conv_flux_w<double>(wp, nx, ny, fcp);
            to_arr(ld4(U + j), uj);
            // SolveViscousFlux (TopologyHolderStrategy.cpp:143-188)
            double vn = dot2(uj[2], uj[3], nx, ny);
            double c = sqrt(G * uj[1] / uj[0]);
            double rA = 1.5 * (fabs(vn) + c);
            if (VISC) rA += smax(4 / (3 * uj[0]), G / uj[0]) * mu_over_pr(mu, mut, i) / sqrt(fvis[f].z);
#pragma unroll
            for (int k = 0; k < 4; k++) {
                double fv = rA * dw[k];
                double dfc = left ? (fcp[k] - fc[k]) : (fc[k] - fcp[k]);
                DF[k] = 0.5 * (dfc - fv) * A;
            }
        }
#pragma unroll
        for (int k = 0; k < 4; k++) dF[k] += DF[k];
    }
    double Di = D[i];
    if (FWD) {
        double r[4];
        to_arr(ld4(R + i), r);
        st4(dW1 + i, d4{(-r[0] - dF[0]) / Di, (-r[1] - dF[1]) / Di, (-r[2] - dF[2]) / Di, (-r[3] - dF[3]) / Di});
    } else {
        double a[4];
        to_arr(ld4(dW1 + i), a);
        st4(dW + i, d4{a[0] - dF[0] / Di, a[1] - dF[1] / Di, a[2] - dF[2] / Di, a[3] - dF[3] / Di});
    }
}

template <class MuT>
static void sweep_t(const DevArrays& d, const LaunchCfg& L, bool viscous, bool forward, int begin, int end,
                    const MuT* mu) {
    int n = end - begin;
    const int* order = forward ? d.fwd_order : d.bwd_order;
    dim3 grid(nblk(n, 128));
    if (viscous) {
        if (forward) k_sweep<true, true, MuT><<<grid, 128, 0, L.stream>>>(begin, end, order, d.cface, d.lr, d.fg0, d.fvis, d.W, d.U, mu, d.R, d.diag, d.dW1, d.dW, d.turb ? d.sstMut : nullptr);
        else k_sweep<true, false, MuT><<<grid, 128, 0, L.stream>>>(begin, end, order, d.cface, d.lr, d.fg0, d.fvis, d.W, d.U, mu, d.R, d.diag, d.dW1, d.dW, d.turb ? d.sstMut : nullptr);
    } else {
        if (forward) k_sweep<false, true, MuT><<<grid, 128, 0, L.stream>>>(begin, end, order, d.cface, d.lr, d.fg0, d.fvis, d.W, d.U, mu, d.R, d.diag, d.dW1, d.dW, d.turb ? d.sstMut : nullptr);
        else k_sweep<false, false, MuT><<<grid, 128, 0, L.stream>>>(begin, end, order, d.cface, d.lr, d.fg0, d.fvis, d.W, d.U, mu, d.R, d.diag, d.dW1, d.dW, d.turb ? d.sstMut : nullptr);
    }
    *L.counter += 1;
}
void launch_sweep_level(const DevArrays& d, const LaunchCfg& L, bool viscous, bool forward, int begin, int end,
                        bool fp32) {
    if (end - begin <= 0) return;
    if (fp32) sweep_t<float>(d, L, viscous, forward, begin, end, d.muf);
    else sweep_t<double>(d, L, viscous, forward, begin, end, d.mu);
}

// ---------------------------------------------------------------------------
// Fast sweeps.  Within one LU-SGS step W, U, mu and the geometry are fixed, so
// the parts of SolveDF that do not depend on the neighbour's increment -
// F_c(W_j) and r_A (SolveViscousFlux) - are computed for every (cell, face slot)
// in one fully parallel pass.  The level kernel then only evaluates
// F_c(W_j + dW_j) and the combination, with 16 lanes per cell (4 face slots x
// 4 equations) so that a cell's dependent binary64 chain is one face long.
// The four slot contributions are added in slot (= ascending face) order
// starting from 0, exactly as the reference's loop, so results are unchanged.

// swfc[(i*4+s)*4+m] = F_c(W_j)[m] (ConservativeParam2ConvectiveFlux), swra[i*4+s] = r_A
template <bool VISC, class MuT>
__global__ void __launch_bounds__(256) k_sweep_prep(int nc, const int4* __restrict__ cface, const int2* __restrict__ lr,
                                                    const d4* __restrict__ fg0, const d4* __restrict__ fvis,
                                                    const d4* __restrict__ W, const d4* __restrict__ U,
                                                    const MuT* __restrict__ mu, double* __restrict__ swfc,
                                                    double* __restrict__ swra, double* __restrict__ dW1,
                                                    double* __restrict__ dW, int reset, const double* __restrict__ mut) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 4 * nc) return;
    if (reset) {  // the dataflow sweep's "not yet computed" marker (see k_sweep_flow)
        dW1[t] = __longlong_as_double((long long)kSentinel);
        dW[t] = __longlong_as_double((long long)kSentinel);
    }
    int i = t >> 2, s = t & 3;
    const double G = 1.4;
    int code = (&cface[i].x)[s];
    double fc[4] = {0.0, 0.0, 0.0, 0.0}, rA = 0.0;
    if (code != 0) {
        int f = code_face(code);
        int2 e = lr[f];
        int j = code > 0 ? e.y : e.x;
        if (j >= 0) {
            double w0[4], uj[4];
            to_arr(ld4(W + j), w0);
            to_arr(ld4(U + j), uj);
            d4 g = fg0[f];
            conv_flux_w<double>(w0, g.x, g.y, fc);
            double vn = dot2(uj[2], uj[3], g.x, g.y);
            double c = sqrt(G * uj[1] / uj[0]);
            rA = 1.5 * (fabs(vn) + c);
            if (VISC) rA += smax(4 / (3 * uj[0]), G / uj[0]) * mu_over_pr(mu, mut, i) / sqrt(fvis[f].z);
        }
    }
    st4(reinterpret_cast<d4*>(swfc) + t, d4{fc[0], fc[1], fc[2], fc[3]});
    swra[t] = rA;
}

template <bool FWD>
__global__ void __launch_bounds__(64) k_sweep16(int begin, int end, const int* __restrict__ order,
                                                const int4* __restrict__ cface, const int2* __restrict__ lr,
                                                const d4* __restrict__ fg0, const d4* __restrict__ W,
                                                const double* __restrict__ swfc, const double* __restrict__ swra,
                                                const d4* __restrict__ R, const double* __restrict__ D, d4* dW1,
                                                d4* dW) {
    const double GM1 = 1.4 - 1.0;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int lane = threadIdx.x & 31;
    int s = (lane >> 2) & 3, m = lane & 3;
    int idx = begin + (t >> 4);
    bool active = idx < end;
    int i = active ? order[idx] : 0;
    int4 cf = active ? cface[i] : make_int4(0, 0, 0, 0);
    int code = s == 0 ? cf.x : s == 1 ? cf.y : s == 2 ? cf.z : cf.w;
    double DF = 0.0;
    if (active && code != 0) {
        int f = code_face(code);
        bool left = code > 0;
        int2 e = lr[f];
        int j = left ? e.y : e.x;
        bool use = FWD ? (j >= 0 && j < i) : (j > i);
        if (use) {
            double w0[4], dw[4], wp[4];
            to_arr(ld4(W + j), w0);
            to_arr(ld4((FWD ? dW1 : dW) + j), dw);
#pragma unroll
            for (int k = 0; k < 4; k++) wp[k] = w0[k] + dw[k];
            d4 g = fg0[f];
            double u = wp[2] / wp[0], v = wp[3] / wp[0];
            double vn = dot2(u, v, g.x, g.y);
            double p = GM1 * (wp[1] - 0.5 * wp[0] * sq2(u, v));
            double fcp = m == 0 ? wp[0] * vn : m == 1 ? (wp[1] + p) * vn : m == 2 ? wp[2] * vn + p * g.x
                                                                                   : wp[3] * vn + p * g.y;
            double fc = swfc[(size_t)i * 16 + s * 4 + m];
            double rA = swra[(size_t)i * 4 + s];
            double dwm = m == 0 ? dw[0] : m == 1 ? dw[1] : m == 2 ? dw[2] : dw[3];
            double fv = rA * dwm;
            double dfc = left ? (fcp - fc) : (fc - fcp);
            DF = 0.5 * (dfc - fv) * g.z;
        }
    }
    // ordered sum over the cell's face slots (lanes m, m+4, m+8, m+12 of its 16-lane group)
    int base = lane & 16;
    double v0 = __shfl_sync(0xffffffffu, DF, base + m);
    double v1 = __shfl_sync(0xffffffffu, DF, base + 4 + m);
    double v2 = __shfl_sync(0xffffffffu, DF, base + 8 + m);
    double v3 = __shfl_sync(0xffffffffu, DF, base + 12 + m);
    if (!active || s != 0) return;
    double dF = 0.0;
    if (cf.x != 0) dF += v0;
    if (cf.y != 0) dF += v1;
    if (cf.z != 0) dF += v2;
    if (cf.w != 0) dF += v3;
    double Di = D[i];
    double* out = reinterpret_cast<double*>(FWD ? dW1 : dW) + (size_t)i * 4 + m;
    if (FWD) *out = (-(&R[i].x)[m] - dF) / Di;
    else *out = (&dW1[i].x)[m] - dF / Di;
}

void launch_sweep_prep(const DevArrays& d, const LaunchCfg& L, bool viscous, bool fp32, bool reset) {
    int n = 4 * d.nc;
    double* a = reinterpret_cast<double*>(d.dW1);
    double* b = reinterpret_cast<double*>(d.dW);
    int r = reset ? 1 : 0;
    if (viscous) {
        if (fp32) k_sweep_prep<true, float><<<nblk(n, 256), 256, 0, L.stream>>>(d.nc, d.cface, d.lr, d.fg0, d.fvis, d.W, d.U, d.muf, d.swfc, d.swra, a, b, r, d.turb ? d.sstMut : nullptr);
        else k_sweep_prep<true, double><<<nblk(n, 256), 256, 0, L.stream>>>(d.nc, d.cface, d.lr, d.fg0, d.fvis, d.W, d.U, d.mu, d.swfc, d.swra, a, b, r, d.turb ? d.sstMut : nullptr);
    } else {
        k_sweep_prep<false, double><<<nblk(n, 256), 256, 0, L.stream>>>(d.nc, d.cface, d.lr, d.fg0, d.fvis, d.W, d.U, (const double*)nullptr, d.swfc, d.swra, a, b, r, d.turb ? d.sstMut : nullptr);
    }
    *L.counter += 1;
}

void launch_sweep16_level(const DevArrays& d, const LaunchCfg& L, bool forward, int begin, int end) {
    int n = end - begin;
    if (n <= 0) return;
    int threads = 16 * n;
    if (forward)
        k_sweep16<true><<<nblk(threads, 64), 64, 0, L.stream>>>(begin, end, d.fwd_order, d.cface, d.lr, d.fg0, d.W, d.swfc, d.swra, d.R, d.diag, d.dW1, d.dW);
    else
        k_sweep16<false><<<nblk(threads, 64), 64, 0, L.stream>>>(begin, end, d.bwd_order, d.cface, d.lr, d.fg0, d.W, d.swfc, d.swra, d.R, d.diag, d.dW1, d.dW);
    *L.counter += 1;
}

// ---------------------------------------------------------------------------
// Dataflow sweep: one persistent cooperative launch per sweep direction.
// Cells are taken in level order, one warp per cell (positions p = k*G +
// warp*B + block); a cell waits only for its own lower (forward) / upper
// (backward) face neighbours.  The increments of a sweep are pre-filled with a
// signalling-NaN sentinel (k_sweep_prep, every step), and a neighbour's
// increment is final once none of its four 8-byte words - each written once,
// single-copy atomic - still holds the sentinel, so the data itself is the
// ready signal: no flags, fences or epochs.  Every dependency sits at an
// earlier position, all warps are resident (cooperative launch), and each warp
// finishes its positions in order, so the earliest unfinished cell can always
// proceed.  Every wait is bounded: after kSpinLimit polls the kernel raises
// ERR_TIMEOUT and goes on, so it always terminates.  Arithmetic never produces
// the sentinel (NaN results are quiet NaNs), so a NaN state cannot stall it.

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Spin until *flag == want, at most `limit` polls; on give-up raise ERR_TIMEOUT
// and return false (the caller goes on, so the kernel always terminates).
__device__ __forceinline__ bool bounded_wait(const unsigned* flag, unsigned want, long long limit, unsigned* err) {
    long long it = 0;
    while (ld_acquire_u32(flag) != want) {
        if (++it > limit) {
            atomicOr(err, ERR_TIMEOUT);
            return false;
        }
    }
    return true;
}

// Self-test of the bounded wait: waits on a flag nothing sets.
__global__ void k_wait_selftest(const unsigned* flag, long long limit, unsigned* err) {
    bounded_wait(flag, 0xffffffffu, limit, err);
}
void launch_wait_selftest(const DevArrays& d, const LaunchCfg& L, long long limit) {
    k_wait_selftest<<<1, 32, 0, L.stream>>>(d.err + 1, limit, d.err);
    *L.counter += 1;
}

template <bool FWD, bool PF>
__global__ void __launch_bounds__(256) k_sweep_flow(int nc, const int* __restrict__ order,
                                                    const int4* __restrict__ cface, const int2* __restrict__ lr,
                                                    const d4* __restrict__ fg0, const d4* __restrict__ W,
                                                    const double* __restrict__ swfc, const double* __restrict__ swra,
                                                    const d4* __restrict__ R, const double* __restrict__ D,
                                                    const double* __restrict__ invD, d4* dW1, d4* dW,
                                                    unsigned* err, int poll_ns) {
    sweep_flow_body<FWD, PF>(blockIdx.x, gridDim.x, nc, order, cface, lr, fg0, W, swfc, swra, R, D, invD, dW1, dW,
                             err, poll_ns, nullptr);
}

cudaError_t launch_sweep_flow(const DevArrays& d, const LaunchCfg& L, bool forward, int grid) {
    int nc = d.nc;
    const int* order = forward ? d.fwd_order : d.bwd_order;
    void* args[] = {(void*)&nc, (void*)&order, (void*)&d.cface, (void*)&d.lr, (void*)&d.fg0, (void*)&d.W,
                    (void*)&d.swfc, (void*)&d.swra, (void*)&d.R, (void*)&d.diag, (void*)&d.invD, (void*)&d.dW1,
                    (void*)&d.dW, (void*)&d.err, (void*)&d.poll_ns};
    void* fn = d.flow_pf ? (forward ? (void*)k_sweep_flow<true, true> : (void*)k_sweep_flow<false, true>)
                         : (forward ? (void*)k_sweep_flow<true, false> : (void*)k_sweep_flow<false, false>);
    cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(d.flow_threads), args, 0, L.stream);
    *L.counter += 1;
    return e;
}

// ---------------------------------------------------------------------------
// Plain-form dataflow sweep with two cells per warp.  Same protocol and the
// same binary64 arithmetic per cell as k_sweep_flow (so the increments are
// bit-identical), but each half-warp (16 lanes: 4 face slots x 4 equations)
// carries its own cell, the two cells of a pair coming from the same level
// (order2).  A warp-wide binary64 instruction holds its sub-partition's FP64
// pipe for 64 cycles however many lanes are active, so serving two cells with
// each instruction halves the pipe time per cell; but each half then computes
// both u = w2/w0 and v = w3/w0 (two divides on its chain instead of one) and a
// warp's two cells finish together, and on C2 the step came out 6% slower
// than with one cell per warp, which stays the default (sweep_mode 0).
template <bool FWD>
__global__ void __launch_bounds__(256) k_sweep_pair64(int npos, const int* __restrict__ order2,
                                                      const int4* __restrict__ cface, const int2* __restrict__ lr,
                                                      const d4* __restrict__ fg0, const d4* __restrict__ W,
                                                      const double* __restrict__ swfc,
                                                      const double* __restrict__ swra, const d4* __restrict__ R,
                                                      const double* __restrict__ D, d4* dW1, d4* dW, unsigned* err,
                                                      int poll_ns) {
    const double GM1 = 1.4 - 1.0;
    const int lane = threadIdx.x & 31;
    const int h = lane >> 4, base = lane & 16;
    const int s = (lane >> 2) & 3, m = lane & 3;
    const int warp = threadIdx.x >> 5;
    const int B = gridDim.x, NW = blockDim.x >> 5;
    d4* dst = FWD ? dW1 : dW;
    const int npairs = npos >> 1;
    const int q0 = ((warp - (int)(blockIdx.x % NW)) % NW + NW) % NW;
    for (long long q = q0;; q += NW) {
        const long long P = (long long)blockIdx.x + (long long)B * q;
        if (P >= npairs) break;
        const int i = order2[2 * P + h];
        const bool active = i >= 0;
        const int4 cf = active ? cface[i] : make_int4(0, 0, 0, 0);
        const int code = s == 0 ? cf.x : s == 1 ? cf.y : s == 2 ? cf.z : cf.w;
        bool use = false, left = false;
        int f = 0, j = 0;
        if (code != 0) {
            f = code_face(code);
            left = code > 0;
            int2 e = lr[f];
            j = left ? e.y : e.x;
            use = FWD ? (j >= 0 && j < i) : (j > i);
        }
        double own = 0.0, dinv = 1.0;
        if (active && s == 0) {
            own = FWD ? (&R[i].x)[m] : (&dW1[i].x)[m];
            dinv = D[i];
        }
        double w0[4] = {1.0, 1.0, 0.0, 0.0}, dw[4] = {0.0, 0.0, 0.0, 0.0};
        d4 g = d4{0.0, 0.0, 0.0, 0.0};
        double fc = 0.0, rA = 0.0;
        if (use) {
            to_arr(ld4(W + j), w0);
            g = fg0[f];
            fc = swfc[(size_t)i * 16 + s * 4 + m];
            rA = swra[(size_t)i * 4 + s];
            const double2* qp = reinterpret_cast<const double2*>(dst + j);
            double2 a, b;
            long long it = 0;
            while (true) {
                a = __ldcv(qp);
                b = __ldcv(qp + 1);
                if (!is_sentinel(a.x) && !is_sentinel(a.y) && !is_sentinel(b.x) && !is_sentinel(b.y)) break;
                if (++it > kSpinLimit) {
                    atomicOr(err, ERR_TIMEOUT);
                    break;
                }
                if (poll_ns > 0) __nanosleep(poll_ns);
            }
            dw[0] = a.x; dw[1] = a.y; dw[2] = b.x; dw[3] = b.y;
        }
        __syncwarp();
        double wp[4];
#pragma unroll
        for (int k = 0; k < 4; k++) wp[k] = w0[k] + dw[k];
        const double u = wp[2] / wp[0], v = wp[3] / wp[0];
        double vn = dot2(u, v, g.x, g.y);
        double pr = GM1 * (wp[1] - 0.5 * wp[0] * sq2(u, v));
        double fcp = m == 0 ? wp[0] * vn : m == 1 ? (wp[1] + pr) * vn : m == 2 ? wp[2] * vn + pr * g.x
                                                                               : wp[3] * vn + pr * g.y;
        double dwm = m == 0 ? dw[0] : m == 1 ? dw[1] : m == 2 ? dw[2] : dw[3];
        double dfc = left ? (fcp - fc) : (fc - fcp);
        double df = 0.5 * (dfc - rA * dwm) * g.z;
        double DF = use ? df : 0.0;
        double v0 = __shfl_sync(0xffffffffu, DF, base + m);
        double v1 = __shfl_sync(0xffffffffu, DF, base + 4 + m);
        double v2 = __shfl_sync(0xffffffffu, DF, base + 8 + m);
        double v3 = __shfl_sync(0xffffffffu, DF, base + 12 + m);
        double dF = 0.0;
        if (cf.x != 0) dF += v0;
        if (cf.y != 0) dF += v1;
        if (cf.z != 0) dF += v2;
        if (cf.w != 0) dF += v3;
        double res = 0.0;
        if (s == 0) res = FWD ? (-own - dF) / dinv : own - dF / dinv;
        double r1 = __shfl_sync(0xffffffffu, res, base + 1);
        double r2 = __shfl_sync(0xffffffffu, res, base + 2);
        double r3 = __shfl_sync(0xffffffffu, res, base + 3);
        if (active && (lane & 15) == 0) {
            double2* o = reinterpret_cast<double2*>(dst + i);
            __stcg(o, make_double2(res, r1));
            __stcg(o + 1, make_double2(r2, r3));
        }
    }
}

cudaError_t launch_sweep_pair64(const DevArrays& d, const LaunchCfg& L, bool forward, int grid) {
    int npos = forward ? d.npos2_fwd : d.npos2_bwd;
    const int* order = forward ? d.fwd_order2 : d.bwd_order2;
    void* args[] = {(void*)&npos, (void*)&order, (void*)&d.cface, (void*)&d.lr, (void*)&d.fg0, (void*)&d.W,
                    (void*)&d.swfc, (void*)&d.swra, (void*)&d.R, (void*)&d.diag, (void*)&d.dW1, (void*)&d.dW,
                    (void*)&d.err, (void*)&d.poll_ns};
    void* fn = forward ? (void*)k_sweep_pair64<true> : (void*)k_sweep_pair64<false>;
    cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(d.flow_threads), args, 0, L.stream);
    *L.counter += 1;
    return e;
}

// ---------------------------------------------------------------------------
// Fast-form dataflow sweep.  Same protocol as k_sweep_flow, but everything on
// the dependence chain except the final update is binary32: float copies of
// W (Wf), of the per-step r_A constants and of the increments (dW1f/dWf,
// published beside the binary64 increments and polled instead of them), so
// the binary64 pipe only sees the widening of the slot sum and
// dW = (-R - sum) * (1/D).  Two cells per warp (16 lanes each): the cells of a
// pair always come from the same level (order2 pads odd levels with -1), so
// the two halves never depend on each other and may wait for each other.

template <bool VISC, class MuT>
__global__ void __launch_bounds__(256) k_sweep_prep32(int nc, const int4* __restrict__ cface, const int2* __restrict__ lr,
                                                      const float4* __restrict__ fg0f, const float4* __restrict__ fvisf,
                                                      const d4* __restrict__ W, const d4* __restrict__ U,
                                                      const MuT* __restrict__ mu,
                                                      float* __restrict__ swraf, float4* __restrict__ Wf,
                                                      float* __restrict__ dW1f, float* __restrict__ dWf,
                                                      const double* __restrict__ mut) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 4 * nc) return;
    int i = t >> 2, s = t & 3;
    const float G = 1.4f;
    dW1f[t] = __uint_as_float(kSentinelF);
    dWf[t] = __uint_as_float(kSentinelF);
    if (s == 0) {
        d4 w = ld4(W + i);
        Wf[i] = make_float4((float)w.x, (float)w.y, (float)w.z, (float)w.w);
    }
    int code = (&cface[i].x)[s];
    float rA = 0.f;
    if (code != 0) {
        int f = code_face(code);
        int2 e = lr[f];
        int j = code > 0 ? e.y : e.x;
        if (j >= 0) {
            d4 ud = ld4(U + j);
            float uj[4] = {(float)ud.x, (float)ud.y, (float)ud.z, (float)ud.w};
            float4 g = fg0f[f];
            float vn = uj[2] * g.x + uj[3] * g.y;
            float c = sqrtf(G * uj[1] / uj[0]);
            rA = 1.5f * (fabsf(vn) + c);
            if (VISC) rA += fmaxf(4.f / (3.f * uj[0]), G / uj[0]) * mu_over_pr_f(mu, mut, i) / sqrtf(fvisf[f].z);
        }
    }
    swraf[t] = rA;
}

void launch_sweep_prep32(const DevArrays& d, const LaunchCfg& L, bool viscous, int mu_kind) {
    int n = 4 * d.nc;
    float* a = reinterpret_cast<float*>(d.dW1f);
    float* b = reinterpret_cast<float*>(d.dWf);
    if (viscous && mu_kind == MU_F64)
        k_sweep_prep32<true, double><<<nblk(n, 256), 256, 0, L.stream>>>(d.nc, d.cface, d.lr, d.fg0f, d.fvisf, d.W, d.U, d.mu, d.swraf, d.Wf, a, b, d.turb ? d.sstMut : nullptr);
    else if (viscous && mu_kind == MU_FF)
        k_sweep_prep32<true, ff><<<nblk(n, 256), 256, 0, L.stream>>>(d.nc, d.cface, d.lr, d.fg0f, d.fvisf, d.W, d.U, d.muq, d.swraf, d.Wf, a, b, d.turb ? d.sstMut : nullptr);
    else if (viscous)
        k_sweep_prep32<true, float><<<nblk(n, 256), 256, 0, L.stream>>>(d.nc, d.cface, d.lr, d.fg0f, d.fvisf, d.W, d.U, d.muf, d.swraf, d.Wf, a, b, d.turb ? d.sstMut : nullptr);
    else
        k_sweep_prep32<false, float><<<nblk(n, 256), 256, 0, L.stream>>>(d.nc, d.cface, d.lr, d.fg0f, d.fvisf, d.W, d.U, (const float*)nullptr, d.swraf, d.Wf, a, b, d.turb ? d.sstMut : nullptr);
    *L.counter += 1;
}

template <bool FWD, bool IND, bool PF>
__global__ void __launch_bounds__(256) k_sweep_flow32(int npos, const int* __restrict__ order2,
                                                      const int4* __restrict__ cface, const int2* __restrict__ lr,
                                                      const float4* __restrict__ fg0f, const float4* __restrict__ Wf,
                                                      const float* __restrict__ swraf,
                                                      const d4* __restrict__ R, const double* __restrict__ invD,
                                                      d4* dW1, d4* dW, float4* dW1f, float4* dWf, unsigned* err,
                                                      int poll_ns) {
    sweep_flow32_body<FWD, IND, PF>(blockIdx.x, gridDim.x, npos, order2, cface, lr, fg0f, Wf, swraf, R, invD, dW1, dW,
                                    dW1f, dWf, err, poll_ns, nullptr);
}

cudaError_t launch_sweep_flow32(const DevArrays& d, const LaunchCfg& L, bool forward, int grid, bool independent) {
    int npos = forward ? d.npos2_fwd : d.npos2_bwd;
    const int* order = forward ? d.fwd_order2 : d.bwd_order2;
    void* args[] = {(void*)&npos, (void*)&order, (void*)&d.cface, (void*)&d.lr, (void*)&d.fg0f, (void*)&d.Wf,
                    (void*)&d.swraf, (void*)&d.R, (void*)&d.invD, (void*)&d.dW1, (void*)&d.dW,
                    (void*)&d.dW1f, (void*)&d.dWf, (void*)&d.err, (void*)&d.poll_ns};
    void* fn;
    if (d.flow_pf)
        fn = independent ? (forward ? (void*)k_sweep_flow32<true, true, true> : (void*)k_sweep_flow32<false, true, true>)
                         : (forward ? (void*)k_sweep_flow32<true, false, true> : (void*)k_sweep_flow32<false, false, true>);
    else
        fn = independent ? (forward ? (void*)k_sweep_flow32<true, true, false> : (void*)k_sweep_flow32<false, true, false>)
                         : (forward ? (void*)k_sweep_flow32<true, false, false> : (void*)k_sweep_flow32<false, false, false>);
    cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(d.flow_threads), args, 0, L.stream);
    *L.counter += 1;
    return e;
}

int sweep_flow_max_grid(bool low, int blocks_per_sm, int threads, bool pf) {
    int dev = 0, sms = 0, per = 0, per2 = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    void* fn = low ? (pf ? (void*)k_sweep_flow32<true, false, true> : (void*)k_sweep_flow32<true, false, false>)
                   : (pf ? (void*)k_sweep_flow<true, true> : (void*)k_sweep_flow<true, false>);
    void* fn2 = low ? (pf ? (void*)k_sweep_flow32<false, false, true> : (void*)k_sweep_flow32<false, false, false>)
                    : (pf ? (void*)k_sweep_flow<false, true> : (void*)k_sweep_flow<false, false>);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, fn2, threads, 0);
    per = per < per2 ? per : per2;
    if (low) {  // the independent-halves variant runs on the same grid
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per2, pf ? (void*)k_sweep_flow32<true, true, true> : (void*)k_sweep_flow32<true, true, false>, threads, 0);
        per = per < per2 ? per : per2;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per2, pf ? (void*)k_sweep_flow32<false, true, true> : (void*)k_sweep_flow32<false, true, false>, threads, 0);
        per = per < per2 ? per : per2;
    }
    if (!low) {  // the plain form's paired kernels run on the same grid
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, (void*)k_sweep_pair64<true>, threads, 0);
        per = per < per2 ? per : per2;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, (void*)k_sweep_pair64<false>, threads, 0);
        per = per < per2 ? per : per2;
    }
    if (per < 1) per = 1;
    int want = blocks_per_sm > 0 ? blocks_per_sm : 2;
    return sms * (want < per ? want : per);
}

// ---------------------------------------------------------------------------
// Chain-scheduled fast-form sweep (sweep_mode 5).
//
// The dataflow sweeps above deal cells to warps round-robin in level order, so
// every dependency, even one on the cell that was finished just before, makes
// the round trip publish -> L2 -> poll, and each level of the dependence chain
// costs one such round trip plus the arithmetic.  Here a host schedule gives
// each half-warp its own list of cells (ascending level), and a cell goes,
// where it can, to the half-warp that ran its latest-level dependency as its
// previous item.  The half-warp keeps its last two results in registers and
// takes a dependency on them without touching memory, so a chain of such cells
// (a quad row along the body, for instance) advances at the speed of the
// arithmetic; only dependencies between half-warps pay the round trip.
//
// The arithmetic of a cell is that of k_sweep_flow32 operation for operation
// (same TU, same -fmad=false), so both give identical bits.  The binary64
// increments are not formed on the chain: the sweep stores its binary32 slot
// sums and k_chain_mid / k_chain_finish form dW1 = (-R - sum) / D and
// dW = dW1 - sum / D with the expressions of k_sweep_flow32.
//
// Per-item data are staged per step in schedule order (16 float4 per
// position, k_chain_cell and k_chain_prep, which also form the neighbour's velocity, pressure
// and normal velocity: the terms of the flux difference that do not depend on
// the increment) and copied ahead into a shared-memory ring of kChainDepth
// items per warp with cp.async; the increment of a remote dependency is also
// read early, kChainAhead items ahead, into shared memory (if it is not
// published yet the cell polls L2 as before).  One list per warp, 16 lanes: two
// lists sharing a warp would issue one after the other.
//
// Progress: all warps are co-resident (cooperative launch, schedule built for
// exactly this grid), each runs its list in ascending level and every
// dependency lies on a strictly lower level, so the lowest unfinished cell can
// always proceed.  Every wait is bounded (kSpinLimit); after one gives up the
// warp stops waiting and the error word carries ERR_TIMEOUT.
//
// Stage record of position p (float4 index p*16 + k), slot s = face slot:
//   k 0-3   (rho, E + p, rho u, rho v) of slot s's neighbour (binary32)   per step (k_chain_cell / _prep)
//   k 4-7   (u, v, u^2 + v^2, u nx + v ny) of the same                    per step
//   k 8-11  (nx, ny, A) of slot s's face; r_A in .w                      static; per step
//   k 12    own term (R forward, dW1 backward, binary32)                 per step
//   k 13    (1/D, cell id, existing-slot bits, 0)                        per step; static
//   k 14-15 (j, face code) bits of slots 0,1 and 2,3                    static
// j: the cell slot s waits for, -1 none, -2 / -3 the list's previous cell /
// the one before it (the warp holds their increments in registers).
// Slots without a dependency hold the neutral state (1, 1, 0, 0).
constexpr int kChainDepth = 8;  // stage records in flight per warp
constexpr int kChainAhead = 2;  // items ahead at which a remote dependency is read early
constexpr int kStageW = 16;
constexpr int kChainWarps = 8;  // warps (lists) per block
static_assert(2 * kChainAhead + 1 < kChainDepth && kChainAhead >= 2 && (kChainDepth & (kChainDepth - 1)) == 0,
              "ring accounting");

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <bool FWD>
__global__ void __launch_bounds__(256) k_sweep_chain32(int nh, const int* __restrict__ hptr,
                                                       const float4* __restrict__ stage, float4* pub,
                                                       float4* __restrict__ dFout, unsigned* err, int poll_ns,
                                                       int tbl_n) {
    __shared__ __align__(16) float4 ring[kChainWarps][kChainDepth][kStageW];
    __shared__ __align__(16) float4 spec[kChainWarps][kChainDepth][4];
    // block-local hand-off table (sweep mode 6): the increment of each cell
    // of this block's lists at positions [0, tbl_n) of the block's range (all
    // of them unless the table was capped to keep the grid co-resident); a
    // slot whose producer has an entry waits here instead of in global memory
    extern __shared__ __align__(16) float4 tbl[];
    const float GM1 = 1.4f - 1.0f;
    const int lane = threadIdx.x & 31;
    const int s = (lane >> 2) & 3, m = lane & 3;
    constexpr unsigned mask = 0x0000ffffu;
    if ((int)(gridDim.x * (blockDim.x >> 5)) != nh) {  // a schedule built for another grid
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(err, ERR_SCHED);
        return;
    }
    const float sent = __uint_as_float(kSentinelF);
    for (int t = threadIdx.x; t < tbl_n; t += blockDim.x) tbl[t] = make_float4(sent, sent, sent, sent);
    __syncthreads();
    if (lane >= 16) return;
    const int warp = threadIdx.x >> 5;
    const int hw = blockIdx.x * (blockDim.x >> 5) + warp;
    const int p0 = hptr[hw], p1 = hptr[hw + 1];
    if (p0 >= p1) return;
    const int n = p1 - p0;
    float4(*R)[kStageW] = ring[warp];
    float4(*S)[4] = spec[warp];
    // cp.async groups: the prologue commits one group per record of items
    // 0 .. kChainDepth-1; item k then commits the early read for item
    // k + kChainAhead and, separately and after it, the refill of item k-1's
    // slot with item k-1 + kChainDepth, so that waiting for an early read does
    // not wait for the refill issued beside it
#pragma unroll
    for (int k = 0; k < kChainDepth; k++) {
        if (k < n) cp_async16(&R[k][lane], stage + (size_t)(p0 + k) * kStageW + lane);
        cp_async_commit();
    }
    float4 hd1 = make_float4(0.f, 0.f, 0.f, 0.f), hd2 = hd1;  // increments of the last two cells
    const int b0 = hptr[blockIdx.x * kChainWarps];  // first position of this block's lists
    bool gave_up = false;
    for (int k = 0; k < n; k++) {
        const int slot = k & (kChainDepth - 1);
        // all but the 2*kChainAhead-1 latest groups are complete: this item's
        // early read and every refill up to item k + kChainAhead's record.
        // The barrier also orders the previous item's reads of its slot
        // before the refill of that slot below.
        cp_async_wait<2 * kChainAhead - 1>();
        __syncwarp(mask);
        const float4 A = R[slot][s];
        const float4 B = R[slot][4 + s];
        const float4 gr = R[slot][8 + s];
        const float ownf_ = (&R[slot][12].x)[m];
        const float4 misc = R[slot][13];
        const float4 jc01 = R[slot][14], jc23 = R[slot][15];
        const float4 early = k >= kChainAhead ? S[slot][s] : make_float4(sent, sent, sent, sent);
        // early read for the item kChainAhead positions on, when it waits for
        // another warp's cell
        int ja = -1;
        if (k + kChainAhead < n) {
            const float4 jca = R[(k + kChainAhead) & (kChainDepth - 1)][14 + (s >> 1)];
            ja = __float_as_int((s & 1) ? jca.z : jca.x);
        }
        if (m == 0 && ja >= 0) cp_async16(&S[(k + kChainAhead) & (kChainDepth - 1)][s], pub + ja);
        cp_async_commit();
        if (k > 0 && k - 1 + kChainDepth < n)
            cp_async16(&R[(k - 1) & (kChainDepth - 1)][lane], stage + (size_t)(p0 + k - 1 + kChainDepth) * kStageW + lane);
        cp_async_commit();
        const int i = __float_as_int(misc.y);
        const float dinvf = misc.x;
        const float4 jc = s < 2 ? jc01 : jc23;
        const int j = __float_as_int((s & 1) ? jc.z : jc.x);
        const int code = __float_as_int((s & 1) ? jc.w : jc.y);
        const bool use = j != -1, left = code > 0;
        const int exm = __float_as_int(misc.z);  // bit s: face slot s exists
        float4 dw = make_float4(0.f, 0.f, 0.f, 0.f);
        if (use) {
            if (j == -2) {
                dw = hd1;
            } else if (j == -3) {
                dw = hd2;
            } else if (j <= -4) {  // produced in this block: wait on the shared-memory table
                const volatile float* q = reinterpret_cast<const volatile float*>(tbl + (-4 - j));
                dw = make_float4(q[0], q[1], q[2], q[3]);
                long long it = 0;
                while (is_sentinel_f(dw.x) || is_sentinel_f(dw.y) || is_sentinel_f(dw.z) || is_sentinel_f(dw.w)) {
                    if (gave_up) break;
                    if (++it > kSpinLimit) {
                        atomicOr(err, ERR_TIMEOUT);
                        gave_up = true;
                        break;
                    }
                    dw = make_float4(q[0], q[1], q[2], q[3]);
                }
            } else {
                dw = early;
                const float4* qf = pub + j;
                long long it = 0;
                while (is_sentinel_f(dw.x) || is_sentinel_f(dw.y) || is_sentinel_f(dw.z) || is_sentinel_f(dw.w)) {
                    dw = __ldcv(qf);
                    if (gave_up) break;
                    if (++it > kSpinLimit) {
                        atomicOr(err, ERR_TIMEOUT);
                        gave_up = true;
                        break;
                    }
                    if (poll_ns > 0) __nanosleep(poll_ns);
                }
            }
        }
        const float rho = A.x, Ep = A.y, mx = A.z, my = A.w;
        const float u = B.x, v = B.y, vv = B.z, vn = B.w;
        const float d0 = dw.x, d1 = dw.y, d2 = dw.z, d3 = dw.w;
        const float rp = 1.f / (rho + d0);
        const float du = (d2 - u * d0) * rp, dv = (d3 - v * d0) * rp;
        const float dq = du * (u + u + du) + dv * (v + v + dv);
        const float dp = GM1 * (d1 - 0.5f * (d0 * (vv + dq) + rho * dq));
        const float dvn = du * gr.x + dv * gr.y;
        const float vnp = vn + dvn;
        const float dfm = m == 0 ? d2 * gr.x + d3 * gr.y
                        : m == 1 ? (d1 + dp) * vnp + Ep * dvn
                        : m == 2 ? d2 * vnp + mx * dvn + dp * gr.x
                                 : d3 * vnp + my * dvn + dp * gr.y;
        float dwm = m == 0 ? dw.x : m == 1 ? dw.y : m == 2 ? dw.z : dw.w;
        float dfc = left ? dfm : -dfm;
        float DF = use ? 0.5f * (dfc - gr.w * dwm) * gr.z : 0.f;
        float v0 = __shfl_sync(mask, DF, m);
        float v1 = __shfl_sync(mask, DF, 4 + m);
        float v2 = __shfl_sync(mask, DF, 8 + m);
        float v3 = __shfl_sync(mask, DF, 12 + m);
        float dF = 0.f;
        if (exm & 1) dF += v0;
        if (exm & 2) dF += v1;
        if (exm & 4) dF += v2;
        if (exm & 8) dF += v3;
        const float resf = FWD ? (-ownf_ - dF) * dinvf : ownf_ - dF * dinvf;
        const float r0 = __shfl_sync(mask, resf, 0);
        const float r1 = __shfl_sync(mask, resf, 1);
        const float r2 = __shfl_sync(mask, resf, 2);
        const float r3 = __shfl_sync(mask, resf, 3);
        if (lane == 0) {
            __stcg(pub + i, make_float4(r0, r1, r2, r3));
            if (p0 + k - b0 < tbl_n) {  // the table may cover only the block's first positions
                volatile float* q = reinterpret_cast<volatile float*>(tbl + (p0 + k - b0));
                q[0] = r0; q[1] = r1; q[2] = r2; q[3] = r3;
            }
        }
        if (s == 0) (&dFout[i].x)[m] = dF;
        hd2 = hd1;
        hd1 = make_float4(r0, r1, r2, r3);
    }
    cp_async_wait<0>();
}

// Static part of the stage records, once per schedule: cell ids, neighbour /
// face-code pairs and binary32 face geometry.
__global__ void k_chain_static(int nc, const int2* __restrict__ cells, const int2* __restrict__ rec,
                               const int* __restrict__ jenc, const float4* __restrict__ fg0f,
                               float4* __restrict__ stage) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 4LL * nc) return;
    const int p = (int)(t >> 2), s = (int)(t & 3);
    float4* st = stage + (size_t)p * kStageW;
    const int2 r = rec[t];
    float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
    if (r.x >= 0) g = fg0f[code_face(r.y)];
    st[8 + s] = make_float4(g.x, g.y, g.z, 0.f);
    const int2 cl = cells[p];
    // -1 none, -2 / -3 the list's previous cell / the one before (registers),
    // <= -4 a cell of the same block (shared-memory table index -4 - j), else the cell id
    const int j = jenc[t];
    reinterpret_cast<float2*>(st + 14 + (s >> 1))[s & 1] = make_float2(__int_as_float(j), __int_as_float(r.y));
    if (s == 0) {
        int exm = 0;
        for (int k = 0; k < 4; k++) exm |= (rec[4 * (long long)p + k].y != 0) << k;
        st[13] = make_float4(0.f, __int_as_float(cl.x), __int_as_float(exm), 0.f);
    }
}

// Per-step cell pass of the chain sweep, in place of k_inv_diag and the cell
// part of k_sweep_prep32: binary32 copies of W and U (each converted once,
// with the conversions those kernels use), 1/D in binary64, and the "not yet
// computed" sentinel in both directions' published increments.
__global__ void k_chain_cell(int nc, const d4* __restrict__ W, const d4* __restrict__ U,
                             const double* __restrict__ D, float4* __restrict__ Wf, float4* __restrict__ Uf,
                             double* __restrict__ invD, float4* __restrict__ pub_f, float4* __restrict__ pub_b) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const d4 w = ld4(W + c), u = ld4(U + c);
    Wf[c] = make_float4((float)w.x, (float)w.y, (float)w.z, (float)w.w);
    Uf[c] = make_float4((float)u.x, (float)u.y, (float)u.z, (float)u.w);
    invD[c] = 1.0 / D[c];
    const float sent = __uint_as_float(kSentinelF);
    pub_f[c] = make_float4(sent, sent, sent, sent);
    pub_b[c] = make_float4(sent, sent, sent, sent);
}

// Per-step slot pass of both directions' stage records, after k_chain_cell,
// in schedule order (coalesced writes): the neighbours' binary32 state, its
// increment-free terms and r_A, each with the expression k_sweep_prep32 and
// k_sweep_flow32 use; binary32 1/D and the forward own term R.  (The backward
// own term, dW1, is written by k_chain_mid.)
template <bool VISC, class MuT>
__global__ void k_chain_prep(int nc, float4* __restrict__ stage_f, float4* __restrict__ stage_b,
                             const int2* __restrict__ rec_f, const int2* __restrict__ rec_b,
                             const float4* __restrict__ fvisf, const float4* __restrict__ Wf,
                             const float4* __restrict__ Uf, const MuT* __restrict__ mu, const d4* __restrict__ R,
                             const double* __restrict__ invD, const double* __restrict__ mut) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 8LL * nc) return;
    const float GM1 = 1.4f - 1.0f;
    const float G = 1.4f;
    const int dir = t >= 4LL * nc;
    const long long q = dir ? t - 4LL * nc : t;
    const int p = (int)(q >> 2), s = (int)(q & 3);
    float4* st = (dir ? stage_b : stage_f) + (size_t)p * kStageW;
    const int2 r = (dir ? rec_b : rec_f)[q];
    const int j = r.x;
    const float4 g = st[8 + s];
    float4 w0 = make_float4(1.f, 1.f, 0.f, 0.f);
    float rA = 0.f, u = 0.f, v = 0.f, vv = 0.f, pb = 0.f, vn = 0.f;
    if (j >= 0) {
        const int i = __float_as_int(st[13].y);
        w0 = Wf[j];
        const float4 uf = Uf[j];
        const float uj[4] = {uf.x, uf.y, uf.z, uf.w};
        const float vr = uj[2] * g.x + uj[3] * g.y;
        const float c = sqrtf(G * uj[1] / uj[0]);
        rA = 1.5f * (fabsf(vr) + c);
        if (VISC) rA += fmaxf(4.f / (3.f * uj[0]), G / uj[0]) * mu_over_pr_f(mu, mut, i) / sqrtf(fvisf[code_face(r.y)].z);
        u = w0.z / w0.x;
        v = w0.w / w0.x;
        vv = u * u + v * v;
        pb = GM1 * (w0.y - 0.5f * w0.x * vv);
        vn = u * g.x + v * g.y;
    }
    st[s] = make_float4(w0.x, w0.y + pb, w0.z, w0.w);
    st[4 + s] = make_float4(u, v, vv, vn);
    st[8 + s] = make_float4(g.x, g.y, g.z, rA);
    if (s == 0) {
        float4 misc = st[13];
        const int i = __float_as_int(misc.y);
        misc.x = (float)invD[i];
        st[13] = misc;
        if (!dir) {
            const d4 rr = ld4(R + i);
            st[12] = make_float4((float)rr.x, (float)rr.y, (float)rr.z, (float)rr.w);
        }
    }
}

// dW1 = (-R - sum) * (1/D) in binary64 (k_sweep_flow32's forward expression),
// and its binary32 copy, the own term of the backward stage records
__global__ void k_chain_mid(int nc, const d4* __restrict__ R, const double* __restrict__ invD,
                            const float4* __restrict__ dF, const int* __restrict__ posb, d4* __restrict__ dW1,
                            float4* __restrict__ stage_b) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    d4 r = ld4(R + c);
    const double dinv = invD[c];
    const float4 f = dF[c];
    d4 o;
    o.x = (-r.x - (double)f.x) * dinv;
    o.y = (-r.y - (double)f.y) * dinv;
    o.z = (-r.z - (double)f.z) * dinv;
    o.w = (-r.w - (double)f.w) * dinv;
    dW1[c] = o;
    stage_b[(size_t)posb[c] * kStageW + 12] = make_float4((float)o.x, (float)o.y, (float)o.z, (float)o.w);
}

// dW = dW1 - sum * (1/D) in binary64 (k_sweep_flow32's backward expression)
__global__ void k_chain_finish(int nc, const d4* __restrict__ dW1, const double* __restrict__ invD,
                               const float4* __restrict__ dF, d4* __restrict__ dW) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    d4 a = ld4(dW1 + c);
    const double dinv = invD[c];
    const float4 f = dF[c];
    d4 o;
    o.x = a.x - (double)f.x * dinv;
    o.y = a.y - (double)f.y * dinv;
    o.z = a.z - (double)f.z * dinv;
    o.w = a.w - (double)f.w * dinv;
    dW[c] = o;
}

// Whether `grid` blocks of the chain sweep, each with `tbl_bytes` of dynamic
// shared memory, are co-resident (a cooperative launch needs all of them).
bool sweep_chain_fits(int grid, int tbl_bytes) {
    int dev = 0, sms = 0, per = 0, per2 = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (tbl_bytes > 48 * 1024) {
        if (cudaFuncSetAttribute((void*)k_sweep_chain32<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, tbl_bytes) ||
            cudaFuncSetAttribute((void*)k_sweep_chain32<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, tbl_bytes)) {
            cudaGetLastError();
            return false;
        }
    }
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (void*)k_sweep_chain32<true>, 256, tbl_bytes) ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, (void*)k_sweep_chain32<false>, 256, tbl_bytes)) {
        cudaGetLastError();
        return false;
    }
    return (long long)sms * (per < per2 ? per : per2) >= grid;
}

int sweep_chain_max_grid(int blocks_per_sm) {
    int dev = 0, sms = 0, per = 0, per2 = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (void*)k_sweep_chain32<true>, 256, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, (void*)k_sweep_chain32<false>, 256, 0);
    per = per < per2 ? per : per2;
    if (per < 1) per = 1;
    int want = blocks_per_sm > 0 ? blocks_per_sm : 2;
    return sms * (want < per ? want : per);
}

void launch_chain_static(const DevArrays& d, const LaunchCfg& L) {
    for (int k = 0; k < 2; k++)
        k_chain_static<<<nblk(4 * d.nc, 256), 256, 0, L.stream>>>(d.nc, d.chain_cells[k], d.chain_rec[k],
                                                                  d.chain_jenc[k], d.fg0f, d.chain_stage[k]);
    *L.counter += 2;
}

cudaError_t launch_sweep_chain32(const DevArrays& d, const LaunchCfg& L, bool forward, int grid, bool viscous,
                                 int mu_kind) {
    const int k = forward ? 0 : 1;
    int nh = d.chain_nh;
    float4* pub = forward ? d.dW1f : d.dWf;
    if (forward) {
        k_chain_cell<<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.W, d.U, d.diag, d.Wf, d.Uf, d.invD, d.dW1f,
                                                            d.dWf);
        const int nb = nblk(8 * d.nc, 256);
        if (viscous && mu_kind == MU_F64)
            k_chain_prep<true, double><<<nb, 256, 0, L.stream>>>(d.nc, d.chain_stage[0], d.chain_stage[1],
                                                                 d.chain_rec[0], d.chain_rec[1], d.fvisf, d.Wf, d.Uf,
                                                                 d.mu, d.R, d.invD, d.turb ? d.sstMut : nullptr);
        else if (viscous && mu_kind == MU_FF)
            k_chain_prep<true, ff><<<nb, 256, 0, L.stream>>>(d.nc, d.chain_stage[0], d.chain_stage[1],
                                                             d.chain_rec[0], d.chain_rec[1], d.fvisf, d.Wf, d.Uf,
                                                             d.muq, d.R, d.invD, d.turb ? d.sstMut : nullptr);
        else if (viscous)
            k_chain_prep<true, float><<<nb, 256, 0, L.stream>>>(d.nc, d.chain_stage[0], d.chain_stage[1],
                                                                d.chain_rec[0], d.chain_rec[1], d.fvisf, d.Wf, d.Uf,
                                                                d.muf, d.R, d.invD, d.turb ? d.sstMut : nullptr);
        else
            k_chain_prep<false, float><<<nb, 256, 0, L.stream>>>(d.nc, d.chain_stage[0], d.chain_stage[1],
                                                                 d.chain_rec[0], d.chain_rec[1], d.fvisf, d.Wf, d.Uf,
                                                                 (const float*)nullptr, d.R, d.invD, d.turb ? d.sstMut : nullptr);
        *L.counter += 2;
    }
    int tbl_n = d.chain_tbl;
    void* args[] = {(void*)&nh, (void*)&d.chain_ptr[k], (void*)&d.chain_stage[k], (void*)&pub, (void*)&d.chain_dF,
                    (void*)&d.err, (void*)&d.poll_ns, (void*)&tbl_n};
    void* fn = forward ? (void*)k_sweep_chain32<true> : (void*)k_sweep_chain32<false>;
    cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(256), args, (size_t)tbl_n * sizeof(float4),
                                                L.stream);
    *L.counter += 1;
    if (e != cudaSuccess) return e;
    if (forward)
        k_chain_mid<<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.R, d.invD, d.chain_dF, d.chain_posb, d.dW1,
                                                           d.chain_stage[1]);
    else
        k_chain_finish<<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.dW1, d.invD, d.chain_dF, d.dW);
    *L.counter += 1;
    return cudaSuccess;
}

// Cp and Mach number of cells [begin, end) as TopologyHolderStrategy::
// writeCellData forms them (TopologyHolderStrategyOutput.cpp:523-538):
// Cp = 2 (p - p_inf) / (u_inf^2 + v_inf^2) and Ma = |u| / sqrt(p / rho).
__global__ void k_cp_ma(int begin, int end, const d4* __restrict__ U, double pinf, double uinf, double vinf,
                        double* __restrict__ out) {
    const int c = begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= end) return;
    const d4 u = ld4(U + c);
    const double vm = uinf * uinf + vinf * vinf;
    const double cp = 2 * (u.y - pinf) / vm;
    const double cs = sqrt(u.y / u.x);
    double vel = 0;
    vel += u.z * u.z;
    vel += u.w * u.w;
    vel = sqrt(vel);
    out[2 * (size_t)(c - begin)] = cp;
    out[2 * (size_t)(c - begin) + 1] = vel / cs;
}

void launch_cp_ma(const DevArrays& d, const LaunchCfg& L, int begin, int end, double pinf, double uinf, double vinf,
                  double* out) {
    if (end <= begin) return;
    k_cp_ma<<<nblk(end - begin, 256), 256, 0, L.stream>>>(begin, end, d.U, pinf, uinf, vinf, out);
    *L.counter += 1;
}

// Limited left / right face states (HLLCFluxStrategy::updateLeftRight,
// HLLCFluxStrategy.h:35-100) of faces [begin, end) from the last binary64
// residual's U, gradients and limiter, with k_face_flux's expressions:
// interior q = (grad q . (x_f - x_c)) * phi + U of that side; boundary faces
// take the face state U_edge on both sides.  out[(f - begin)] = 4 values.
__global__ void k_face_lr(int begin, int end, int right, const int2* __restrict__ lr, const d4* __restrict__ fg1,
                          const d4* __restrict__ U, const d4* __restrict__ grad, const d4* __restrict__ phi,
                          const d4* __restrict__ Ue, d4* __restrict__ out) {
    const int f = begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= end) return;
    const int2 e = lr[f];
    d4 o;
    if (e.y >= 0) {
        const int c = right ? e.y : e.x;
        const d4 d = ld4(fg1 + f);
        const double dx = right ? d.z : d.x, dy = right ? d.w : d.y;
        const d4 g0 = ld4(grad + 2 * (size_t)c), g1 = ld4(grad + 2 * (size_t)c + 1);
        const double gx[4] = {g0.x, g0.z, g1.x, g1.z}, gy[4] = {g0.y, g0.w, g1.y, g1.w};
        double u[4], p[4], q[4];
        to_arr(ld4(U + c), u);
        to_arr(ld4(phi + c), p);
        for (int j = 0; j < 4; j++) q[j] = dot2(gx[j], gy[j], dx, dy) * p[j] + u[j];
        o = d4{q[0], q[1], q[2], q[3]};
    } else {
        o = ld4(Ue + f);
    }
    out[f - begin] = o;
}
void launch_face_lr(const DevArrays& d, const LaunchCfg& L, int begin, int end, bool right, d4* out) {
    if (end <= begin) return;
    k_face_lr<<<nblk(end - begin, 256), 256, 0, L.stream>>>(begin, end, right ? 1 : 0, d.lr, d.fg1, d.U, d.grad,
                                                             d.phi, d.Ue, out);
    *L.counter += 1;
}

// 1/D for the fast form's sweep (binary64)
__global__ void k_inv_diag(int nc, const double* __restrict__ D, double* __restrict__ invD) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < nc) invD[c] = 1.0 / D[c];
}
void launch_inv_diag(const DevArrays& d, const LaunchCfg& L) {
    k_inv_diag<<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.diag, d.invD);
    *L.counter += 1;
}

// W += dW, U = prim(W)  (LUSGSIntegrator::UpdatePrimitiveVariable, LUSGS_Integrator.cpp:242-255)
__global__ void k_lusgs_update(int nc, const d4* __restrict__ dW, d4* __restrict__ W, d4* __restrict__ U,
                               float4* __restrict__ Uf, unsigned* __restrict__ err, const int* __restrict__ iblank) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    if (iblank && iblank[c] != 1) return;  // overset holes and receptors keep their state
    double w[4], dw[4], u[4];
    to_arr(ld4(W + c), w);
    to_arr(ld4(dW + c), dw);
#pragma unroll
    for (int k = 0; k < 4; k++) w[k] = w[k] + dw[k];
    prim_from_cons<double>(w, u);
    st4(W + c, d4{w[0], w[1], w[2], w[3]});
    st4(U + c, d4{u[0], u[1], u[2], u[3]});
    if (Uf) Uf[c] = make_float4((float)u[0], (float)u[1], (float)u[2], (float)u[3]);
    if (!(u[0] > 0.0) || !(u[1] > 0.0)) atomicOr(err, ERR_NONPHYS);
}
void launch_lusgs_update(const DevArrays& d, const LaunchCfg& L, bool fp32_copy) {
    k_lusgs_update<<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.dW, d.W, d.U, fp32_copy ? d.Uf : nullptr, d.err,
                                                          d.iblank_cell);
    *L.counter += 1;
}

// W = cons(U) (TopologyHolderStrategy::initializeConsData, .cpp:48-66)
__global__ void k_cons_from_prim(int begin, int end, const d4* __restrict__ U, d4* __restrict__ W) {
    int c = begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= end) return;
    double u[4], w[4];
    to_arr(ld4(U + c), u);
    cons_from_prim<double>(u, w);
    st4(W + c, d4{w[0], w[1], w[2], w[3]});
}
void launch_cons_from_prim(const DevArrays& d, const LaunchCfg& L, int begin, int end) {
    if (end <= begin) return;
    k_cons_from_prim<<<nblk(end - begin, 256), 256, 0, L.stream>>>(begin, end, d.U, d.W);
    *L.counter += 1;
}

// dt = CFL*vol/spec_c (Euler2D::SolveTime / ViscousFlow2D::SolveTime laminar branch)
template <class T>
__global__ void k_local_dt(int nc, const d4* __restrict__ cgeo, const T* __restrict__ specc, double cfl,
                           double* __restrict__ dt) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    dt[c] = cfl * cgeo[c].x / (double)specc[c];
}
void launch_local_dt(const DevArrays& d, const LaunchCfg& L, double cfl, int form) {
    if (form == 1) k_local_dt<float><<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.cgeo, d.speccf, cfl, d.dt);
    else if (form == 2) k_local_dt<ff><<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.cgeo, d.speccq, cfl, d.dt);
    else k_local_dt<double><<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.cgeo, d.specc, cfl, d.dt);
    *L.counter += 1;
}

}  // namespace cfdgb

namespace cfdgb {

// ---------------------------------------------------------------------------
// Projected wall distance, UnstructBlock2D::ComputeWallCellDistance
// (UnstructBlock.h:265-298): min over the mesh's wall faces of
// |(x_c - x_f) . n_f|, starting from 1e11.  A minimum is order-independent, so
// the brute-force scan (wall faces staged in shared memory) is exact.
__global__ void __launch_bounds__(256) k_wall_distance(int nc, const int* __restrict__ cmesh,
                                                       const d4* __restrict__ cgeo, const int* __restrict__ wall_ptr,
                                                       const int* __restrict__ wall_faces, const d4* __restrict__ fgeo,
                                                       const d2* __restrict__ fcen, double* __restrict__ walld) {
    __shared__ double sx[256], sy[256], snx[256], sny[256];
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    int m = c < nc ? cmesh[c] : 0;
    // all cells of a block belong to meshes in [m_lo, m_hi]; stage each mesh's wall list in turn
    int m_lo = cmesh[min(blockIdx.x * blockDim.x, nc - 1)];
    int m_hi = cmesh[min(blockIdx.x * blockDim.x + blockDim.x - 1, nc - 1)];
    double xc = 0, yc = 0;
    if (c < nc) {
        d4 g = cgeo[c];
        xc = g.y;
        yc = g.z;
    }
    double d = 100000000000.0;
    for (int mm = m_lo; mm <= m_hi; mm++) {
        int b = wall_ptr[mm], e = wall_ptr[mm + 1];
        for (int t0 = b; t0 < e; t0 += 256) {
            int t = t0 + threadIdx.x;
            __syncthreads();
            if (t < e) {
                int f = wall_faces[t];
                d2 xf = fcen[f];
                d4 g = fgeo[f];
                sx[threadIdx.x] = xf.x; sy[threadIdx.x] = xf.y; snx[threadIdx.x] = g.x; sny[threadIdx.x] = g.y;
            }
            __syncthreads();
            if (c < nc && m == mm) {
                int n = min(256, e - t0);
                for (int k = 0; k < n; k++) {
                    double x = xc - sx[k], y = yc - sy[k];
                    d = smin(d, fabs(dot2(x, y, snx[k], sny[k])));
                }
            }
        }
    }
    if (c < nc) walld[c] = d;
}

void launch_wall_distance(const DevArrays& d, const LaunchCfg& L) {
    k_wall_distance<<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.cmesh, d.cgeo, d.wall_ptr, d.wall_faces, d.fgeo,
                                                           d.fcen, d.walld);
    *L.counter += 1;
}

// ---------------------------------------------------------------------------
// Force on the walls of each mesh: sum over wall faces of the momentum flux the
// fluid sends through the face (convective minus viscous, the same terms that
// enter R[lC]); faces in ascending index within fixed 256-face chunks, chunks
// added in order, so the result is deterministic.  The reference integrates Cp
// only (Euler2D.cpp:392-618); lift and drag follow on the host.
template <class T, bool VISC>
__global__ void __launch_bounds__(256) k_wall_force(const int* __restrict__ wall_ptr, const int* __restrict__ wall_faces,
                                                    const int4* __restrict__ wblocks, const v4<T>* __restrict__ Fc,
                                                    const v4<T>* __restrict__ Fv, double* __restrict__ partial) {
    __shared__ double sxs[256], sys_[256];
    int4 b = wblocks[blockIdx.x];  // (mesh, begin, end) in wall_faces
    double fx = 0.0, fy = 0.0;
    int t = b.y + threadIdx.x;
    if (t < b.z) {
        int f = wall_faces[t];
        v4<T> c = ld4(Fc + f);
        fx = (double)c.z;
        fy = (double)c.w;
        if (VISC) {
            v4<T> v = ld4(Fv + f);
            fx = fx - (double)v.z;
            fy = fy - (double)v.w;
        }
    }
    sxs[threadIdx.x] = fx;
    sys_[threadIdx.x] = fy;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sxs[threadIdx.x] += sxs[threadIdx.x + s];
            sys_[threadIdx.x] += sys_[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = sxs[0];
        partial[2 * blockIdx.x + 1] = sys_[0];
    }
}

__global__ void k_wall_force_final(int nblk_total, const int4* __restrict__ wblocks, const double* __restrict__ partial,
                                   int nmesh, double* __restrict__ out) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmesh) return;
    double fx = 0.0, fy = 0.0;
    for (int i = 0; i < nblk_total; i++)
        if (wblocks[i].x == m) {
            fx += partial[2 * i];
            fy += partial[2 * i + 1];
        }
    out[2 * m] = fx;
    out[2 * m + 1] = fy;
}

void launch_wall_force(const DevArrays& d, const LaunchCfg& L, bool viscous, int form) {
    if (d.nwblk > 0) {
        if (form == 2) {
            if (viscous) k_wall_force<ff, true><<<d.nwblk, 256, 0, L.stream>>>(d.wall_ptr, d.wall_faces, d.wblocks, d.Fcq, d.Fvq, d.wpartial);
            else k_wall_force<ff, false><<<d.nwblk, 256, 0, L.stream>>>(d.wall_ptr, d.wall_faces, d.wblocks, d.Fcq, d.Fvq, d.wpartial);
        } else if (form == 1) {
            if (viscous) k_wall_force<float, true><<<d.nwblk, 256, 0, L.stream>>>(d.wall_ptr, d.wall_faces, d.wblocks, d.Fcf, d.Fvf, d.wpartial);
            else k_wall_force<float, false><<<d.nwblk, 256, 0, L.stream>>>(d.wall_ptr, d.wall_faces, d.wblocks, d.Fcf, d.Fvf, d.wpartial);
        } else {
            if (viscous) k_wall_force<double, true><<<d.nwblk, 256, 0, L.stream>>>(d.wall_ptr, d.wall_faces, d.wblocks, d.Fc, d.Fv, d.wpartial);
            else k_wall_force<double, false><<<d.nwblk, 256, 0, L.stream>>>(d.wall_ptr, d.wall_faces, d.wblocks, d.Fc, d.Fv, d.wpartial);
        }
        *L.counter += 1;
    }
    k_wall_force_final<<<nblk(d.nmesh, 128), 128, 0, L.stream>>>(d.nwblk, d.wblocks, d.wpartial, d.nmesh, d.wforce);
    *L.counter += 1;
}

}  // namespace cfdgb
