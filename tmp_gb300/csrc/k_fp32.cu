// Binary32 instantiation of the residual kernels (the fast form): face states,
// gradients, limiter and fluxes in binary32 from a binary32 copy of U; the
// residual gather, local time step, RK update and LU-SGS diagonal stay in
// binary64 (k_cell_update widens every flux before summing).
#include "case.hpp"
#include "fv_kernels.cuh"

namespace cfdgb {

static inline int nblk(int n, int bs) { return (n + bs - 1) / bs; }

template <bool V>
static void residual32(const DevArrays& d, const LaunchCfg& L, int first_order, int which) {
    if (which < 0 || which == 0) {
        k_face_state<float, V><<<nblk(d.nf, 256), 256, 0, L.stream>>>(d.nf, d.lr, d.fmesh, d.prm, d.fg0f, d.Uf,
                                                                       d.Uef, d.fspecf, d.muef, d.err,
                                                                       (const double*)nullptr, (double*)nullptr);
        *L.counter += 1;
    }
    if (which < 0 || which == 1) {
        k_cell_grad<float, V><<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.cface, d.lr, d.cmesh, d.prm, d.cgeof,
                                                                      d.fg0f, d.fg1f, d.Uf, d.Uef, d.fspecf,
                                                                      first_order, d.gradf, d.phif, d.speccf,
                                                                      d.specvf, d.gradTf, d.muf);
        *L.counter += 1;
    }
    if (which < 0 || which == 2) {
        k_face_flux<float, V><<<nblk(d.nf, 256), 256, 0, L.stream>>>(d.nf, d.lr, d.fg0f, d.fg1f, d.fvisf, d.Uf,
                                                                      d.gradf, d.phif, d.Uef, d.muef, d.gradTf, d.Fcf,
                                                                      d.Fvf, d.err, (const double*)nullptr);
        *L.counter += 1;
    }
}
void launch_residual_fp32(const DevArrays& d, const LaunchCfg& L, bool viscous, int first_order, int which) {
    if (viscous) residual32<true>(d, L, first_order, which);
    else residual32<false>(d, L, first_order, which);
}

template <bool V, int M>
static void update32(const DevArrays& d, const LaunchCfg& L, double cfl, int stage, double alpha) {
    k_cell_update<float, V, M><<<nblk(d.nc, 256), 256, 0, L.stream>>>(
        d.nc, d.cface, d.cgeo, d.Fcf, d.Fvf, d.speccf, d.specvf, cfl, stage, alpha, d.R, d.U, d.W, d.W0, d.dt, d.diag,
        d.Uf, d.cflmul, 0);
    *L.counter += 1;
}
void launch_update_fp32(const DevArrays& d, const LaunchCfg& L, bool viscous, int mode, double cfl, int stage,
                        double alpha) {
    if (viscous) {
        if (mode == UPD_RESID) update32<true, UPD_RESID>(d, L, cfl, stage, alpha);
        else if (mode == UPD_RK) update32<true, UPD_RK>(d, L, cfl, stage, alpha);
        else update32<true, UPD_LUSGS>(d, L, cfl, stage, alpha);
    } else {
        if (mode == UPD_RESID) update32<false, UPD_RESID>(d, L, cfl, stage, alpha);
        else if (mode == UPD_RK) update32<false, UPD_RK>(d, L, cfl, stage, alpha);
        else update32<false, UPD_LUSGS>(d, L, cfl, stage, alpha);
    }
}

}  // namespace cfdgb
