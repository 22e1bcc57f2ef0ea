// The MIXFF form's residual: the residual passes instantiated on float-float
// pairs (ff_arith.h), with the gather summing in float-float and rounding each
// cell's residual to binary64 once.  The state, the update and the binary32
// sweep are the mixed form's; only the residual's arithmetic differs, so the
// form converges to the same discrete solution (to within the pairs' rounding
// floor near 1e-14 relative) at a fraction of the binary64 residual's cost on
// GB300's narrow binary64 pipe.
//
// Compiled with -fmad=false: the error-free transformations must see each
// binary32 product and sum rounded exactly as written; the fused multiply-adds
// they rely on are explicit.
#include "case.hpp"
#include "fv_kernels.cuh"

namespace cfdgb {

static inline int nblk(int n, int bs) { return (n + bs - 1) / bs; }

__global__ void k_to_q4(int n, const d4* __restrict__ a, q4* __restrict__ b) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const d4 v = ld4(a + i);
    st4(b + i, q4{ff(v.x), ff(v.y), ff(v.z), ff(v.w)});
}

void launch_to_ff(const DevArrays& d, const LaunchCfg& L, bool geometry) {
    if (geometry) {
        k_to_q4<<<nblk(d.nf, 256), 256, 0, L.stream>>>(d.nf, d.fg0, d.fg0q);
        k_to_q4<<<nblk(d.nf, 256), 256, 0, L.stream>>>(d.nf, d.fg1, d.fg1q);
        k_to_q4<<<nblk(d.nf, 256), 256, 0, L.stream>>>(d.nf, d.fvis, d.fvisq);
        k_to_q4<<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.cgeo, d.cgeoq);
        *L.counter += 4;
    }
    k_to_q4<<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.U, d.Uq);
    *L.counter += 1;
}

// which: -1 = all passes, 0 = face_state (with the state's float-float copy),
// 1 = cell_grad, 2 = face_flux
template <bool V>
static void residualq(const DevArrays& d, const LaunchCfg& L, int first_order, int which) {
    if (which < 0 || which == 0) {
        k_to_q4<<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.U, d.Uq);
        k_face_state<ff, V><<<nblk(d.nf, 256), 256, 0, L.stream>>>(d.nf, d.lr, d.fmesh, d.prm, d.fg0q, d.Uq, d.Ueq,
                                                                    d.fspecq, d.mueq, d.err,
                                                                    d.turb ? d.sstMut : nullptr,
                                                                    d.turb ? d.sstMutf : nullptr);
        *L.counter += 2;
    }
    if (which < 0 || which == 1) {
        k_cell_grad<ff, V><<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.cface, d.lr, d.cmesh, d.prm, d.cgeoq,
                                                                   d.fg0q, d.fg1q, d.Uq, d.Ueq, d.fspecq, first_order,
                                                                   d.gradq, d.phiq, d.speccq, d.specvq, d.gradTq,
                                                                   d.muq);
        *L.counter += 1;
    }
    if (which < 0 || which == 2) {
        k_face_flux<ff, V><<<nblk(d.nf, 256), 256, 0, L.stream>>>(d.nf, d.lr, d.fg0q, d.fg1q, d.fvisq, d.Uq, d.gradq,
                                                                   d.phiq, d.Ueq, d.mueq, d.gradTq, d.Fcq, d.Fvq,
                                                                   d.err, d.turb ? d.sstMutf : nullptr);
        *L.counter += 1;
    }
}
void launch_residual_ff(const DevArrays& d, const LaunchCfg& L, bool viscous, int first_order, int which) {
    if (viscous) residualq<true>(d, L, first_order, which);
    else residualq<false>(d, L, first_order, which);
}

template <bool V, int M>
static void updateq(const DevArrays& d, const LaunchCfg& L, double cfl, int stage, double alpha) {
    k_cell_update<ff, V, M><<<nblk(d.nc, 256), 256, 0, L.stream>>>(
        d.nc, d.cface, d.cgeo, d.Fcq, d.Fvq, d.speccq, d.specvq, cfl, stage, alpha, d.R, d.U, d.W, d.W0, d.dt,
        d.diag, (q4*)nullptr, d.cflmul, 0);
    *L.counter += 1;
}
void launch_update_ff(const DevArrays& d, const LaunchCfg& L, bool viscous, int mode, double cfl, int stage,
                      double alpha) {
    if (viscous) {
        if (mode == UPD_RESID) updateq<true, UPD_RESID>(d, L, cfl, stage, alpha);
        else if (mode == UPD_RK) updateq<true, UPD_RK>(d, L, cfl, stage, alpha);
        else updateq<true, UPD_LUSGS>(d, L, cfl, stage, alpha);
    } else {
        if (mode == UPD_RESID) updateq<false, UPD_RESID>(d, L, cfl, stage, alpha);
        else if (mode == UPD_RK) updateq<false, UPD_RK>(d, L, cfl, stage, alpha);
        else updateq<false, UPD_LUSGS>(d, L, cfl, stage, alpha);
    }
}

}  // namespace cfdgb
