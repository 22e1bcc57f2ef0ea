// The binary64 residual passes compiled with multiply-add contraction, for the
// mixed form: its binary64 residual defines the fixed point the binary32 sweep
// converges to, but need not reproduce the reference's operation-by-operation
// rounding as the plain form does (k_fp64.cu, -fmad=false), and a fused
// multiply-add is one FP64 instruction where a multiply and an add are two on a
// part whose binary64 pipe bounds these passes.
#include "case.hpp"
#include "fv_kernels.cuh"

namespace cfdgb {

static inline int nblk(int n, int bs) { return (n + bs - 1) / bs; }

template <bool V>
static void residual64c(const DevArrays& d, const LaunchCfg& L, int first_order, int which) {
    if (which < 0 || which == 0) {
        k_face_state<double, V, 1><<<nblk(d.nf, 256), 256, 0, L.stream>>>(d.nf, d.lr, d.fmesh, d.prm, d.fg0, d.U, d.Ue,
                                                                        d.fspec, d.mue, d.err,
                                                                        d.turb ? d.sstMut : nullptr,
                                                                        d.turb ? d.sstMutf : nullptr);
        *L.counter += 1;
    }
    if (which < 0 || which == 1) {
        k_cell_grad<double, V, 1><<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.cface, d.lr, d.cmesh, d.prm, d.cgeo,
                                                                       d.fg0, d.fg1, d.U, d.Ue, d.fspec, first_order,
                                                                       d.grad, d.phi, d.specc, d.specv, d.gradT, d.mu);
        *L.counter += 1;
    }
    if (which < 0 || which == 2) {
        k_face_flux<double, V, 1><<<nblk(d.nf, 256), 256, 0, L.stream>>>(d.nf, d.lr, d.fg0, d.fg1, d.fvis, d.U, d.grad,
                                                                       d.phi, d.Ue, d.mue, d.gradT, d.Fc, d.Fv, d.err,
                                                                       d.turb ? d.sstMutf : nullptr);
        *L.counter += 1;
    }
}
void launch_residual_fp64_contracted(const DevArrays& d, const LaunchCfg& L, bool viscous, int first_order, int which) {
    if (viscous) residual64c<true>(d, L, first_order, which);
    else residual64c<false>(d, L, first_order, which);
}


}  // namespace cfdgb
