/*
 * cfdgb_adapter.hpp - the reference-side binding of libcfdgb.so.
 *
 * A TimeIntegrator (UnstructSolver/TimeIntegrator.h:5-26) whose steps run on
 * the GPU through the C ABI of cfdgb.h, for a build of the reference solver
 * that wants to swap its CPU integrator for this library: WrapSolver::Loop
 * (UnstructSolver/SolverWrapper.h:71-90) keeps calling singleStep and
 * converged, and the strategy's U array is read and written through
 * pullU / pushU.  Include it after the reference's own headers
 * (UnstructSolver/TimeIntegrator.h and UnstructSolver/UnstructIntegrator.h).
 *
 * Mesh hand-over: every block's points and edges go to cfd_mesh_from_arrays in
 * the block's own order (edge nodes and cells 1-based, the boundary codes the
 * reader assigned: -2 wall, -3 far field), so cells, faces and the LU-SGS
 * order are the reference's.
 */
#ifndef CFDGB_ADAPTER_HPP
#define CFDGB_ADAPTER_HPP

#include <stdexcept>
#include <string>
#include <vector>

#include "cfdgb.h"

class GpuIntegrator : public TimeIntegrator {
public:
    // flow: "Euler2D" | "ViscousFlow2D" (WrapSolver::setParams' names); sst: the
    // ViscousFlow2D branch with the SST model coupled; adv: "LUSGS" | "RungeKutta5"
    GpuIntegrator(UnstructTopologyHolder* h, TopologyHolderStrategy* s, const std::string& flow,
                  const std::string& adv, double Ma, double Re, double aoa_deg, double cfl, int precision = CFD_PREC_FP64,
                  bool sst = false)
        : TimeIntegrator(h, s) {
        meshes_ = meshes_from(h);
        std::vector<cfd_freestream_t> fs(meshes_.size(), cfd_freestream_t{Ma, aoa_deg, Re, 1.225, 101325.0});
        cfd_params_t p{};
        p.flow = flow == "Euler2D" ? CFD_FLOW_EULER : (sst ? CFD_FLOW_SST : CFD_FLOW_LAMINAR);
        p.advance = adv == "LUSGS" ? CFD_ADV_LUSGS : CFD_ADV_RK5;
        p.precision = precision;
        p.cfl = cfl;
        check(cfd_case_create(meshes_.data(), (int)meshes_.size(), fs.data(), &p, nullptr, &case_));
        norm_ = p.advance == CFD_ADV_LUSGS ? CFD_NORM_DW_RHO2 : CFD_NORM_RK_DRHO;
    }
    // TimeIntegrator has no virtual destructor: own a GpuIntegrator through its
    // own type (or a std::unique_ptr<GpuIntegrator>), not a TimeIntegrator*.
    ~GpuIntegrator() {
        if (case_) cfd_case_free(case_);
        for (cfd_mesh_t m : meshes_) cfd_mesh_free(m);
    }
    GpuIntegrator(const GpuIntegrator&) = delete;
    GpuIntegrator& operator=(const GpuIntegrator&) = delete;

    // LUSGSIntegrator / RungeKuttaStrategy::initializeData: the uniform freestream
    void initializeData() override { check(cfd_init_freestream(case_)); }
    // one integrator step (singleStep), on the case's stream
    void singleStep(int) override { check(cfd_step(case_, 1)); }
    // the reference's converged() has no criterion (LUSGS_Integrator.cpp:163-168); this one
    // synchronises, reports device-side errors, keeps the norm of the last step
    // (postprocessUpdate's sum dW_rho^2, or RungeKuttaStrategy's sum |rho - rho0|)
    // and returns false so the loop runs its steps
    bool converged() override {
        check(cfd_residual_norm(case_, 0, norm_, &last_norm_));
        return false;
    }
    double last_norm() const { return last_norm_; }
    // the strategy's primitive field [NEQU*cell + eq] per mesh, both ways
    void pullU(double** U) {
        for (int m = 0; m < d_nmesh; m++) check(cfd_get_field(case_, m, CFD_FIELD_U, U[m]));
    }
    void pushU(double** U) {
        for (int m = 0; m < d_nmesh; m++) check(cfd_put_field(case_, m, CFD_FIELD_U, U[m]));
    }
    cfd_case_t handle() const { return case_; }

    // The library's mesh of every block of the holder (host only, no GPU):
    // points and edges in the block's own order; the caller frees them.
    static std::vector<cfd_mesh_t> meshes_from(UnstructTopologyHolder* h) {
        std::vector<cfd_mesh_t> out;
        for (int m = 0; m < h->d_nmesh; m++) {
            auto& b = h->blk2D[m];
            std::vector<double> xy;
            std::vector<int> en, ec;
            for (int p = 0; p < b.nPoints(); p++) {
                xy.push_back(b.d_localPoints[p][0]);
                xy.push_back(b.d_localPoints[p][1]);
            }
            for (int k = 0; k < b.nEdges(); k++) {
                auto& e = b.d_localEdges[k];
                en.push_back(e.pointInd(0) + 1);
                en.push_back(e.pointInd(1) + 1);
                ec.push_back(e.lCInd() + 1);
                ec.push_back(e.rCInd() >= 0 ? e.rCInd() + 1 : e.rCInd());
            }
            cfd_mesh_t mesh = nullptr;
            const int rc = cfd_mesh_from_arrays(b.nPoints(), xy.data(), b.nEdges(), en.data(), ec.data(), b.nCells(),
                                                CFD_BC_WALL, CFD_BC_FARFIELD, &mesh);
            if (rc != CFD_OK) {
                for (cfd_mesh_t q : out) cfd_mesh_free(q);
                check(rc);
            }
            out.push_back(mesh);
        }
        return out;
    }

private:
    static void check(int rc) {
        if (rc != CFD_OK) throw std::runtime_error(cfd_last_error());
    }
    std::vector<cfd_mesh_t> meshes_;
    cfd_case_t case_ = nullptr;
    int norm_ = CFD_NORM_DW_RHO2;
    double last_norm_ = 0.0;
};

#endif /* CFDGB_ADAPTER_HPP */
