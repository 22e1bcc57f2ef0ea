// Test-oracle driver: links the reference solver's own serial path (compiled
// from its sources by oracle/build_ref.sh) and dumps per-phase arrays for
// parity checks.  This file is test infrastructure only; nothing in the
// product links or runs it.
//
// Usage:
//   ref_driver MESH WALL_TAG FAR_TAG FLOW ADVANCE MACH AOA RE CFL NSTEPS OUTDIR
//              [INIT_U.bin|-] [FIRST_ORDER]
//   FLOW    = euler | viscous          (Euler2D / ViscousFlow2D)
//   ADVANCE = rk5 | lusgs              (RungeKuttaStrategy(5) / LUSGSIntegrator)
//   environment WRITE_TECPLOT=1: also the reference's Tecplot field dumps (end of main)
//
// Setup follows WrapSolver::setParams/init (UnstructSolver/SolverWrapper.h:27-69):
// default-constructed strategy, set_fs_variable2(Ma, AoA, 1.225, 101325, Re),
// initializeStrategy, integrator initializeStrategy + initializeData.
// Stepping uses the serial entry points singleStepSerial / UpdateSerial.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <set>
#include <map>
#include <fstream>
#include <iostream>
#include <algorithm>
#include <memory>
#include <stdexcept>
#include <sys/stat.h>
#include <chrono>

// Give the driver read access to the strategies' internal arrays.
#define private public
#define protected public
#include "UnstructSolver/SolverWrapper.h"
#include "UnstructSolver/HLLCFluxStrategy.h"
#include "reader/UnstructReader.h"
#undef private
#undef protected

static std::string g_out;

static void dump(const char* name, const void* p, size_t bytes) {
    std::string f = g_out + "/" + name + ".bin";
    FILE* fp = fopen(f.c_str(), "wb");
    if (!fp) { perror(f.c_str()); exit(3); }
    fwrite(p, 1, bytes, fp);
    fclose(fp);
}

// A limiter that returns phi = 0 everywhere: the reference has no switch for
// first-order reconstruction, so the driver substitutes this strategy object
// (UL/UR then equal the cell values exactly: 0*delta + U = U).
class ZeroLimiter : public LimiterStrategy {
public:
    ZeroLimiter(UnstructTopologyHolder* h, TopologyHolderStrategy* s) : LimiterStrategy(h, s) {}
    void computeLimiter(double** UL, double** UR) override {
        for (int i = 0; i < d_nmesh; i++)
            for (int k = 0; k < d_hder->nEdges(i) * d_NEQU; k++) { UL[i][k] = 0; UR[i][k] = 0; }
    }
    double getLimiter(int, int, int) override { return 0.0; }
    void init() override {}
};

int main(int argc, char** argv) {
    if (argc < 12) {
        fprintf(stderr, "usage: %s MESH WALL FAR FLOW ADVANCE MACH AOA RE CFL NSTEPS OUTDIR [INIT_U|-] [FIRST_ORDER]\n", argv[0]);
        return 2;
    }
    std::string mesh = argv[1];
    int wall = atoi(argv[2]), far = atoi(argv[3]);
    std::string flow = argv[4], adv = argv[5];
    double ma = atof(argv[6]), aoa = atof(argv[7]), re = atof(argv[8]), cfl = atof(argv[9]);
    int nsteps = atoi(argv[10]);
    g_out = argv[11];
    std::string initU = argc > 12 ? argv[12] : "-";
    int first_order = argc > 13 ? atoi(argv[13]) : 0;
    mkdir(g_out.c_str(), 0755);

    // Silence the reference's chatty std::cout during setup and stepping.
    std::ofstream devnull("/dev/null");
    std::streambuf* saved = std::cout.rdbuf(devnull.rdbuf());

    UnstructReader* rd = new UnstructReader[1];
    rd->setOverSign(far);
    rd->setWallSign(wall);
    rd->addFile(mesh);
    rd->setDim(2);
    rd->num_proc = 0;  // arrange_communication with no partition maps
    rd->cur_proc = 0;
    rd->readAll();

    WrapSolver ws;
    ws.setTopology(rd);
    std::string flowT = flow == "euler" ? "Euler2D" : "ViscousFlow2D";
    std::string advT = adv == "rk5" ? "RungeKutta5" : "LUSGS";
    ws.setParams(flowT, advT, "STABLE", 0, 0.0, ma, re, &aoa);
    ws.init(rd);

    TopologyHolderStrategy* st = ws.d_flow_strategy;
    UnstructTopologyHolder* h = ws.d_topology_holder;
    auto& blk = h->blk2D[0];
    int nc = h->nCells(0), ne = h->nEdges(0), np = h->nPoints(0);

    HLLCFluxStrategy* hllc = nullptr;
    if (flow == "euler") hllc = (HLLCFluxStrategy*)((Euler2D*)st)->d_fluxComputer;
    else hllc = (HLLCFluxStrategy*)((ViscousFlow2D*)st)->d_cfluxComputer;
    if (first_order) hllc->d_limiter = new ZeroLimiter(h, st);

    LUSGSIntegrator* lu = adv == "lusgs" ? (LUSGSIntegrator*)ws.d_advance_strategy : nullptr;
    RungeKuttaStrategy* rk = adv == "rk5" ? (RungeKuttaStrategy*)ws.d_advance_strategy : nullptr;
    if (lu) lu->d_CFL_number = cfl;

    // Optional non-uniform initial primitive field (4*nc doubles, [rho,p,u,v] per cell).
    if (initU != "-") {
        std::vector<double> u(4 * (size_t)nc);
        FILE* fp = fopen(initU.c_str(), "rb");
        if (!fp || fread(u.data(), 8, u.size(), fp) != u.size()) { std::cout.rdbuf(saved); fprintf(stderr, "bad init file\n"); return 4; }
        fclose(fp);
        memcpy(st->getU()[0], u.data(), u.size() * 8);
        if (lu) st->initializeConsData(lu->W_scratch);
    }

    // Geometry and topology as the reference computed them.
    {
        std::vector<double> vol(nc), cen(2 * (size_t)nc), nrm(2 * (size_t)ne), area(ne), ecen(2 * (size_t)ne);
        std::vector<int> lr(2 * (size_t)ne), cedges(4 * (size_t)nc, -1), cverts(4 * (size_t)nc, -1), csize(2 * (size_t)nc);
        for (int k = 0; k < nc; k++) {
            auto& c = blk.d_localCells[k];
            vol[k] = c.volume();
            cen[2 * k] = c.center()[0]; cen[2 * k + 1] = c.center()[1];
            csize[2 * k] = c.size(); csize[2 * k + 1] = c.edge_size();
            for (int j = 0; j < c.edge_size(); j++) cedges[4 * k + j] = c.edgeInd(j);
            for (int j = 0; j < c.size(); j++) cverts[4 * k + j] = c.pointInd(j);
        }
        for (int k = 0; k < ne; k++) {
            auto& e = blk.d_localEdges[k];
            nrm[2 * k] = e.normal_vector()[0]; nrm[2 * k + 1] = e.normal_vector()[1];
            area[k] = e.area();
            ecen[2 * k] = e.center()[0]; ecen[2 * k + 1] = e.center()[1];
            lr[2 * k] = e.lCInd(); lr[2 * k + 1] = e.rCInd();
        }
        dump("geo_vol", vol.data(), vol.size() * 8);
        dump("geo_cen", cen.data(), cen.size() * 8);
        dump("geo_nrm", nrm.data(), nrm.size() * 8);
        dump("geo_area", area.data(), area.size() * 8);
        dump("geo_ecen", ecen.data(), ecen.size() * 8);
        dump("topo_lr", lr.data(), lr.size() * 4);
        dump("topo_cedges", cedges.data(), cedges.size() * 4);
        dump("topo_cverts", cverts.data(), cverts.size() * 4);
        dump("topo_csize", csize.data(), csize.size() * 4);
        dump("geo_wall", blk.wallCellDistance, (size_t)nc * 8);
        int dims[3] = {np, ne, nc};
        dump("dims", dims, sizeof(dims));
        double fs[8] = {st->fs_primVar[0], st->fs_primVar[1], st->fs_primVar[2], st->fs_primVar[3],
                        st->fsnd_soundSpeed, st->fs_Temperature, st->fs_mu, st->fs_Re};
        dump("freestream", fs, sizeof(fs));
    }

    // Phase dump: one residual evaluation from the initial state.
    st->preprocessAdvanceSerial(0);
    dump("res0_U", st->getU()[0], (size_t)nc * 32);
    dump("res0_R", st->getResidual()[0], (size_t)nc * 32);
    dump("res0_Uedge", st->getUEdge()[0], (size_t)ne * 32);
    dump("res0_grad", st->getGradientPrimitive()[0], (size_t)nc * 64);
    dump("res0_specc", st->getSpectrumConvective()[0], (size_t)nc * 8);
    dump("res0_UL", hllc->UL[0], (size_t)ne * 32);
    dump("res0_UR", hllc->UR[0], (size_t)ne * 32);
    {
        std::vector<double> phi(4 * (size_t)nc);
        for (int k = 0; k < nc; k++)
            for (int j = 0; j < 4; j++) phi[4 * k + j] = hllc->d_limiter->getLimiter(0, j, k);
        dump("res0_phi", phi.data(), phi.size() * 8);
    }
    if (flow == "viscous") {
        ViscousFlow2D* vf = (ViscousFlow2D*)st;
        dump("res0_gradT", vf->getGradientT()[0], (size_t)nc * 16);
        dump("res0_specv", vf->getSpectrumViscous()[0], (size_t)nc * 8);
        dump("res0_mu", vf->d_vfluxComputer->mu[0], (size_t)nc * 8);
        dump("res0_muedge", vf->d_vfluxComputer->mu_edge[0], (size_t)ne * 8);
    }
    st->SolveTime(lu ? cfl : 0.8);
    dump("res0_dt", st->getStableTime()[0], (size_t)nc * 8);

    // SST k-omega phase (environment SST_T = file of 2*nc doubles: per cell,
    // multipliers of the freestream k and omega; optional SST_MUT = nc
    // multipliers of the freestream mu_t).  The reference never runs
    // this model (ViscousFlow2D::preprocessAdvanceSerial skips it and
    // isLaminar() is true), so its functions are called here one by one on the
    // laminar residual's arrays.  Two set-up steps make them callable:
    //  * the model copied the flow's freestream when the flow was constructed,
    //    before WrapSolver::setParams set Mach/Re, so it is copied again;
    //  * FaceConvectiveTFlux / FaceViscousTFlux are allocated with 2*nCells
    //    entries but indexed by faces (SSTKWStrategy.h:556-557 vs :805-815,
    //    :907-913), so they are replaced by 2*nEdges arrays.
    if (const char* sp = getenv("SST_T")) {
        ViscousFlow2D* vf = (ViscousFlow2D*)st;
        auto* sst = vf->d_turbulentModel;
        sst->set_fs_variable(st);
        sst->FaceConvectiveTFlux[0] = new double[2 * (size_t)ne];
        sst->FaceViscousTFlux[0] = new double[2 * (size_t)ne];
        sst->InitializeturbulenceVariable();
        double inf[3] = {sst->fsnd_turbulenceValue[0], sst->fsnd_turbulenceValue[1], sst->fsnd_mut};
        dump("sst_inf", inf, sizeof(inf));
        std::vector<double> t(2 * (size_t)nc);
        FILE* fp = fopen(sp, "rb");
        if (!fp || fread(t.data(), 8, t.size(), fp) != t.size()) { std::cout.rdbuf(saved); fprintf(stderr, "bad SST_T\n"); return 4; }
        fclose(fp);
        for (int k = 0; k < nc; k++) {
            sst->turbulenceCellValue[0][2 * k] = inf[0] * t[2 * k];
            sst->turbulenceCellValue[0][2 * k + 1] = inf[1] * t[2 * k + 1];
        }
        if (const char* mp = getenv("SST_MUT")) {
            std::vector<double> m(nc);
            FILE* fm = fopen(mp, "rb");
            if (!fm || fread(m.data(), 8, nc, fm) != (size_t)nc) { std::cout.rdbuf(saved); fprintf(stderr, "bad SST_MUT\n"); return 4; }
            fclose(fm);
            for (int k = 0; k < nc; k++) sst->vCellMut[0][k] = inf[2] * m[k];
        }
        dump("sst_T_in", sst->turbulenceCellValue[0], (size_t)nc * 16);
        dump("sst_mut_in", sst->vCellMut[0], (size_t)nc * 8);
        sst->SolveTurbulenceEquation();
        dump("sst_tface", sst->turbulenceFaceValue[0], (size_t)ne * 16);
        dump("sst_tgrad", sst->turbulenceCellGrad[0], (size_t)nc * 32);
        dump("sst_f1", sst->cellF1[0], (size_t)nc * 8);
        dump("sst_f2", sst->cellF2[0], (size_t)nc * 8);
        dump("sst_mutf", sst->vFaceMut[0], (size_t)ne * 8);
        dump("sst_fconv", sst->FaceConvectiveTFlux[0], (size_t)ne * 16);
        dump("sst_fvisc", sst->FaceViscousTFlux[0], (size_t)ne * 16);
        dump("sst_R", sst->CellTotalTFlux[0], (size_t)nc * 16);
        std::vector<double> dg(2 * (size_t)nc);
        double* dgp = dg.data();
        sst->SolveDiag(&dgp);
        dump("sst_diag", dg.data(), dg.size() * 8);
        std::vector<double> w(2 * (size_t)nc);
        double* wp = w.data();
        sst->initializeConsData(&wp);
        sst->UpdatePrimitiveVariables(&wp);
        dump("sst_T2", sst->turbulenceCellValue[0], (size_t)nc * 16);
        dump("sst_mut", sst->vCellMut[0], (size_t)nc * 8);
    }

    // Full steps.  For LU-SGS the first step re-evaluates the same residual.
    std::vector<double> hist;
    auto t0 = std::chrono::steady_clock::now();
    for (int s = 0; s < nsteps; s++) {
        if (lu) {
            lu->singleStepSerial(s);
            double r = 0;
            for (int k = 0; k < nc; k++) r += lu->d_deltaW[0][4 * k] * lu->d_deltaW[0][4 * k];
            hist.push_back(r);
        } else {
            rk->singleStepSerial(s);
            double r = 0;
            for (int k = 0; k < nc; k++) r += std::abs<double>(st->getU()[0][4 * k] - rk->W_scratch[0][4 * k]);
            hist.push_back(r);
        }
    }
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (nsteps > 0) {
        dump("end_U", st->getU()[0], (size_t)nc * 32);
        dump("hist", hist.data(), hist.size() * 8);
        if (lu) {
            dump("end_D", lu->d_diagOperator[0], (size_t)nc * 32);
            dump("end_dW1", lu->d_deltaW1[0], (size_t)nc * 32);
            dump("end_dW", lu->d_deltaW[0], (size_t)nc * 32);
            dump("end_W", lu->W_scratch[0], (size_t)nc * 32);
            dump("end_R", st->getResidual()[0], (size_t)nc * 32);
            dump("end_dt", st->getStableTime()[0], (size_t)nc * 8);
        } else {
            dump("end_W0", rk->W_scratch[0], (size_t)nc * 32);
        }
    }
    // Field dumps in the reference's Tecplot layouts (environment WRITE_TECPLOT
    // set): TopologyHolderStrategy::writeCellData of the final cell state,
    // writeNOdeData of node data (node i, variable k: 0.001*i + k), and
    // writeTiogaFormat of cell data (cell c: c % 3 - 1), all into OUTDIR.
    if (getenv("WRITE_TECPLOT")) {
        st->writeCellData(g_out + "/cells", 0, 0, st->getU());
        std::vector<double> nodeq(4 * (size_t)np);
        for (int i = 0; i < np; i++)
            for (int k = 0; k < 4; k++) nodeq[4 * (size_t)i + k] = 0.001 * i + k;
        double* nq[1] = {nodeq.data()};
        st->writeNOdeData(g_out + "/nodes", 0, 0, nq);
        std::vector<int> ic(nc);
        for (int c = 0; c < nc; c++) ic[c] = c % 3 - 1;
        st->writeTiogaFormat(g_out + "/tioga", 0, 0, ic.data());
    }
    std::cout.rdbuf(saved);
    printf("{\"ncell\": %d, \"nedge\": %d, \"nsteps\": %d, \"seconds\": %.6f, \"cell_iters_per_s\": %.6e}\n",
           nc, ne, nsteps, secs, nsteps > 0 ? (double)nc * nsteps / secs : 0.0);
    return 0;
}
