// Compiles the reference-side adapter (include/cfdgb_adapter.hpp) against the
// reference's own headers and objects and checks, without a GPU, that the
// meshes it hands to libcfdgb.so have the reference's topology: the same edge
// cells, and every cell's edge list in the reference's cell3d order.  Built
// and run by tests/test_adapter_build.py (test infrastructure only).
//   usage: adapter_check MESH WALL_TAG FAR_TAG
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <vector>

#include "UnstructSolver/SolverWrapper.h"
#include "reader/UnstructReader.h"
#include "cfdgb_adapter.hpp"

int main(int argc, char** argv) {
    if (argc < 4) return 2;
    std::ofstream devnull("/dev/null");
    std::streambuf* saved = std::cout.rdbuf(devnull.rdbuf());
    UnstructReader* rd = new UnstructReader[1];
    rd->setOverSign(atoi(argv[3]));
    rd->setWallSign(atoi(argv[2]));
    rd->addFile(argv[1]);
    rd->setDim(2);
    rd->num_proc = 0;
    rd->cur_proc = 0;
    rd->readAll();
    WrapSolver ws;
    ws.setTopology(rd);
    double aoa = 2.0;
    ws.setParams("ViscousFlow2D", "LUSGS", "STABLE", 0, 0.0, 0.3, 1000.0, &aoa);
    ws.init(rd);
    std::cout.rdbuf(saved);
    UnstructTopologyHolder* h = ws.d_topology_holder;
    std::vector<cfd_mesh_t> ms = GpuIntegrator::meshes_from(h);
    int bad = 0;
    for (int m = 0; m < h->d_nmesh; m++) {
        auto& b = h->blk2D[m];
        int nn = 0, ne = 0, nc = 0;
        if (cfd_mesh_info(ms[m], &nn, &ne, &nc) != CFD_OK) return 3;
        if (nn != b.nPoints() || ne != b.nEdges() || nc != b.nCells()) bad++;
        std::vector<int> lr(2 * ne), ce(4 * nc), cv(4 * nc), cs(2 * nc);
        if (cfd_mesh_topology(ms[m], lr.data(), ce.data(), cv.data(), cs.data()) != CFD_OK) return 3;
        for (int k = 0; k < ne; k++) {
            auto& e = b.d_localEdges[k];
            int r = e.rCInd() >= 0 ? e.rCInd() : (e.rCInd() == -2 ? CFD_BC_WALL : CFD_BC_FARFIELD);
            if (lr[2 * k] != e.lCInd() || lr[2 * k + 1] != r) bad++;
        }
        for (int k = 0; k < nc; k++) {
            auto& c = b.d_localCells[k];
            if (cs[2 * k] != c.size() || cs[2 * k + 1] != c.edge_size()) bad++;
            for (int j = 0; j < c.edge_size(); j++)
                if (ce[4 * k + j] != c.edgeInd(j)) bad++;
            for (int j = 0; j < c.size(); j++)
                if (cv[4 * k + j] != c.pointInd(j)) bad++;
        }
        printf("{\"mesh\": %d, \"nodes\": %d, \"edges\": %d, \"cells\": %d, \"mismatches\": %d}\n", m, nn, ne, nc, bad);
    }
    for (cfd_mesh_t q : ms) cfd_mesh_free(q);
    return bad ? 1 : 0;
}
