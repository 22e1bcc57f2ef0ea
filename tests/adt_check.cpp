// CPU harness for the host half of the donor search's tree order
// (tmp_gb300/csrc/adt.cpp, compiled in with g++): for a mesh and a query point
// set it prints each cell's preorder number in the search tree (-1: not in the
// tree), each point's coincident-point tag and the merged resolutions.
//   adt_check IN OUT
//   IN:  int32 nnode, ncell; double xy[2*nnode]; int32 nvert[ncell];
//        int32 verts[4*ncell] (0-based); int32 n; double pts[2*n]; int32 tags[n]; double res[n]
//   OUT: int32 rank[ncell]; int32 xtag[n]; double res[n]
#include <cstdio>
#include <vector>

#include "adt.hpp"

template <class T>
static bool rd(FILE* f, T* p, size_t n) {
    return fread(p, sizeof(T), n, f) == n;
}

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 3;
    int nnode, ncell, n;
    if (!rd(f, &nnode, 1) || !rd(f, &ncell, 1)) return 3;
    std::vector<double> xy(2 * (size_t)nnode);
    std::vector<int> nvert(ncell), verts(4 * (size_t)ncell);
    if (!rd(f, xy.data(), xy.size()) || !rd(f, nvert.data(), ncell) || !rd(f, verts.data(), verts.size())) return 3;
    if (!rd(f, &n, 1)) return 3;
    std::vector<double> pts(2 * (size_t)n), res(n);
    std::vector<int> tags(n), xtag(n);
    if (!rd(f, pts.data(), pts.size()) || !rd(f, tags.data(), n) || !rd(f, res.data(), n)) return 3;
    fclose(f);
    std::vector<int> cv(4 * (size_t)ncell), order;
    for (int c = 0; c < ncell; c++)
        for (int m = 0; m < 4; m++) cv[4 * c + m] = m < nvert[c] ? verts[4 * c + m] : -1;
    for (int pass = 0; pass < 2; pass++)
        for (int c = 0; c < ncell; c++)
            if ((nvert[c] == 3) == (pass == 0)) order.push_back(c);
    const cfdgb::adt::Obb o = cfdgb::adt::find_obb(pts.data(), n);
    std::vector<unsigned char> cross(ncell);
    for (int c = 0; c < ncell; c++) {
        double x[8];
        for (int m = 0; m < nvert[c]; m++) x[2 * m] = xy[2 * cv[4 * c + m]], x[2 * m + 1] = xy[2 * cv[4 * c + m] + 1];
        cross[c] = cfdgb::adt::crosses(o, nvert[c], x);
    }
    const std::vector<int> rank = cfdgb::adt::tree_ranks(ncell, xy.data(), cv.data(), order.data(), cross.data());
    cfdgb::adt::coincident(n, pts.data(), tags.data(), res.data(), xtag.data());
    FILE* g = fopen(argv[2], "wb");
    if (!g) return 4;
    fwrite(rank.data(), 4, rank.size(), g);
    fwrite(xtag.data(), 4, xtag.size(), g);
    fwrite(res.data(), 8, res.size(), g);
    fclose(g);
    return 0;
}
