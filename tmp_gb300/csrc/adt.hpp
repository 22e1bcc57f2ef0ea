// Host side of the donor search's tree order (MeshBlock::search,
// UniTioga/search.cpp:81-270).  The reference walks an alternating digital
// tree over the boxes of the cells near the query points and takes the first
// containing cell of its walk; the device search reproduces that choice from
// each cell's place in the walk order.  These functions build that order and
// the coincident-point hash the search applies before it.
#pragma once

#include <cmath>
#include <vector>

#if defined(__CUDACC__)
#define CFDGB_HD __host__ __device__
#else
#define CFDGB_HD
#endif

namespace cfdgb {
namespace adt {

// Oriented box of a point set (findOBB, UniTioga/utils.cpp:43-291, with
// Kaiser's Jacobi eigen-solver, mathTools/kaiser.cpp:9-160): centre xc, half
// extents dxc and basis rows vec, in the reference's arithmetic order.
struct Obb {
    double xc[2], dxc[2], vec[2][2];
};
Obb find_obb(const double* xy, long long n);

// Whether a cell goes into the tree (search.cpp:116-156): its vertices'
// box in the oriented box's frame overlaps that box.  x[2*m], x[2*m+1]: the
// cell's nv vertices in order.  Host and device evaluate it alike.
CFDGB_HD inline bool crosses(const Obb& o, int nv, const double* x) {
    double mn[2] = {1.0e15, 1.0e15}, mx[2] = {-1.0e15, -1.0e15};
    for (int m = 0; m < nv; m++)
        for (int j = 0; j < 2; j++) {
            double d = 0;
            for (int k = 0; k < 2; k++) d += (x[2 * m + k] - o.xc[k]) * o.vec[j][k];
            mn[j] = mn[j] < d ? mn[j] : d;
            mx[j] = mx[j] > d ? mx[j] : d;
        }
    bool hit = true;
    for (int j = 0; j < 2; j++) {
        const double ctr = (mx[j] + mn[j]) * 0.5, half = (mx[j] - mn[j]) * 0.5;
        hit = hit && (fabs(ctr) <= half + o.dxc[j]);
    }
    return hit;
}

// Preorder node of every element in the tree ADT::buildADT makes over nelem
// boxes (box[4*e..] = min x, min y, max x, max y; ADT.cpp:15-91,
// buildADTrecursion, recursiveADT.cpp:8-109, median split of
// mathTools/median.cpp).  The walk of searchIntersections visits nodes in
// this order, so the first containing cell it meets has the lowest node.
std::vector<int> node_order(int nelem, const double* box);

// Preorder number of every cell in the tree (-1: not in it): the crossing
// cells pushed on search.cpp's LIFO list (the last MeshBlock number first),
// their axis-aligned boxes (search.cpp:166-205), then node_order.
// cv[4*c ..]: the vertices of mesh cell c, cv[4*c+3] < 0 for a triangle;
// order[p]: the mesh cell of MeshBlock cell p; cross[c]: crosses() of cell c.
std::vector<int> tree_ranks(int ncell, const double* xy, const int* cv, const int* order, const unsigned char* cross);

// uniquenodes_octree (utils.cpp:484-643): points closer than TOL in L1 with
// the same tag share one search; xtag[i] is the point whose search point i
// takes (xtag[i] <= i; follow it to a fixed point), res[] is merged in place
// (the larger resolution of each coincident pair, kept at the smaller index).
void coincident(long long n, const double* xy, const int* tag, double* res, int* xtag);

}  // namespace adt
}  // namespace cfdgb
