// Host-side mesh: .grd topology restated from the reference reader, plus the
// LU-SGS level schedule.  Geometry (areas, normals, centres) is computed on
// the device (geometry kernels), never here.
#pragma once
#include <string>
#include <vector>
#include <cstdint>

namespace cfdgb {

constexpr int kWall = -2;      // edge3d<2>::BoundaryType::WALL
constexpr int kFarfield = -3;  // edge3d<2>::BoundaryType::FARFIELD

struct HostMesh {
    int nnode = 0, nedge = 0, ncell = 0;
    std::vector<double> xy;          // 2*nnode
    std::vector<int> edge_nodes;     // 2*nedge, 0-based, file order of the two ends
    std::vector<int> lr;             // 2*nedge: left cell (0-based), right cell or kWall/kFarfield
    std::vector<int> cell_verts;     // 4*ncell, -1 padded (cell3d::pointInd order)
    std::vector<int> cell_nvert;     // ncell
    std::vector<int> cell_edges;     // 4*ncell, ascending edge index, -1 padded
    std::vector<int> cell_nedge;     // ncell
    // LU-SGS schedule: forward level of each cell counts the longest chain of
    // lower-indexed face neighbours; backward level the same on higher ones.
    std::vector<int> lev_fwd, lev_bwd;
    int n_lev_fwd = 0, n_lev_bwd = 0;
};

// Parse a 2D .grd file (throws std::runtime_error with a message).
HostMesh load_grd(const std::string& path, int wall_tag, int far_tag);
// Build from arrays in .grd order (1-based ids as in the file).
HostMesh mesh_from_arrays(int nnode, const double* xy, int nedge, const int* edge_nodes,
                          const int* edge_cells, int ncell, int wall_tag, int far_tag);
// Compute lev_fwd / lev_bwd (called by the builders).
void build_levels(HostMesh& m);

// Lets translation units other than the ABI's report through cfd_last_error().
int set_last_error(int code, const std::string& msg);

}  // namespace cfdgb

// The opaque cfd_mesh_t handle of the C ABI.
struct cfd_mesh_s {
    cfdgb::HostMesh m;
};
