// .grd reader and cell topology.
//
// The file layout and the way cells are assembled follow the reference reader
// (reader/UnstructReader.h:124-272): a 3-int header line, "nnode nedge ncell x x",
// nnode coordinate pairs, then per edge "count n0 n1 lC rC" with 1-based ids and a
// negative rC naming a boundary.  A cell's vertex list is assembled edge by edge
// in file order with the same rules as Brick4Cobalt2D::insert
// (UniTioga/CellBrick.cpp:13-136), so vertex order - and hence the summation
// order of the cell centre and the triangle split of the area - matches the
// reference.  A cell's edge list is in ascending edge index (cell3d::push_edge
// called in file order), which fixes the face order of every per-cell sum and of
// the LU-SGS sweeps.
#include "mesh.hpp"

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>

namespace cfdgb {
namespace {

// Incremental vertex assembly of one 2D cell from its edges.
struct CellBuilder {
    int nodes[4] = {-1, -1, -1, -1};
    int size = 0;
    bool closed = false;
    void insert(const int* e) {
        if (closed) return;
        if (size == 0) {
            nodes[0] = e[0];
            nodes[1] = e[1];
            size = 2;
            return;
        }
        int idx[8];
        int k = 0;
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 2; j++)
                if (nodes[i] == e[j]) { idx[k++] = i; idx[k++] = j; }
        if (k == 0) return;  // opposite side of a quadrilateral: nothing to place yet
        if (k == 2) {        // one shared vertex: place the other end next to it
            if (idx[0] < 2) nodes[3 - idx[0]] = e[1 - idx[1]];
            else nodes[5 - idx[0]] = e[1 - idx[1]];
            size += 1;
            if (size == 4) closed = true;
            return;
        }
        // both ends already present: the edge closes a triangle
        if (size == 3 && nodes[2] == -1 && nodes[3] != -1) {
            nodes[2] = nodes[3];
            nodes[3] = -1;
        }
        closed = true;
    }
};

struct Cursor {
    const char* p;
    const char* end;
    long next_long() {
        while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) p++;
        if (p >= end) throw std::runtime_error("unexpected end of .grd file");
        char* q;
        errno = 0;
        long v = strtol(p, &q, 10);
        if (q == p) throw std::runtime_error("malformed integer in .grd file");
        p = q;
        return v;
    }
    double next_double() {
        while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) p++;
        if (p >= end) throw std::runtime_error("unexpected end of .grd file");
        char* q;
        double v = strtod(p, &q);
        if (q == p) throw std::runtime_error("malformed number in .grd file");
        p = q;
        return v;
    }
};

HostMesh assemble(int nnode, std::vector<double>&& xy, int nedge, const std::vector<int>& counts,
                  const std::vector<int>& en, const std::vector<int>& ec, int ncell, int wall_tag,
                  int far_tag) {
    HostMesh m;
    m.nnode = nnode;
    m.nedge = nedge;
    m.ncell = ncell;
    m.xy = std::move(xy);
    m.edge_nodes.resize(2 * (size_t)nedge);
    m.lr.resize(2 * (size_t)nedge);
    m.cell_edges.assign(4 * (size_t)ncell, -1);
    m.cell_nedge.assign(ncell, 0);
    std::vector<CellBuilder> cb(ncell);
    for (int i = 0; i < nedge; i++) {
        if (counts[i] != 2) throw std::runtime_error("edge " + std::to_string(i) + " has " + std::to_string(counts[i]) + " nodes (2D edges need 2)");
        int n0 = en[2 * i], n1 = en[2 * i + 1];
        if (n0 < 1 || n0 > nnode || n1 < 1 || n1 > nnode) throw std::runtime_error("edge " + std::to_string(i) + " names a node out of range");
        int l = ec[2 * i], r = ec[2 * i + 1];
        if (l <= 0 || l > ncell) throw std::runtime_error("edge " + std::to_string(i) + ": left cell can't be negative or out of range");
        int e[2] = {n0, n1};
        cb[l - 1].insert(e);
        if (r > 0) {
            if (r > ncell) throw std::runtime_error("edge " + std::to_string(i) + ": right cell out of range");
            cb[r - 1].insert(e);
        }
        m.edge_nodes[2 * i] = n0 - 1;
        m.edge_nodes[2 * i + 1] = n1 - 1;
        m.lr[2 * i] = l - 1;
        auto push = [&](int c) {
            if (m.cell_nedge[c] >= 4) throw std::runtime_error("cell " + std::to_string(c) + " has more than 4 edges");
            m.cell_edges[4 * (size_t)c + m.cell_nedge[c]++] = i;
        };
        push(l - 1);
        if (r > 0) {
            m.lr[2 * i + 1] = r - 1;
            push(r - 1);
        } else if (r == wall_tag) {
            m.lr[2 * i + 1] = kWall;
        } else if (r == far_tag) {
            m.lr[2 * i + 1] = kFarfield;
        } else {
            throw std::runtime_error("edge " + std::to_string(i) + ": not a valid boundary type (" + std::to_string(r) + ")");
        }
    }
    m.cell_verts.assign(4 * (size_t)ncell, -1);
    m.cell_nvert.assign(ncell, 0);
    for (int c = 0; c < ncell; c++) {
        if (cb[c].size < 3) throw std::runtime_error("cell " + std::to_string(c) + " has fewer than 3 vertices");
        m.cell_nvert[c] = cb[c].size;
        for (int j = 0; j < cb[c].size; j++) m.cell_verts[4 * (size_t)c + j] = cb[c].nodes[j] - 1;
    }
    build_levels(m);
    return m;
}

}  // namespace

void build_levels(HostMesh& m) {
    m.lev_fwd.assign(m.ncell, 0);
    m.lev_bwd.assign(m.ncell, 0);
    int nf = 0, nb = 0;
    for (int c = 0; c < m.ncell; c++) {
        int lv = 0;
        for (int s = 0; s < m.cell_nedge[c]; s++) {
            int e = m.cell_edges[4 * (size_t)c + s];
            int l = m.lr[2 * e], r = m.lr[2 * e + 1];
            int j = (l == c) ? r : l;
            if (j >= 0 && j < c && m.lev_fwd[j] + 1 > lv) lv = m.lev_fwd[j] + 1;
        }
        m.lev_fwd[c] = lv;
        if (lv + 1 > nf) nf = lv + 1;
    }
    for (int c = m.ncell - 1; c >= 0; c--) {
        int lv = 0;
        for (int s = 0; s < m.cell_nedge[c]; s++) {
            int e = m.cell_edges[4 * (size_t)c + s];
            int l = m.lr[2 * e], r = m.lr[2 * e + 1];
            int j = (l == c) ? r : l;
            if (j > c && m.lev_bwd[j] + 1 > lv) lv = m.lev_bwd[j] + 1;
        }
        m.lev_bwd[c] = lv;
        if (lv + 1 > nb) nb = lv + 1;
    }
    m.n_lev_fwd = nf;
    m.n_lev_bwd = nb;
}

HostMesh load_grd(const std::string& path, int wall_tag, int far_tag) {
    FILE* fp = fopen(path.c_str(), "rb");
    if (!fp) throw std::runtime_error("Open file Failure: " + path);
    std::string buf;
    {
        char tmp[1 << 16];
        size_t n;
        while ((n = fread(tmp, 1, sizeof(tmp), fp)) > 0) buf.append(tmp, n);
        fclose(fp);
    }
    Cursor cur{buf.data(), buf.data() + buf.size()};
    cur.next_long();
    cur.next_long();
    cur.next_long();
    long nnode = cur.next_long(), nedge = cur.next_long(), ncell = cur.next_long();
    cur.next_long();
    cur.next_long();
    if (nnode <= 0 || nedge <= 0 || ncell <= 0 || nnode > (1L << 30) || nedge > (1L << 30) || ncell > (1L << 30))
        throw std::runtime_error("implausible .grd header sizes");
    std::vector<double> xy(2 * (size_t)nnode);
    for (size_t i = 0; i < xy.size(); i++) xy[i] = cur.next_double();
    std::vector<int> counts(nedge), en(2 * (size_t)nedge), ec(2 * (size_t)nedge);
    for (long i = 0; i < nedge; i++) {
        long cnt = cur.next_long();
        counts[i] = (int)cnt;
        if (cnt != 2) throw std::runtime_error("edge " + std::to_string(i) + " has " + std::to_string(cnt) + " nodes (2D edges need 2)");
        en[2 * i] = (int)cur.next_long();
        en[2 * i + 1] = (int)cur.next_long();
        ec[2 * i] = (int)cur.next_long();
        ec[2 * i + 1] = (int)cur.next_long();
    }
    return assemble((int)nnode, std::move(xy), (int)nedge, counts, en, ec, (int)ncell, wall_tag, far_tag);
}

HostMesh mesh_from_arrays(int nnode, const double* xy, int nedge, const int* edge_nodes,
                          const int* edge_cells, int ncell, int wall_tag, int far_tag) {
    if (nnode <= 0 || nedge <= 0 || ncell <= 0 || !xy || !edge_nodes || !edge_cells)
        throw std::runtime_error("mesh_from_arrays: empty mesh or null array");
    std::vector<double> v(xy, xy + 2 * (size_t)nnode);
    std::vector<int> counts(nedge, 2);
    std::vector<int> en(edge_nodes, edge_nodes + 2 * (size_t)nedge);
    std::vector<int> ec(edge_cells, edge_cells + 2 * (size_t)nedge);
    return assemble(nnode, std::move(v), nedge, counts, en, ec, ncell, wall_tag, far_tag);
}

}  // namespace cfdgb
