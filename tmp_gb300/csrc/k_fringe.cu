// Case-level overset exchange: the per-iteration data update between the
// components of one case (tioga::dataUpdate, UniTioga/tioga.cpp:326-471, on
// node arrays registered by Orchestra::init, src/Orchestra.cpp:201-291).
//
// The reference exchanges node values: the solver's cell field is not
// registered with TIOGA directly.  Each step here:
//   1. the donor nodes (the vertices of every donor cell of the lists) get the
//      mean of their cells' primitive values, cells in ascending order;
//   2. every receptor node's values are interpolated from its donor cell's
//      nodes with the list's weights (getInterpolatedSolution: sum over the
//      nodes in list order from 0), all before any is written;
//   3. the values are written into the receptor nodes (updateSolnData);
//   4. every receptor cell (iblank_cell -1: all of its nodes are receptors)
//      takes the mean of its nodes (the node-to-cell mean of
//      Orchestra.cpp:270-291, vertices in cell order), and its conservative
//      state is formed from it.
// Hole cells (iblank_cell 0) keep their state: the LU-SGS update skips every
// cell that is not a field cell.
#include <cuda_runtime.h>

#include "case.hpp"

namespace cfdgb {
namespace {

inline unsigned nb(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

__global__ void k_fringe_node_mean(int n, const int* __restrict__ nodes, const int* __restrict__ ptr,
                                   const int* __restrict__ cells, const d4* __restrict__ U, double* __restrict__ qn) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    const int b = ptr[t], e = ptr[t + 1];
    for (int q = b; q < e; q++) {
        const d4 u = ld4(U + cells[q]);
        s[0] += u.x; s[1] += u.y; s[2] += u.z; s[3] += u.w;
    }
    const double cnt = (double)(e - b);
    const long long node = nodes[t];
    for (int k = 0; k < 4; k++) qn[node * 4 + k] = s[k] / cnt;
}

__global__ void k_fringe_gather(int n, const int* __restrict__ nw, const int* __restrict__ inode,
                                const double* __restrict__ w, const double* __restrict__ qn, double* __restrict__ vals) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= 4LL * n) return;
    const int i = (int)(t >> 2), k = (int)(t & 3);
    double qq = 0;
    for (int m = 0; m < 4; m++)
        if (m < nw[i]) qq += qn[(long long)inode[4 * i + m] * 4 + k] * w[4 * i + m];
    vals[t] = qq;
}

__global__ void k_fringe_scatter(int n, const int* __restrict__ recv, const double* __restrict__ vals,
                                 double* __restrict__ qn) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= 4LL * n) return;
    const int i = (int)(t >> 2), k = (int)(t & 3);
    qn[(long long)recv[i] * 4 + k] = vals[t];
}

__global__ void k_fringe_cells(int n, const int* __restrict__ rc, const int4* __restrict__ cv, const int* __restrict__ cnv,
                               const double* __restrict__ qn, d4* __restrict__ U, d4* __restrict__ W,
                               float4* __restrict__ Uf) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int c = rc[t];
    const int4 v = cv[c];
    const int vv[4] = {v.x, v.y, v.z, v.w};
    const int nv = cnv[c];
    double u[4];
    for (int k = 0; k < 4; k++) {
        double s = 0;
        for (int j = 0; j < nv; j++) s += qn[(long long)vv[j] * 4 + k];
        u[k] = s / nv;
    }
    double w[4];
    cons_from_prim<double>(u, w);
    st4(U + c, d4{u[0], u[1], u[2], u[3]});
    st4(W + c, d4{w[0], w[1], w[2], w[3]});
    if (Uf) Uf[c] = make_float4((float)u[0], (float)u[1], (float)u[2], (float)u[3]);
}

}  // namespace

void launch_fringe(const DevArrays& d, const FringePlan& f, const LaunchCfg& L) {
    if (f.nsrc > 0)
        k_fringe_node_mean<<<nb(f.nsrc, 256), 256, 0, L.stream>>>(f.nsrc, f.src_nodes, f.src_ptr, f.src_cells, d.U,
                                                                  f.qn);
    if (f.nrecv > 0) {
        k_fringe_gather<<<nb(4LL * f.nrecv, 256), 256, 0, L.stream>>>(f.nrecv, f.nw, f.inode, f.w, f.qn, f.vals);
        k_fringe_scatter<<<nb(4LL * f.nrecv, 256), 256, 0, L.stream>>>(f.nrecv, f.recv_node, f.vals, f.qn);
    }
    if (f.ncells > 0)
        k_fringe_cells<<<nb(f.ncells, 256), 256, 0, L.stream>>>(f.ncells, f.recv_cells, d.cverts, d.cnvert, f.qn, d.U,
                                                               d.W, d.resid32 ? d.Uf : nullptr);
    *L.counter += 4;
}

}  // namespace cfdgb
