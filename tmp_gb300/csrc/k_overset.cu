// Overset connectivity and fringe exchange on the device: interpolation
// weights, donor search and the fringe data update of UniTioga's MeshBlock
// (mathTools/math.cpp, UniTioga/search.cpp, checkContainment.cpp,
// dataUpdate.cpp), plus the node-to-cell mean of Orchestra.cpp, and the C ABI
// entry points for them.
//
// This unit is compiled with -fmad=false: every a*b+c is rounded twice, as in
// the reference's compiled code, so the weights are bit-identical to
// computeNodalWeight2D's.
//
// Donor search.  The reference (MeshBlock::search, search.cpp:81-270) puts
// the cells whose boxes cross the oriented box of the query points in an
// alternating digital tree and walks it per point; the walk checks, in the
// tree's preorder, every cell whose TOL-widened box holds the point
// (recursiveADT.cpp:111-156) and stops at the first that contains it
// (checkContainment.cpp:4-62: every weight in [-TOL, 1 + TOL]) unless that
// cell may not donate (cellRes = BIGVALUE) and one of its weights vanishes;
// without such a stop the last check of the walk decides.  So the donor is
// fixed by each candidate cell's preorder number alone: the host builds the
// tree's order (adt.cpp) and the device evaluates the choice per point.
// The donor block keeps a uniform grid of bins over its bounding box; each
// cell is listed in every bin its TOL-widened bounding box touches (a radix
// sort of (bin, cell) keys makes the lists).  A query thread tests every cell
// of its bin that is in the tree and keeps the contained, acceptable one of
// lowest preorder number, else the outcome of the highest-numbered check.
// Coincident query points (uniquenodes_octree) take the donor cell of the
// first of them, with their own weights in it.
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <exception>
#include <new>
#include <stdexcept>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "../../include/cfdgb.h"
#include "adt.hpp"
#include "mesh.hpp"

namespace {

constexpr double kTol = 1.0e-10;  // TOL, UniTioga/codetypes.h:54
constexpr int kNewtonMax = 500;   // newtonSolve2D itmax, math.cpp:131

struct OversetError : std::runtime_error {
    int code;
    OversetError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw OversetError(CFD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T>
void dalloc(T** p, size_t n) {
    ck(cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T)), "cudaMalloc");
}

template <class T>
void dfree(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}

// ---------------------------------------------------------------------------
// Weights (mathTools/math.cpp)
// ---------------------------------------------------------------------------

// solvec (math.cpp:4-60) for a 2x2 system: Gaussian elimination in which a
// pivot below 1e-8 in magnitude is exchanged with the next row's, then back
// substitution.  Returns false where the reference sets iflag = 0.
__device__ __forceinline__ bool solvec2(double& a00, double& a01, double& a10, double& a11, double& b0,
                                        double& b1) {
    const double eps = 1e-8;
    if (fabs(a00) < eps) {
        if (fabs(a10) < eps) return false;
        double t;
        t = a10; a10 = a00; a00 = t;
        t = a11; a11 = a01; a01 = t;
        t = b1; b1 = b0; b0 = t;
    }
    const double fact = -a10 / a00;
    a10 += fact * a00;
    a11 += fact * a01;
    b1 += fact * b0;
    if (fabs(a11) < eps) return false;
    double sum = 0;
    b1 = (b1 - sum) / a11;
    sum = 0;
    sum += a01 * b1;
    b0 = (b0 - sum) / a00;
    return true;
}

// Bilinear parameters (u, v) of the point by Newton's method from (0.5, 0.5)
// (newtonSolve2D, math.cpp:126-187).  f[term][coord] as in the reference:
// f0 = v1 - p, f1 = v2 - v1, f2 = v4 - v1, f3 = v1 - v2 + v3 - v4.
__device__ __forceinline__ void newton2(const double f[4][2], double& u_out, double& v_out) {
    double u = 0.5, v = 0.5;
    bool ok = true;
    int iter;
    for (iter = 0; iter < kNewtonMax; iter++) {
        const double uv = u * v;
        double r0 = f[0][0] + f[1][0] * u + f[2][0] * v + f[3][0] * uv;
        double r1 = f[0][1] + f[1][1] * u + f[2][1] * v + f[3][1] * uv;
        const double norm = r0 * r0 + r1 * r1;
        if (sqrt(norm) <= 1e-14) break;
        double l00 = f[1][0] + f[3][0] * v, l01 = f[2][0] + f[3][0] * u;
        double l10 = f[1][1] + f[3][1] * v, l11 = f[2][1] + f[3][1] * u;
        if (!solvec2(l00, l01, l10, l11, r0, r1)) {
            ok = false;
            break;
        }
        u -= r0 * 1.0;
        v -= r1 * 1.0;
    }
    if (iter == kNewtonMax || !ok) {
        u = 2.0;
        v = 0.0;
    }
    u_out = u;
    v_out = v;
}

// computeNodalWeight2D (math.cpp:229-312).  x[2*m], y = x[2*m+1] for the cell's
// vertices in its own order; frac[m] receives the weights in that order.
// Returns false for a triangle whose system is singular (the reference throws).
__device__ bool nodal_weights(int nvert, const double x[8], double px, double py, double frac[4]) {
    frac[0] = frac[1] = frac[2] = frac[3] = 0.0;
    if (nvert == 3) {
        double a00 = x[0] - x[4], a01 = x[2] - x[4];
        double a10 = x[1] - x[5], a11 = x[3] - x[5];
        double b0 = px - x[4], b1 = py - x[5];
        if (!solvec2(a00, a01, a10, a11, b0, b1)) return false;
        frac[0] = b0;
        frac[1] = b1;
        frac[2] = 1. - frac[0] - frac[1];
        return true;
    }
    // findClockWise (math.cpp:190-227): which pair of vertices is the diagonal,
    // from the signs of the z components of AB x AC, AB x AD and AC x AD.
    const double abx = x[2] - x[0], aby = x[3] - x[1];
    const double acx = x[4] - x[0], acy = x[5] - x[1];
    const double adx = x[6] - x[0], ady = x[7] - x[1];
    const double z_abac = abx * acy - aby * acx;
    const double z_abad = abx * ady - aby * adx;
    int m0 = 0, m1 = 1, m2 = 2, m3 = 3;
    if (z_abac * z_abad > 0) {
        const double z_acad = acx * ady - acy * adx;
        if (!(z_acad * z_abad > 0)) {
            m2 = 3;
            m3 = 2;
        }
    } else {
        m1 = 2;
        m2 = 1;
    }
    double f[4][2];
    const double p[2] = {px, py};
    for (int i = 0; i < 2; i++) {
        const double x0 = x[2 * m0 + i], x1 = x[2 * m1 + i], x2 = x[2 * m2 + i], x3 = x[2 * m3 + i];
        f[0][i] = x0 - p[i];
        f[1][i] = x1 - x0;
        f[2][i] = x3 - x0;
        f[3][i] = x0 - x1 + x2 - x3;
    }
    double u, v;
    newton2(f, u, v);
    const double w0 = (1 - u) * (1 - v), w1 = u * (1 - v), w2 = u * v, w3 = (1 - u) * v;
    // scatter through the mapping without a dynamically indexed local array
    frac[0] = m0 == 0 ? w0 : 0.0;  // m0 is always 0
    frac[1] = m1 == 1 ? w1 : (m2 == 1 ? w2 : 0.0);
    frac[2] = m2 == 2 ? w2 : (m1 == 2 ? w1 : (m3 == 2 ? w3 : 0.0));
    frac[3] = m3 == 3 ? w3 : (m2 == 3 ? w2 : 0.0);
    return true;
}

__device__ __forceinline__ bool inside_weights(int nvert, const double frac[4]) {
    for (int m = 0; m < 4; m++) {
        if (m < nvert && (frac[m] + kTol) * (frac[m] - 1.0 - kTol) > 0) return false;
    }
    return true;
}

__global__ void k_nodal_weights(long long n, const int* __restrict__ nvert, const double* __restrict__ xv,
                                const double* __restrict__ xp, double* __restrict__ frac, int* err) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x[8];
    for (int k = 0; k < 8; k++) x[k] = xv[8 * i + k];
    double f[4];
    const int nv = nvert[i];
    if (nv != 3 && nv != 4) {
        atomicOr(err, 2);
        for (int k = 0; k < 4; k++) frac[4 * i + k] = 0.0;
        return;
    }
    if (!nodal_weights(nv, x, xp[2 * i], xp[2 * i + 1], f)) atomicOr(err, 1);
    for (int k = 0; k < 4; k++) frac[4 * i + k] = f[k];
}

// ---------------------------------------------------------------------------
// Search bins
// ---------------------------------------------------------------------------

struct BinGrid {
    double x0, y0, inv_hx, inv_hy;
    int nbx, nby;
};

__device__ __forceinline__ int bin_coord(double x, double x0, double inv_h, int nb) {
    double d = floor((x - x0) * inv_h);
    if (!(d >= 0.0)) d = 0.0;
    if (d > nb - 1) d = nb - 1;
    return (int)d;
}

// Per cell: float prefilter box (the TOL-widened box rounded outwards), the
// range of bins that box touches and their number.
__global__ void k_cell_boxes(int ncell, const double* __restrict__ xy, const int4* __restrict__ cv, BinGrid g,
                             float4* __restrict__ fbox, int4* __restrict__ brange, long long* __restrict__ count) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int4 v = cv[c];
    const int nv = v.w < 0 ? 3 : 4;
    const int id[4] = {v.x, v.y, v.z, v.w};
    double xmin = 1.0e15, ymin = 1.0e15, xmax = -1.0e15, ymax = -1.0e15;  // BIGVALUE
    for (int m = 0; m < 4; m++) {
        if (m < nv) {
            const double px = xy[2 * id[m]], py = xy[2 * id[m] + 1];
            xmin = xmin < px ? xmin : px;
            ymin = ymin < py ? ymin : py;
            xmax = xmax > px ? xmax : px;
            ymax = ymax > py ? ymax : py;
        }
    }
    const double lx = xmin - kTol, ly = ymin - kTol, hx = xmax + kTol, hy = ymax + kTol;
    fbox[c] = make_float4(__double2float_rd(lx), __double2float_rd(ly), __double2float_ru(hx),
                          __double2float_ru(hy));
    const int ix0 = bin_coord(lx, g.x0, g.inv_hx, g.nbx), ix1 = bin_coord(hx, g.x0, g.inv_hx, g.nbx);
    const int iy0 = bin_coord(ly, g.y0, g.inv_hy, g.nby), iy1 = bin_coord(hy, g.y0, g.inv_hy, g.nby);
    brange[c] = make_int4(ix0, iy0, ix1, iy1);
    count[c] = (long long)(ix1 - ix0 + 1) * (iy1 - iy0 + 1);
}

__global__ void k_emit_keys(int ncell, const int4* __restrict__ brange, const long long* __restrict__ offs, int nbx,
                            unsigned long long* __restrict__ keys) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int4 r = brange[c];
    long long o = offs[c];
    for (int iy = r.y; iy <= r.w; iy++)
        for (int ix = r.x; ix <= r.z; ix++) {
            const unsigned long long b = (unsigned long long)iy * nbx + ix;
            keys[o++] = (b << 32) | (unsigned)c;
        }
}

// binptr[b] = first entry of bin b (lower bound of b << 32 in the sorted keys);
// also peels the cell number off every key.
__global__ void k_bin_ptr(long long nbins, long long nent, const unsigned long long* __restrict__ keys,
                          int* __restrict__ binptr, int* __restrict__ cells) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < nent) cells[t] = (int)(keys[t] & 0xffffffffull);
    if (t > nbins) return;
    const unsigned long long key = (unsigned long long)t << 32;
    long long lo = 0, hi = nent;
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (keys[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    binptr[t] = (int)lo;
}

// Cells whose box in the frame of the query points' oriented box overlaps that
// box: the cells the reference puts in its tree.
__global__ void k_obb_cross(int ncell, const double* __restrict__ xy, const int4* __restrict__ cv, cfdgb::adt::Obb o,
                            unsigned char* __restrict__ cross, int* __restrict__ rank0) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int4 v = cv[c];
    const int nv = v.w < 0 ? 3 : 4;
    const int id[4] = {v.x, v.y, v.z, v.w};
    double x[8];
    for (int m = 0; m < 4; m++)
        if (m < nv) x[2 * m] = xy[2 * id[m]], x[2 * m + 1] = xy[2 * id[m] + 1];
    const bool hit = cfdgb::adt::crosses(o, nv, x);
    cross[c] = hit ? 1 : 0;
    rank0[c] = hit ? 0 : -1;  // one rank for every tree cell until the tree's order is needed
}

__device__ __forceinline__ void cell_coords(const double* __restrict__ xy, int4 v, double x[8]) {
    x[0] = xy[2 * v.x]; x[1] = xy[2 * v.x + 1];
    x[2] = xy[2 * v.y]; x[3] = xy[2 * v.y + 1];
    x[4] = xy[2 * v.z]; x[5] = xy[2 * v.z + 1];
    if (v.w >= 0) {
        x[6] = xy[2 * v.w]; x[7] = xy[2 * v.w + 1];
    } else {
        x[6] = x[4]; x[7] = x[5];
    }
}

__device__ __forceinline__ void put_donor(long long i, int cell, int4 v, const double f[4], int* __restrict__ donor,
                                          int* __restrict__ dnodes, double* __restrict__ w) {
    donor[i] = cell;
    if (dnodes) {
        dnodes[4 * i] = cell >= 0 ? v.x : -1;
        dnodes[4 * i + 1] = cell >= 0 ? v.y : -1;
        dnodes[4 * i + 2] = cell >= 0 ? v.z : -1;
        dnodes[4 * i + 3] = cell >= 0 ? v.w : -1;
    }
    if (w)
        for (int m = 0; m < 4; m++) w[4 * i + m] = cell >= 0 ? f[m] : 0.0;
}

// rank[c]: the cell's preorder number in the search tree, -1 if not in it;
// unacc[c] (may be null): the cell may not donate (cellRes = BIGVALUE).
__global__ void k_donor_search(long long n, const double* __restrict__ pts, const double* __restrict__ xy,
                               const int4* __restrict__ cv, const float4* __restrict__ fbox,
                               const int* __restrict__ binptr, const int* __restrict__ cells, BinGrid g,
                               const int* __restrict__ rank, const unsigned char* __restrict__ unacc,
                               int* __restrict__ donor, int* __restrict__ dnodes, double* __restrict__ w, int* err,
                               int* ambiguous) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double px = pts[2 * i], py = pts[2 * i + 1];
    const float pxu = __double2float_ru(px), pxd = __double2float_rd(px);
    const float pyu = __double2float_ru(py), pyd = __double2float_rd(py);
    const int b = bin_coord(py, g.y0, g.inv_hy, g.nby) * g.nbx + bin_coord(px, g.x0, g.inv_hx, g.nbx);
    int good = -1, good_rank = INT_MAX;  // contained and acceptable, lowest preorder number
    int last = -1, last_rank = -1;       // the highest-numbered check and its outcome
    int ngood = 0, nrefused = 0;         // contained cells that stop the walk / that do not
    int4 good_v = make_int4(-1, -1, -1, -1), last_v = good_v;
    double good_w[4] = {0.0, 0.0, 0.0, 0.0}, last_w[4] = {0.0, 0.0, 0.0, 0.0};
    const int e1 = binptr[b + 1];
    for (int e = binptr[b]; e < e1; e++) {
        const int c = cells[e];
        const int r = rank[c];
        if (r < 0) continue;
        const float4 fb = fbox[c];
        if (pxu < fb.x || pyu < fb.y || pxd > fb.z || pyd > fb.w) continue;
        const int4 v = cv[c];
        const int nv = v.w < 0 ? 3 : 4;
        double x[8];
        cell_coords(xy, v, x);
        double xmin = 1.0e15, ymin = 1.0e15, xmax = -1.0e15, ymax = -1.0e15;
        for (int m = 0; m < 4; m++) {
            if (m < nv) {
                xmin = xmin < x[2 * m] ? xmin : x[2 * m];
                ymin = ymin < x[2 * m + 1] ? ymin : x[2 * m + 1];
                xmax = xmax > x[2 * m] ? xmax : x[2 * m];
                ymax = ymax > x[2 * m + 1] ? ymax : x[2 * m + 1];
            }
        }
        if (!(px >= xmin - kTol && py >= ymin - kTol && px <= xmax + kTol && py <= ymax + kTol)) continue;
        double f[4];
        bool in = nodal_weights(nv, x, px, py, f);
        if (!in) atomicOr(err, 1);  // the reference throws here
        in = in && inside_weights(nv, f);
        bool refused = false;
        if (in && unacc && unacc[c])
            for (int m = 0; m < 4; m++) refused = refused || (m < nv && fabs(f[m]) < kTol);
        ngood += in && !refused;
        nrefused += in && refused;
        if (in && !refused && r < good_rank) {
            good = c, good_rank = r, good_v = v;
            for (int m = 0; m < 4; m++) good_w[m] = f[m];
        }
        if (r > last_rank) {
            last_rank = r;
            last = in ? c : -1;
            last_v = v;
            for (int m = 0; m < 4; m++) last_w[m] = f[m];
        }
    }
    if (good >= 0) put_donor(i, good, good_v, good_w, donor, dnodes, w);
    else put_donor(i, last, last_v, last_w, donor, dnodes, w);
    // the choice depends on the tree's order only where several cells stop the walk, or none does and a
    // refused cell contains the point
    if (ambiguous && (ngood > 1 || (ngood == 0 && nrefused > 0))) atomicOr(ambiguous, 1);
}

// Coincident query points, screened on the device.  The reference's hash
// (uniquenodes_octree) merges only points closer than TOL in L1 that carry the
// same tag; where no such pair exists it merges nothing, and the host's octree
// restatement can be skipped.  The points are sorted by (tag, x, y) - three
// stable radix passes on order-preserving keys, -0.0 taken as +0.0 - and point
// i is compared with the next point (the nearest larger y of its tag and x)
// and with the nearest y of every following x within TOL (of its tag), found
// by binary search: every pair closer than TOL in L1 is one of those.
__device__ __forceinline__ unsigned long long order_key(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v == 0.0 ? 0.0 : v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__global__ void k_coinc_keys(long long n, const double* __restrict__ pts, const int* __restrict__ tags, int coord,
                             const int* __restrict__ perm, unsigned long long* __restrict__ key) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int p = perm[i];
    key[i] = coord < 2 ? order_key(pts[2 * (size_t)p + coord]) : (unsigned long long)(unsigned)(tags[p] ^ INT_MIN);
}
__global__ void k_coinc_iota(long long n, int* __restrict__ perm) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) perm[i] = (int)i;
}
__global__ void k_coinc_gather(long long n, const double* __restrict__ pts, const int* __restrict__ tags,
                               const int* __restrict__ perm, double* __restrict__ sx, double* __restrict__ sy,
                               int* __restrict__ st) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int p = perm[i];
    sx[i] = pts[2 * (size_t)p];
    sy[i] = pts[2 * (size_t)p + 1];
    st[i] = tags[p];
}
__device__ __forceinline__ bool coinc_pair(double x0, double y0, double x1, double y1) {
    return fabs(x0 - x1) + fabs(y0 - y1) < kTol;
}
__global__ void k_coinc_scan(long long n, const double* __restrict__ sx, const double* __restrict__ sy,
                             const int* __restrict__ st, int* __restrict__ found) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double xi = sx[i], yi = sy[i];
    const int ti = st[i];
    if (i + 1 < n && st[i + 1] == ti && coinc_pair(xi, yi, sx[i + 1], sy[i + 1])) {
        atomicOr(found, 1);
        return;
    }
    // end of this tag's run, then the following x groups within TOL
    long long lo = i + 1, hi = n;  // first index with tag != ti or x > xi
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (st[mid] == ti && !(sx[mid] > xi)) lo = mid + 1;
        else hi = mid;
    }
    long long g = lo;
    while (g < n && st[g] == ti && sx[g] - xi < kTol) {
        const double xg = sx[g];
        long long e = g + 1, h2 = n;  // end of the group of x = xg
        while (e < h2) {
            const long long mid = (e + h2) >> 1;
            if (st[mid] == ti && !(sx[mid] > xg)) e = mid + 1;
            else h2 = mid;
        }
        long long a = g, b = e;  // first y >= yi in [g, e)
        while (a < b) {
            const long long mid = (a + b) >> 1;
            if (sy[mid] < yi) a = mid + 1;
            else b = mid;
        }
        if ((a < e && coinc_pair(xi, yi, xg, sy[a])) || (a > g && coinc_pair(xi, yi, xg, sy[a - 1]))) {
            atomicOr(found, 1);
            return;
        }
        g = e;
    }
}

// A point whose search was merged into an earlier coincident one's takes that
// point's donor cell (search.cpp:255-262) and its own weights in it.
__global__ void k_take_coincident(long long n, const int* __restrict__ xtag, const double* __restrict__ pts,
                                  const double* __restrict__ xy, const int4* __restrict__ cv, int* __restrict__ donor,
                                  int* __restrict__ dnodes, double* __restrict__ w, int* err) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n || xtag[i] == i) return;
    long long r = i;
    while (xtag[r] != r) r = xtag[r];  // xtag[r] < r: ends at the first point of the group
    const int c = donor[r];
    double f[4] = {0.0, 0.0, 0.0, 0.0};
    int4 v = make_int4(-1, -1, -1, -1);
    if (c >= 0) {
        v = cv[c];
        double x[8];
        cell_coords(xy, v, x);
        if (!nodal_weights(v.w < 0 ? 3 : 4, x, pts[2 * i], pts[2 * i + 1], f)) atomicOr(err, 1);
    }
    put_donor(i, c, v, f, donor, dnodes, w);
}

// ---------------------------------------------------------------------------
// Fringe exchange (dataUpdate.cpp) and the node-to-cell mean (Orchestra.cpp)
// ---------------------------------------------------------------------------

// One thread per (receptor, variable): qq = sum over the donor's nodes, in list
// order, of q[node] * weight, starting from 0 (getInterpolatedSolution).
__global__ void k_interp_gather(long long n, int nvar, int layout, const int* __restrict__ nw,
                                const int* __restrict__ inode, const double* __restrict__ w,
                                const double* __restrict__ q, long long nnodes, double* __restrict__ vals) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n * nvar) return;
    const long long i = t / nvar;
    const int k = (int)(t - i * nvar);
    const int nwi = nw[i];
    double qq = 0;
    for (int m = 0; m < 4; m++) {
        if (m < nwi) {
            const double weight = w[4 * i + m];
            const long long node = inode[4 * i + m];
            const double qv = layout == CFD_LAYOUT_ROW ? q[node * nvar + k] : q[(long long)k * nnodes + node];
            qq += qv * weight;
        }
    }
    vals[t] = qq;
}

// updateSolnData: receptor i's values into node recv[i] of the receiving array.
__global__ void k_interp_scatter(long long n, int nvar, int layout, const int* __restrict__ recv,
                                 const double* __restrict__ vals, double* __restrict__ q, long long nnodes) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n * nvar) return;
    const long long i = t / nvar;
    const int k = (int)(t - i * nvar);
    const long long node = recv[i];
    if (layout == CFD_LAYOUT_ROW) q[node * nvar + k] = vals[t];
    else q[(long long)k * nnodes + node] = vals[t];
}

__global__ void k_node_to_cell(int ncell, int nvar, const int4* __restrict__ cv, const double* __restrict__ qn,
                               double* __restrict__ qc) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)ncell * nvar) return;
    const int c = (int)(t / nvar);
    const int k = (int)(t - (long long)c * nvar);
    const int4 v = cv[c];
    const int nv = v.w < 0 ? 3 : 4;
    double s = 0;
    s += qn[(long long)v.x * nvar + k];
    s += qn[(long long)v.y * nvar + k];
    s += qn[(long long)v.z * nvar + k];
    if (nv == 4) s += qn[(long long)v.w * nvar + k];
    s /= nv;
    qc[t] = s;
}


// ---------------------------------------------------------------------------
// Hole map (holeMap.cpp, MeshBlock.cpp:653-778, utils.cpp:645-860)
// ---------------------------------------------------------------------------

struct MapGeom {
    double lo[2], hi[2], ds[2];
    int nx, ny;
};

// Box of the wall nodes (getWallBounds): one block, exact min / max.
__global__ void k_wall_box(int nwall, const int* __restrict__ wn, const double* __restrict__ xy, double* box) {
    __shared__ double s[4][256];
    double lo0 = 1.0e15, lo1 = 1.0e15, hi0 = -1.0e15, hi1 = -1.0e15;  // BIGVALUE
    for (int i = threadIdx.x; i < nwall; i += blockDim.x) {
        const double x = xy[2 * wn[i]], y = xy[2 * wn[i] + 1];
        lo0 = lo0 < x ? lo0 : x;
        lo1 = lo1 < y ? lo1 : y;
        hi0 = hi0 > x ? hi0 : x;
        hi1 = hi1 > y ? hi1 : y;
    }
    s[0][threadIdx.x] = lo0;
    s[1][threadIdx.x] = lo1;
    s[2][threadIdx.x] = hi0;
    s[3][threadIdx.x] = hi1;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            const int o = threadIdx.x + h;
            s[0][threadIdx.x] = s[0][threadIdx.x] < s[0][o] ? s[0][threadIdx.x] : s[0][o];
            s[1][threadIdx.x] = s[1][threadIdx.x] < s[1][o] ? s[1][threadIdx.x] : s[1][o];
            s[2][threadIdx.x] = s[2][threadIdx.x] > s[2][o] ? s[2][threadIdx.x] : s[2][o];
            s[3][threadIdx.x] = s[3][threadIdx.x] > s[3][o] ? s[3][threadIdx.x] : s[3][o];
        }
        __syncthreads();
    }
    if (threadIdx.x < 4) box[threadIdx.x] = s[threadIdx.x][0];
}

__device__ __forceinline__ int map_floor(double v) {
    const double f = floor(v);
    if (!(f > -2147483648.0)) return INT_MIN;
    if (f > 2147483647.0) return INT_MAX;
    return (int)f;
}

// markWallBoundary: every cell with a wall node marks the map cells its
// vertices' box spans with 2.
__global__ void k_mark_walls(int ncell, const int4* __restrict__ cv, const unsigned char* __restrict__ wflag,
                             const double* __restrict__ xy, MapGeom g, int* __restrict__ sam) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int4 v = cv[c];
    const int nv = v.w < 0 ? 3 : 4;
    const int id[4] = {v.x, v.y, v.z, v.w};
    bool wall = false;
    for (int m = 0; m < 4; m++)
        if (m < nv && wflag[id[m]]) wall = true;
    if (!wall) return;
    int imin[2] = {INT_MAX, INT_MAX}, imax[2] = {-INT_MAX, -INT_MAX};
    for (int m = 0; m < 4; m++) {
        if (m >= nv) continue;
        for (int k = 0; k < 2; k++) {
            const int iv = map_floor((xy[2 * id[m] + k] - g.lo[k]) / g.ds[k]);
            imin[k] = imin[k] < iv ? imin[k] : iv;
            imax[k] = imax[k] > iv ? imax[k] : iv;
        }
    }
    const int nxk[2] = {g.nx, g.ny};
    for (int k = 0; k < 2; k++) {
        imin[k] = imin[k] > 0 ? imin[k] : 0;
        imax[k] = imax[k] < nxk[k] - 1 ? imax[k] : nxk[k] - 1;
    }
    for (int jj = imin[1]; jj <= imax[1]; jj++)
        for (int ii = imin[0]; ii <= imax[0]; ii++) sam[jj * g.nx + ii] = 2;
}

// fillHoleMap2D in one block, in shared memory: the border is set to 1, then
// sweeps paint every 0 cell with a painted neighbour until a sweep paints
// nothing (the painted set is the same whatever the sweep order); finally
// sam = 1 for unpainted and wall cells.  A sweep that paints nothing ends the
// loop, so at most nx*ny sweeps run.
__global__ void k_fill_map(int nx, int ny, int isym, int* __restrict__ sam) {
    extern __shared__ unsigned char hm[];
    volatile unsigned char* h = hm;
    const int n = nx * ny;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int x = i % nx, y = i / nx;
        h[i] = (x == 0 || x == nx - 1 || y == 0 || y == ny - 1) ? 1 : (unsigned char)sam[i];
    }
    __syncthreads();
    for (int sweep = 0; sweep < n; sweep++) {
        int painted = 0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int x = i % nx, y = i / nx;
            if (x == 0 || x == nx - 1 || y == 0 || y == ny - 1 || h[i] != 0) continue;
            bool p;
            if (isym == 1) p = h[i - nx] == 1 || h[i + nx] == 1;
            else if (isym == 2) p = h[i - 1] == 1 || h[i + 1] == 1;
            else p = h[i - nx] == 1 || h[i + nx] == 1 || h[i - 1] == 1 || h[i + 1] == 1;
            if (p) {
                h[i] = 1;
                painted = 1;
            }
        }
        if (!__syncthreads_or(painted)) break;
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) sam[i] = (h[i] == 0 || h[i] == 2) ? 1 : 0;
}

// checkHoleMap: the map cell of the point by truncation; outside the map is 0.
__device__ __forceinline__ int hole_at(double px, double py, const MapGeom& g, const int* __restrict__ sam) {
    const double q[2] = {px, py};
    const int nxk[2] = {g.nx, g.ny};
    int ix[2];
    for (int k = 0; k < 2; k++) {
        const double t = (q[k] - g.lo[k]) / g.ds[k];
        ix[k] = !(t > -2147483648.0) ? INT_MIN : (t > 2147483647.0 ? INT_MAX : (int)t);
        if (ix[k] < 0 || ix[k] > nxk[k] - 1) return 0;
    }
    return sam[ix[1] * g.nx + ix[0]];
}

__global__ void k_hole_check(long long n, const double* __restrict__ pts, MapGeom g, const int* __restrict__ sam,
                             int* __restrict__ inside) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    inside[i] = hole_at(pts[2 * i], pts[2 * i + 1], g, sam);
}

// Cell resolution of the assembly: computeCellVolume2D (mathTools/
// cellVolume.cpp:6-75) of the cell's vertices in their own order: a triangle's
// area by the shoelace sum of triangle_area, a quadrilateral split along the
// diagonal the cross-product sign tests pick (Vector3D::cross_product /
// dot_product, vector3d.cpp:43-97, in 3-D with zero z).
__device__ double ref_triangle_area(const double* p1, const double* p2, const double* p3) {
    double area = 0.5 * ((p1[0] - p2[0]) * (p1[1] + p2[1]) + (p2[0] - p3[0]) * (p2[1] + p3[1]) +
                         (p3[0] - p1[0]) * (p3[1] + p1[1]));
    if (area < 0) area = -area;
    return area;
}

__device__ double ref_cross_dot(const double* a, const double* b, const double* c, const double* d) {
    // (a x b) . (c x d) for in-plane vectors: z components only, as the 3-D
    // products with zero z give them
    const double z1 = a[0] * b[1] - a[1] * b[0];
    const double z2 = c[0] * d[1] - c[1] * d[0];
    double r = 0;
    r += (a[1] * 0.0 - 0.0 * b[1]) * (c[1] * 0.0 - 0.0 * d[1]);
    r += (0.0 * b[0] - a[0] * 0.0) * (0.0 * d[0] - c[0] * 0.0);
    r += z1 * z2;
    return r;
}

__global__ void k_cell_volume(int ncell, const double* __restrict__ xy, const int4* __restrict__ cv,
                              double* __restrict__ vol) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int4 v = cv[c];
    double x[4][2];
    const int ids[4] = {v.x, v.y, v.z, v.w};
    const int nv = v.w < 0 ? 3 : 4;
    for (int m = 0; m < nv; m++) {
        x[m][0] = xy[2 * ids[m]];
        x[m][1] = xy[2 * ids[m] + 1];
    }
    if (nv == 3) {
        vol[c] = ref_triangle_area(x[0], x[1], x[2]);
        return;
    }
    const double AB[2] = {x[1][0] - x[0][0], x[1][1] - x[0][1]};
    const double AC[2] = {x[2][0] - x[0][0], x[2][1] - x[0][1]};
    const double AD[2] = {x[3][0] - x[0][0], x[3][1] - x[0][1]};
    double area = 0;
    if (ref_cross_dot(AB, AC, AB, AD) > 0) {
        if (ref_cross_dot(AC, AD, AB, AD) > 0) {
            area += ref_triangle_area(x[0], x[2], x[1]);
            area += ref_triangle_area(x[0], x[2], x[3]);
        } else {
            area += ref_triangle_area(x[0], x[3], x[1]);
            area += ref_triangle_area(x[0], x[3], x[2]);
        }
    } else {
        area += ref_triangle_area(x[0], x[1], x[2]);
        area += ref_triangle_area(x[0], x[1], x[3]);
    }
    vol[c] = area;
}

// getCellIblanks (bookkeeping.cpp:654-705): a cell is a hole (0) if any of
// its nodes is, a receptor (-1) if all of its nodes are, else a field cell (1).
__global__ void k_cell_iblank(int ncell, const int4* __restrict__ cv, const int* __restrict__ ibl,
                              int* __restrict__ icell) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int4 v = cv[c];
    const int nv = v.w < 0 ? 3 : 4;
    const int id[4] = {v.x, v.y, v.z, v.w};
    int out = 1, nrec = 0;
    for (int m = 0; m < 4; m++) {
        if (m >= nv) break;
        const int b = ibl[id[m]];
        if (b == 0) {
            out = 0;
            break;
        }
        nrec += b == -1;
    }
    if (out != 0 && nrec == nv) out = -1;
    icell[c] = out;
}

// processDonors' hole test for one other block: a node without a donor cell
// in that block and inside its map is blanked.
__global__ void k_blank_nodes(int n, const double* __restrict__ xy, const int* __restrict__ donor, MapGeom g,
                              const int* __restrict__ sam, int* __restrict__ iblank) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (donor[i] < 0 && hole_at(xy[2 * i], xy[2 * i + 1], g, sam)) iblank[i] = 0;
}

// One layer of mandatory fringes: every cell with a tagged vertex tags all of
// its vertices in the next generation.
__global__ void k_fringe_layer(int ncell, const int4* __restrict__ cv, const int* __restrict__ tag,
                               int* __restrict__ tag1) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int4 v = cv[c];
    const bool quad = v.w >= 0;
    if (tag[v.x] == 1 || tag[v.y] == 1 || tag[v.z] == 1 || (quad && tag[v.w] == 1)) {
        tag1[v.x] = 1;
        tag1[v.y] = 1;
        tag1[v.z] = 1;
        if (quad) tag1[v.w] = 1;
    }
}

__global__ void k_tag_holes(int n, const int* __restrict__ iblank, int* __restrict__ tag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) tag[i] = iblank[i] == 0 ? 1 : 0;
}

__global__ void k_mandatory(int n, const int* __restrict__ iblank, const int* __restrict__ tag,
                            int* __restrict__ mand) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) mand[i] = (tag[i] && iblank[i]) ? 1 : 0;
}

inline unsigned blocks_for(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

}  // namespace

// ---------------------------------------------------------------------------
// Handles
// ---------------------------------------------------------------------------

struct cfd_block_s {
    int nnode = 0, ncell = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    double* xy = nullptr;  // 2*nnode
    int4* cv = nullptr;    // ncell, w = -1 for a triangle
    float4* fbox = nullptr;
    BinGrid grid{};
    long long nbins = 0, nent = 0;
    int* binptr = nullptr;  // nbins + 1
    int* cells = nullptr;   // nent
    int* err = nullptr;
    int nwall = 0;
    int* wall_nodes = nullptr;           // ends of the wall faces, ascending
    unsigned char* wall_flag = nullptr;  // per node: 1 on a wall face
    // host copies for the search tree: nodes, cells, and MeshBlock's cell
    // numbering (triangles first, then quadrilaterals, each in mesh order)
    std::vector<double> hxy;
    std::vector<int4> hcv;
    std::vector<int> order;
    ~cfd_block_s() {
        dfree(wall_nodes);
        dfree(wall_flag);
        dfree(xy);
        dfree(cv);
        dfree(fbox);
        dfree(binptr);
        dfree(cells);
        dfree(err);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
};

struct cfd_interp_s {
    long long n = 0, requested = 0;
    cudaStream_t stream = nullptr;
    std::vector<int> h_recv, h_donor, h_nw, h_inode;
    std::vector<double> h_w;
    int* recv = nullptr;
    int* nw = nullptr;
    int* inode = nullptr;
    double* w = nullptr;
    double* vals = nullptr;
    long long vals_cap = 0;
    ~cfd_interp_s() {
        dfree(recv);
        dfree(nw);
        dfree(inode);
        dfree(w);
        dfree(vals);
    }
};

struct cfd_holemap_s {
    MapGeom g{};
    cudaStream_t stream = nullptr;
    int* sam = nullptr;  // nx*ny on the device
    ~cfd_holemap_s() { dfree(sam); }
};

namespace {

int report(const OversetError& e) { return cfdgb::set_last_error(e.code, e.what()); }

void read_err(int* d_err, cudaStream_t s, int* h) {
    ck(cudaMemcpyAsync(h, d_err, sizeof(int), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
    ck(cudaStreamSynchronize(s), "cudaStreamSynchronize");
}

// below this many query points the host hash is cheaper than the device screen
constexpr long long kScreenMin = 1 << 16;

template <class T>
struct DevBuf {  // a device temporary freed on scope exit
    T* p = nullptr;
    explicit DevBuf(size_t n) { dalloc(&p, n); }
    ~DevBuf() { dfree(p); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
};

// What MeshBlock::search is given besides the points: per point a mesh tag
// and a resolution (merged in place over coincident points), per donor cell
// whether it may donate.  Null tags / res: one tag and unit resolutions, as a
// lone search of one point set.
struct SearchQuery {
    const double* h_pts = nullptr;           // host copy of the points
    const int* tags = nullptr;
    double* res = nullptr;                   // in / out
    const unsigned char* d_unacc = nullptr;  // device, per cell (null: every cell may donate)
    int* xtag = nullptr;                     // out (may be null): the point whose search each took
};

// Whether the coincident-point hash of n device points (tags on the host, null:
// one tag) can merge anything (see k_coinc_scan).
bool coincident_possible(long long n, const double* d_pts, const int* tags, cudaStream_t s) {
    DevBuf<int> d_tags(n), p0(n), p1(n), d_found(1);
    DevBuf<unsigned long long> k0(n), k1(n);
    DevBuf<double> sx(n), sy(n);
    DevBuf<int> st(n);
    if (tags) ck(cudaMemcpyAsync(d_tags.p, tags, n * sizeof(int), cudaMemcpyHostToDevice, s), "copy");
    else ck(cudaMemsetAsync(d_tags.p, 0, n * sizeof(int), s), "cudaMemsetAsync");
    k_coinc_iota<<<blocks_for(n, 256), 256, 0, s>>>(n, p0.p);
    ck(cudaGetLastError(), "k_coinc_iota");
    size_t tb = 0;
    ck(cub::DeviceRadixSort::SortPairs(nullptr, tb, k0.p, k1.p, p0.p, p1.p, (int)n, 0, 64, s), "sort size");
    DevBuf<unsigned char> tmp(tb);
    int* cur = p0.p;
    int* nxt = p1.p;
    for (int coord : {1, 0, 2}) {  // y, then x, then the tag: stable passes give (tag, x, y) order
        k_coinc_keys<<<blocks_for(n, 256), 256, 0, s>>>(n, d_pts, d_tags.p, coord, cur, k0.p);
        ck(cudaGetLastError(), "k_coinc_keys");
        ck(cub::DeviceRadixSort::SortPairs(tmp.p, tb, k0.p, k1.p, cur, nxt, (int)n, 0, 64, s), "sort");
        std::swap(cur, nxt);
    }
    k_coinc_gather<<<blocks_for(n, 256), 256, 0, s>>>(n, d_pts, d_tags.p, cur, sx.p, sy.p, st.p);
    ck(cudaGetLastError(), "k_coinc_gather");
    ck(cudaMemsetAsync(d_found.p, 0, sizeof(int), s), "cudaMemsetAsync");
    k_coinc_scan<<<blocks_for(n, 256), 256, 0, s>>>(n, sx.p, sy.p, st.p, d_found.p);
    ck(cudaGetLastError(), "k_coinc_scan");
    int found = 0;
    ck(cudaMemcpyAsync(&found, d_found.p, sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
    ck(cudaStreamSynchronize(s), "sync");
    return found != 0;
}

// Search n points (device d_pts, host copy in q) in block b, as
// MeshBlock::search does; outputs are device arrays (d_nodes, d_w may be null).
void search_device(cfd_block_t b, long long n, const double* d_pts, const SearchQuery& q, int* d_donor, int* d_nodes,
                   double* d_w) {
    if (n == 0) return;
    if (n > INT_MAX) throw OversetError(CFD_ERR_ARG, "donor search: more than 2^31-1 points");
    cudaStream_t s = b->stream;
    // the coincident-point hash runs on a host thread while the tree is built
    std::vector<int> xtag(n), ones;
    std::vector<double> unit;
    const int* tags = q.tags;
    double* res = q.res;
    if (!tags) {
        ones.assign(n, 1);
        tags = ones.data();
    }
    if (!res) {
        unit.assign(n, 1.0);
        res = unit.data();
    }
    std::exception_ptr hash_err;  // declared before the thread's joiner: it outlives the thread
    struct Joiner {
        std::thread t;
        ~Joiner() {
            if (t.joinable()) t.join();
        }
    } hash;
    // the reference's hash only where some pair can merge (else xtag is the identity and res is unchanged)
    if (n < kScreenMin || coincident_possible(n, d_pts, q.tags, s)) {
        hash.t = std::thread([&] {
            try {
                cfdgb::adt::coincident(n, q.h_pts, tags, res, xtag.data());
            } catch (...) {
                hash_err = std::current_exception();  // rethrown after the join
            }
        });
    } else {
        for (long long i = 0; i < n; i++) xtag[i] = (int)i;
    }
    const cfdgb::adt::Obb o = cfdgb::adt::find_obb(q.h_pts, n);
    DevBuf<unsigned char> d_cross(b->ncell);
    DevBuf<int> d_rank(b->ncell), d_err(2);  // d_err[1]: some point's donor depends on the tree's order
    k_obb_cross<<<blocks_for(b->ncell, 256), 256, 0, s>>>(b->ncell, b->xy, b->cv, o, d_cross.p, d_rank.p);
    ck(cudaGetLastError(), "k_obb_cross");
    ck(cudaMemsetAsync(d_err.p, 0, 2 * sizeof(int), s), "cudaMemsetAsync");
    // first pass with one rank for all tree cells: exact wherever at most one cell stops the walk
    k_donor_search<<<blocks_for(n, 128), 128, 0, s>>>(n, d_pts, b->xy, b->cv, b->fbox, b->binptr, b->cells, b->grid,
                                                       d_rank.p, q.d_unacc, d_donor, d_nodes, d_w, d_err.p,
                                                       d_err.p + 1);
    ck(cudaGetLastError(), "k_donor_search");
    int amb = 0;
    ck(cudaMemcpyAsync(&amb, d_err.p + 1, sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
    ck(cudaStreamSynchronize(s), "sync");
    if (amb) {
        // the tree's preorder numbers, then the search again with them
        std::vector<unsigned char> cross(b->ncell);
        ck(cudaMemcpyAsync(cross.data(), d_cross.p, b->ncell, cudaMemcpyDeviceToHost, s), "copy");
        ck(cudaStreamSynchronize(s), "sync");
        static_assert(sizeof(int4) == 4 * sizeof(int), "int4 holds four ints");
        const std::vector<int> rank = cfdgb::adt::tree_ranks(
            b->ncell, b->hxy.data(), reinterpret_cast<const int*>(b->hcv.data()), b->order.data(), cross.data());
        ck(cudaMemcpyAsync(d_rank.p, rank.data(), b->ncell * sizeof(int), cudaMemcpyHostToDevice, s), "copy");
        k_donor_search<<<blocks_for(n, 128), 128, 0, s>>>(n, d_pts, b->xy, b->cv, b->fbox, b->binptr, b->cells,
                                                           b->grid, d_rank.p, q.d_unacc, d_donor, d_nodes, d_w,
                                                           d_err.p, nullptr);
        ck(cudaGetLastError(), "k_donor_search");
    }
    if (hash.t.joinable()) hash.t.join();
    if (hash_err) std::rethrow_exception(hash_err);
    bool merged = false;
    for (long long i = 0; i < n && !merged; i++) merged = xtag[i] != i;
    if (merged) {
        DevBuf<int> d_xtag(n);
        ck(cudaMemcpyAsync(d_xtag.p, xtag.data(), n * sizeof(int), cudaMemcpyHostToDevice, s), "copy");
        k_take_coincident<<<blocks_for(n, 128), 128, 0, s>>>(n, d_xtag.p, d_pts, b->xy, b->cv, d_donor, d_nodes, d_w,
                                                              d_err.p);
        ck(cudaGetLastError(), "k_take_coincident");
        ck(cudaStreamSynchronize(s), "sync");
    }
    int h = 0;
    read_err(d_err.p, s, &h);
    if (h & 1) throw OversetError(CFD_ERR_MESH, "donor search: a triangle's weight system is singular (matrix degenerate)");
    if (q.xtag) std::copy(xtag.begin(), xtag.end(), q.xtag);
}

// Keep the last entry per receiving node (updateSolnData writes in list order,
// so the last one wins) and upload the list.
void finish_list(cfd_interp_s* it) {
    const long long n0 = (long long)it->h_recv.size();
    std::vector<char> keep(n0, 1);
    {
        std::vector<std::pair<int, long long>> order(n0);
        for (long long i = 0; i < n0; i++) order[i] = {it->h_recv[i], i};
        std::stable_sort(order.begin(), order.end(),
                         [](const auto& a, const auto& b) { return a.first < b.first; });
        for (long long j = 0; j + 1 < n0; j++)
            if (order[j].first == order[j + 1].first) keep[order[j].second] = 0;
    }
    long long n = 0;
    for (long long i = 0; i < n0; i++) {
        if (!keep[i]) continue;
        it->h_recv[n] = it->h_recv[i];
        it->h_donor[n] = it->h_donor[i];
        it->h_nw[n] = it->h_nw[i];
        for (int m = 0; m < 4; m++) {
            it->h_inode[4 * n + m] = it->h_inode[4 * i + m];
            it->h_w[4 * n + m] = it->h_w[4 * i + m];
        }
        n++;
    }
    it->n = n;
    it->h_recv.resize(n);
    it->h_donor.resize(n);
    it->h_nw.resize(n);
    it->h_inode.resize(4 * n);
    it->h_w.resize(4 * n);
    dalloc(&it->recv, n);
    dalloc(&it->nw, n);
    dalloc(&it->inode, 4 * n);
    dalloc(&it->w, 4 * n);
    ck(cudaMemcpyAsync(it->recv, it->h_recv.data(), n * sizeof(int), cudaMemcpyHostToDevice, it->stream), "copy");
    ck(cudaMemcpyAsync(it->nw, it->h_nw.data(), n * sizeof(int), cudaMemcpyHostToDevice, it->stream), "copy");
    ck(cudaMemcpyAsync(it->inode, it->h_inode.data(), 4 * n * sizeof(int), cudaMemcpyHostToDevice, it->stream),
       "copy");
    ck(cudaMemcpyAsync(it->w, it->h_w.data(), 4 * n * sizeof(double), cudaMemcpyHostToDevice, it->stream), "copy");
    ck(cudaStreamSynchronize(it->stream), "cudaStreamSynchronize");
}

}  // namespace

extern "C" {

int cfd_nodal_weights(long long n, const int* nvert, const double* xv, const double* xp, double* frac) {
    if (n < 0 || (n > 0 && (!nvert || !xv || !xp || !frac))) return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_nodal_weights: bad argument");
    if (n == 0) return CFD_OK;
    int *d_nv = nullptr, *d_err = nullptr;
    double *d_xv = nullptr, *d_xp = nullptr, *d_f = nullptr;
    int rc = CFD_OK;
    try {
        dalloc(&d_nv, n);
        dalloc(&d_xv, 8 * n);
        dalloc(&d_xp, 2 * n);
        dalloc(&d_f, 4 * n);
        dalloc(&d_err, 1);
        ck(cudaMemcpy(d_nv, nvert, n * sizeof(int), cudaMemcpyHostToDevice), "copy");
        ck(cudaMemcpy(d_xv, xv, 8 * n * sizeof(double), cudaMemcpyHostToDevice), "copy");
        ck(cudaMemcpy(d_xp, xp, 2 * n * sizeof(double), cudaMemcpyHostToDevice), "copy");
        ck(cudaMemset(d_err, 0, sizeof(int)), "cudaMemset");
        k_nodal_weights<<<blocks_for(n, 128), 128>>>(n, d_nv, d_xv, d_xp, d_f, d_err);
        ck(cudaGetLastError(), "k_nodal_weights");
        ck(cudaMemcpy(frac, d_f, 4 * n * sizeof(double), cudaMemcpyDeviceToHost), "copy");
        int h = 0;
        ck(cudaMemcpy(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost), "copy");
        if (h & 2) throw OversetError(CFD_ERR_ARG, "cfd_nodal_weights: nvert must be 3 or 4");
        if (h & 1) throw OversetError(CFD_ERR_MESH, "cfd_nodal_weights: Error matrix degenerate (singular triangle)");
    } catch (const OversetError& e) {
        rc = report(e);
    }
    dfree(d_nv);
    dfree(d_xv);
    dfree(d_xp);
    dfree(d_f);
    dfree(d_err);
    return rc;
}

int cfd_block_create(cfd_mesh_t mesh, void* stream, cfd_block_t* out) {
    if (!mesh || !out) return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_block_create: null argument");
    *out = nullptr;
    const cfdgb::HostMesh& m = mesh->m;
    if (m.ncell <= 0 || m.nnode <= 0) return cfdgb::set_last_error(CFD_ERR_MESH, "cfd_block_create: empty mesh");
    cfd_block_s* b = new (std::nothrow) cfd_block_s;
    if (!b) return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_block_create: out of host memory");
    void* tmp = nullptr;
    long long* d_count = nullptr;
    long long* d_offs = nullptr;
    int4* d_brange = nullptr;
    unsigned long long *d_k0 = nullptr, *d_k1 = nullptr;
    try {
        b->nnode = m.nnode;
        b->ncell = m.ncell;
        if (stream) {
            b->stream = (cudaStream_t)stream;
        } else {
            ck(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate");
            b->own_stream = true;
        }
        cudaStream_t s = b->stream;
        std::vector<int4> hcv(m.ncell);
        for (int c = 0; c < m.ncell; c++) {
            const int* v = &m.cell_verts[4 * c];
            if (m.cell_nvert[c] != 3 && m.cell_nvert[c] != 4)
                throw OversetError(CFD_ERR_MESH, "cfd_block_create: only triangles and quadrilaterals");
            hcv[c] = make_int4(v[0], v[1], v[2], m.cell_nvert[c] == 4 ? v[3] : -1);
        }
        b->hxy = m.xy;
        b->hcv = hcv;
        b->order.reserve(m.ncell);
        for (int pass = 0; pass < 2; pass++)
            for (int c = 0; c < m.ncell; c++)
                if ((hcv[c].w < 0) == (pass == 0)) b->order.push_back(c);
        // Bins: a uniform grid over the nodes' box with about four bins per cell.
        double x0 = 1e300, y0 = 1e300, x1 = -1e300, y1 = -1e300;
        for (int i = 0; i < m.nnode; i++) {
            x0 = std::min(x0, m.xy[2 * i]);
            x1 = std::max(x1, m.xy[2 * i]);
            y0 = std::min(y0, m.xy[2 * i + 1]);
            y1 = std::max(y1, m.xy[2 * i + 1]);
        }
        const double ex = std::max(x1 - x0, 1e-300), ey = std::max(y1 - y0, 1e-300);
        const double h = std::sqrt(ex * ey / (4.0 * m.ncell));
        const int nbx = (int)std::min(16384.0, std::max(1.0, std::ceil(ex / h)));
        const int nby = (int)std::min(16384.0, std::max(1.0, std::ceil(ey / h)));
        b->grid = BinGrid{x0, y0, nbx / ex, nby / ey, nbx, nby};
        b->nbins = (long long)nbx * nby;

        dalloc(&b->xy, 2 * (size_t)m.nnode);
        dalloc(&b->cv, m.ncell);
        dalloc(&b->fbox, m.ncell);
        dalloc(&b->err, 1);
        dalloc(&d_count, m.ncell);
        dalloc(&d_offs, m.ncell + 1);
        dalloc(&d_brange, m.ncell);
        ck(cudaMemcpyAsync(b->xy, m.xy.data(), 2 * (size_t)m.nnode * sizeof(double), cudaMemcpyHostToDevice, s),
           "copy");
        ck(cudaMemcpyAsync(b->cv, hcv.data(), m.ncell * sizeof(int4), cudaMemcpyHostToDevice, s), "copy");
        {
            std::vector<unsigned char> flag(m.nnode, 0);
            for (int e = 0; e < m.nedge; e++)
                if (m.lr[2 * e + 1] == cfdgb::kWall) flag[m.edge_nodes[2 * e]] = flag[m.edge_nodes[2 * e + 1]] = 1;
            std::vector<int> wn;
            for (int i = 0; i < m.nnode; i++)
                if (flag[i]) wn.push_back(i);
            b->nwall = (int)wn.size();
            dalloc(&b->wall_nodes, wn.size());
            dalloc(&b->wall_flag, m.nnode);
            ck(cudaMemcpyAsync(b->wall_nodes, wn.data(), wn.size() * sizeof(int), cudaMemcpyHostToDevice, s), "copy");
            ck(cudaMemcpyAsync(b->wall_flag, flag.data(), m.nnode, cudaMemcpyHostToDevice, s), "copy");
            ck(cudaStreamSynchronize(s), "sync");
        }
        k_cell_boxes<<<blocks_for(m.ncell, 256), 256, 0, s>>>(m.ncell, b->xy, b->cv, b->grid, b->fbox, d_brange,
                                                             d_count);
        ck(cudaGetLastError(), "k_cell_boxes");
        size_t tb_scan = 0, tb_sort = 0;
        ck(cub::DeviceScan::InclusiveSum(nullptr, tb_scan, d_count, d_offs + 1, m.ncell, s), "scan size");
        ck(cudaMemsetAsync(d_offs, 0, sizeof(long long), s), "cudaMemsetAsync");
        ck(cudaMalloc(&tmp, std::max<size_t>(tb_scan, 1)), "cudaMalloc");
        ck(cub::DeviceScan::InclusiveSum(tmp, tb_scan, d_count, d_offs + 1, m.ncell, s), "scan");
        long long nent = 0;
        ck(cudaMemcpyAsync(&nent, d_offs + m.ncell, sizeof(long long), cudaMemcpyDeviceToHost, s), "copy");
        ck(cudaStreamSynchronize(s), "sync");
        if (nent >= (1ll << 31)) throw OversetError(CFD_ERR_MESH, "cfd_block_create: too many bin entries");
        b->nent = nent;
        dalloc(&d_k0, nent);
        dalloc(&d_k1, nent);
        k_emit_keys<<<blocks_for(m.ncell, 256), 256, 0, s>>>(m.ncell, d_brange, d_offs, nbx, d_k0);
        ck(cudaGetLastError(), "k_emit_keys");
        int bin_bits = 1;
        while ((1ll << bin_bits) < b->nbins + 1) bin_bits++;
        cub::DoubleBuffer<unsigned long long> keys(d_k0, d_k1);
        ck(cub::DeviceRadixSort::SortKeys(nullptr, tb_sort, keys, (int)nent, 0, 32 + bin_bits, s), "sort size");
        ck(cudaStreamSynchronize(s), "sync");
        cudaFree(tmp);
        tmp = nullptr;
        ck(cudaMalloc(&tmp, std::max<size_t>(tb_sort, 1)), "cudaMalloc");
        ck(cub::DeviceRadixSort::SortKeys(tmp, tb_sort, keys, (int)nent, 0, 32 + bin_bits, s), "sort");
        dalloc(&b->binptr, b->nbins + 1);
        dalloc(&b->cells, nent);
        const long long nt = std::max(nent, b->nbins + 1);
        k_bin_ptr<<<blocks_for(nt, 256), 256, 0, s>>>(b->nbins, nent, keys.Current(), b->binptr, b->cells);
        ck(cudaGetLastError(), "k_bin_ptr");
        ck(cudaStreamSynchronize(s), "sync");
    } catch (const OversetError& e) {
        if (tmp) cudaFree(tmp);
        dfree(d_count);
        dfree(d_offs);
        dfree(d_brange);
        dfree(d_k0);
        dfree(d_k1);
        delete b;
        return report(e);
    }
    cudaFree(tmp);
    dfree(d_count);
    dfree(d_offs);
    dfree(d_brange);
    dfree(d_k0);
    dfree(d_k1);
    *out = b;
    return CFD_OK;
}

void cfd_block_free(cfd_block_t b) { delete b; }

int cfd_block_search_ex(cfd_block_t b, long long npts, const double* xy, const int* tags, double* res,
                        const unsigned char* cell_unaccept, int* donor_cell, int* donor_nodes, double* weights,
                        int* xtag) {
    if (!b || npts < 0 || (npts > 0 && (!xy || !donor_cell)))
        return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_block_search: bad argument");
    if (npts == 0) return CFD_OK;
    double *d_pts = nullptr, *d_w = nullptr;
    int *d_donor = nullptr, *d_nodes = nullptr;
    unsigned char* d_unacc = nullptr;
    int rc = CFD_OK;
    try {
        cudaStream_t s = b->stream;
        dalloc(&d_pts, 2 * npts);
        dalloc(&d_donor, npts);
        if (donor_nodes) dalloc(&d_nodes, 4 * npts);
        if (weights) dalloc(&d_w, 4 * npts);
        if (cell_unaccept) {
            dalloc(&d_unacc, b->ncell);
            ck(cudaMemcpyAsync(d_unacc, cell_unaccept, b->ncell, cudaMemcpyHostToDevice, s), "copy");
        }
        ck(cudaMemcpyAsync(d_pts, xy, 2 * npts * sizeof(double), cudaMemcpyHostToDevice, s), "copy");
        SearchQuery q;
        q.h_pts = xy;
        q.tags = tags;
        q.res = res;
        q.d_unacc = d_unacc;
        q.xtag = xtag;
        search_device(b, npts, d_pts, q, d_donor, d_nodes, d_w);
        ck(cudaMemcpyAsync(donor_cell, d_donor, npts * sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
        if (donor_nodes)
            ck(cudaMemcpyAsync(donor_nodes, d_nodes, 4 * npts * sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
        if (weights) ck(cudaMemcpyAsync(weights, d_w, 4 * npts * sizeof(double), cudaMemcpyDeviceToHost, s), "copy");
        ck(cudaStreamSynchronize(s), "sync");
    } catch (const OversetError& e) {
        rc = report(e);
    } catch (const std::bad_alloc&) {
        rc = cfdgb::set_last_error(CFD_ERR_CUDA, "cfd_block_search: host allocation failed");
    } catch (const std::system_error&) {
        rc = cfdgb::set_last_error(CFD_ERR_CUDA, "cfd_block_search: could not start a host thread");
    }
    dfree(d_pts);
    dfree(d_donor);
    dfree(d_nodes);
    dfree(d_w);
    dfree(d_unacc);
    return rc;
}

int cfd_block_search(cfd_block_t b, long long npts, const double* xy, int* donor_cell, int* donor_nodes,
                     double* weights) {
    return cfd_block_search_ex(b, npts, xy, nullptr, nullptr, nullptr, donor_cell, donor_nodes, weights, nullptr);
}

int cfd_block_node_to_cell(cfd_block_t b, const double* d_q_node, int nvar, double* d_q_cell, void* stream) {
    if (!b || !d_q_node || !d_q_cell || nvar <= 0)
        return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_block_node_to_cell: bad argument");
    cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
    const long long n = (long long)b->ncell * nvar;
    k_node_to_cell<<<blocks_for(n, 256), 256, 0, s>>>(b->ncell, nvar, b->cv, d_q_node, d_q_cell);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cfdgb::set_last_error(CFD_ERR_CUDA, std::string("k_node_to_cell: ") + cudaGetErrorString(e));
    return CFD_OK;
}

int cfd_interp_create(cfd_block_t donor, long long n, const double* xy, const int* recv_node, cfd_interp_t* out) {
    if (!donor || !out || n < 0 || (n > 0 && (!xy || !recv_node)))
        return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_interp_create: bad argument");
    *out = nullptr;
    cfd_interp_s* it = new (std::nothrow) cfd_interp_s;
    if (!it) return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_interp_create: out of host memory");
    it->stream = donor->stream;
    it->requested = n;
    double *d_pts = nullptr, *d_w = nullptr;
    int *d_donor = nullptr, *d_nodes = nullptr;
    try {
        std::vector<int> hd(n), hn(4 * n);
        std::vector<double> hw(4 * n);
        if (n > 0) {
            cudaStream_t s = donor->stream;
            dalloc(&d_pts, 2 * n);
            dalloc(&d_donor, n);
            dalloc(&d_nodes, 4 * n);
            dalloc(&d_w, 4 * n);
            ck(cudaMemcpyAsync(d_pts, xy, 2 * n * sizeof(double), cudaMemcpyHostToDevice, s), "copy");
            SearchQuery q;
            q.h_pts = xy;
            search_device(donor, n, d_pts, q, d_donor, d_nodes, d_w);
            ck(cudaMemcpyAsync(hd.data(), d_donor, n * sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
            ck(cudaMemcpyAsync(hn.data(), d_nodes, 4 * n * sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
            ck(cudaMemcpyAsync(hw.data(), d_w, 4 * n * sizeof(double), cudaMemcpyDeviceToHost, s), "copy");
            ck(cudaStreamSynchronize(s), "sync");
        }
        for (long long i = 0; i < n; i++) {
            if (hd[i] < 0) continue;
            it->h_recv.push_back(recv_node[i]);
            it->h_donor.push_back(hd[i]);
            it->h_nw.push_back(hn[4 * i + 3] < 0 ? 3 : 4);
            for (int m = 0; m < 4; m++) {
                it->h_inode.push_back(hn[4 * i + m] < 0 ? 0 : hn[4 * i + m]);
                it->h_w.push_back(hw[4 * i + m]);
            }
        }
        finish_list(it);
    } catch (const OversetError& e) {
        dfree(d_pts);
        dfree(d_donor);
        dfree(d_nodes);
        dfree(d_w);
        delete it;
        return report(e);
    }
    dfree(d_pts);
    dfree(d_donor);
    dfree(d_nodes);
    dfree(d_w);
    *out = it;
    return CFD_OK;
}

int cfd_interp_create_list(long long n, const int* recv_node, const int* nweights, const int* inode,
                           const double* weights, void* stream, cfd_interp_t* out) {
    if (!out || n < 0 || (n > 0 && (!recv_node || !nweights || !inode || !weights)))
        return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_interp_create_list: bad argument");
    *out = nullptr;
    for (long long i = 0; i < n; i++)
        if ((nweights[i] != 3 && nweights[i] != 4) || recv_node[i] < 0)
            return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_interp_create_list: nweights must be 3 or 4 and recv_node >= 0");
    for (long long i = 0; i < 4 * n; i++) {
        if ((i % 4) >= nweights[i / 4]) continue;
        if (inode[i] < 0) return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_interp_create_list: negative donor node");
        // getInterpolatedSolution's convexity check (dataUpdate.cpp:52-55), made once here
        if (weights[i] < -kTol || weights[i] > 1.0 + kTol)
            return cfdgb::set_last_error(CFD_ERR_MESH, "cfd_interp_create_list: weights are not convex");
    }
    cfd_interp_s* it = new (std::nothrow) cfd_interp_s;
    if (!it) return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_interp_create_list: out of host memory");
    try {
        if (stream) {
            it->stream = (cudaStream_t)stream;
        } else {
            it->stream = cudaStreamPerThread;
        }
        it->requested = n;
        it->h_recv.assign(recv_node, recv_node + n);
        it->h_donor.assign(n, -1);
        it->h_nw.assign(nweights, nweights + n);
        it->h_inode.resize(4 * n);
        it->h_w.resize(4 * n);
        for (long long i = 0; i < 4 * n; i++) {
            const bool used = (i % 4) < nweights[i / 4];
            it->h_inode[i] = used ? inode[i] : 0;
            it->h_w[i] = used ? weights[i] : 0.0;
        }
        finish_list(it);
    } catch (const OversetError& e) {
        delete it;
        return report(e);
    } catch (const std::exception& e) {  // host allocation or thread start
        delete it;
        return cfdgb::set_last_error(CFD_ERR_CUDA, std::string("cfd_interp_create: ") + e.what());
    }
    *out = it;
    return CFD_OK;
}

int cfd_interp_info(cfd_interp_t it, long long* n_found, long long* n_requested) {
    if (!it) return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_interp_info: null handle");
    if (n_found) *n_found = it->n;
    if (n_requested) *n_requested = it->requested;
    return CFD_OK;
}

int cfd_interp_get(cfd_interp_t it, int* recv_node, int* donor_cell, int* inode, double* weights) {
    if (!it) return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_interp_get: null handle");
    if (recv_node) std::copy(it->h_recv.begin(), it->h_recv.end(), recv_node);
    if (donor_cell) std::copy(it->h_donor.begin(), it->h_donor.end(), donor_cell);
    if (inode)
        for (long long i = 0; i < 4 * it->n; i++) inode[i] = (i % 4) < it->h_nw[i / 4] ? it->h_inode[i] : -1;
    if (weights) std::copy(it->h_w.begin(), it->h_w.end(), weights);
    return CFD_OK;
}

int cfd_interp_update(cfd_interp_t it, const double* d_q_donor, long long nnodes_donor, double* d_q_recv,
                      long long nnodes_recv, int nvar, int layout, void* stream) {
    if (!it || !d_q_donor || !d_q_recv || nvar <= 0 || (layout != CFD_LAYOUT_ROW && layout != CFD_LAYOUT_COLUMN))
        return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_interp_update: bad argument");
    if (it->n == 0) return CFD_OK;
    for (long long i = 0; i < it->n; i++)
        if (it->h_recv[i] >= nnodes_recv)
            return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_interp_update: a receptor node is beyond nnodes_recv");
    for (long long i = 0; i < 4 * it->n; i++)
        if ((i % 4) < it->h_nw[i / 4] && it->h_inode[i] >= nnodes_donor)
            return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_interp_update: a donor node is beyond nnodes_donor");
    cudaStream_t s = stream ? (cudaStream_t)stream : it->stream;
    try {
        const long long nv = it->n * nvar;
        if (nv > it->vals_cap) {
            dfree(it->vals);
            dalloc(&it->vals, nv);
            it->vals_cap = nv;
        }
        k_interp_gather<<<blocks_for(nv, 256), 256, 0, s>>>(it->n, nvar, layout, it->nw, it->inode, it->w, d_q_donor,
                                                           nnodes_donor, it->vals);
        ck(cudaGetLastError(), "k_interp_gather");
        k_interp_scatter<<<blocks_for(nv, 256), 256, 0, s>>>(it->n, nvar, layout, it->recv, it->vals, d_q_recv,
                                                            nnodes_recv);
        ck(cudaGetLastError(), "k_interp_scatter");
    } catch (const OversetError& e) {
        return report(e);
    }
    return CFD_OK;
}

void cfd_interp_free(cfd_interp_t it) { delete it; }

constexpr int kHoleMapSize = 192;  // HOLEMAPSIZE, UniTioga/codetypes.h:55

int cfd_holemap_create(cfd_block_t b, int isym, cfd_holemap_t* out) {
    if (!b || !out || isym < 1 || isym > 3) return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_holemap_create: bad argument");
    *out = nullptr;
    if (b->nwall == 0) return cfdgb::set_last_error(CFD_ERR_MESH, "cfd_holemap_create: the block has no wall faces");
    cfd_holemap_s* h = new (std::nothrow) cfd_holemap_s;
    if (!h) return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_holemap_create: out of host memory");
    double* d_box = nullptr;
    try {
        cudaStream_t s = b->stream;
        h->stream = s;
        dalloc(&d_box, 4);
        k_wall_box<<<1, 256, 0, s>>>(b->nwall, b->wall_nodes, b->xy, d_box);
        ck(cudaGetLastError(), "k_wall_box");
        double box[4];
        ck(cudaMemcpyAsync(box, d_box, sizeof(box), cudaMemcpyDeviceToHost, s), "copy");
        ck(cudaStreamSynchronize(s), "sync");
        // tioga::getHoleMap (holeMap.cpp:89-116) for one block in 2D.  The
        // reference also folds an unset third extent into dsmax; it is taken as 0.
        MapGeom& g = h->g;
        double ds[2], dsmax, dsbox;
        int nxk[2];
        for (int j = 0; j < 2; j++) {
            g.lo[j] = box[j];
            g.hi[j] = box[2 + j];
            ds[j] = g.hi[j] - g.lo[j];
        }
        dsmax = ds[0] > ds[1] ? ds[0] : ds[1];
        dsbox = dsmax / kHoleMapSize;
        for (int j = 0; j < 2; j++) {
            g.lo[j] -= (2 * dsbox);
            g.hi[j] += (2 * dsbox);
            const double r = (g.hi[j] - g.lo[j]) / dsbox;
            nxk[j] = (int)floor(r > 1 ? r : 1);
        }
        g.nx = nxk[0];
        g.ny = nxk[1];
        for (int k = 0; k < 2; k++) g.ds[k] = (g.hi[k] - g.lo[k]) / nxk[k];
        const long long ncell_map = (long long)g.nx * g.ny;
        if (!(dsbox > 0) || g.nx < 3 || g.ny < 3 || ncell_map > 200000)
            throw OversetError(CFD_ERR_MESH, "cfd_holemap_create: degenerate wall box");
        dalloc(&h->sam, ncell_map);
        ck(cudaMemsetAsync(h->sam, 0, ncell_map * sizeof(int), s), "cudaMemsetAsync");
        k_mark_walls<<<blocks_for(b->ncell, 256), 256, 0, s>>>(b->ncell, b->cv, b->wall_flag, b->xy, g, h->sam);
        ck(cudaGetLastError(), "k_mark_walls");
        ck(cudaFuncSetAttribute(k_fill_map, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ncell_map),
           "cudaFuncSetAttribute");
        k_fill_map<<<1, 1024, ncell_map, s>>>(g.nx, g.ny, isym, h->sam);
        ck(cudaGetLastError(), "k_fill_map");
        ck(cudaStreamSynchronize(s), "sync");
    } catch (const OversetError& e) {
        dfree(d_box);
        delete h;
        return report(e);
    }
    dfree(d_box);
    *out = h;
    return CFD_OK;
}

int cfd_holemap_info(cfd_holemap_t h, int* nx, double* extents) {
    if (!h) return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_holemap_info: null handle");
    if (nx) {
        nx[0] = h->g.nx;
        nx[1] = h->g.ny;
    }
    if (extents) {
        extents[0] = h->g.lo[0];
        extents[1] = h->g.lo[1];
        extents[2] = h->g.hi[0];
        extents[3] = h->g.hi[1];
    }
    return CFD_OK;
}

int cfd_holemap_get(cfd_holemap_t h, int* sam) {
    if (!h || !sam) return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_holemap_get: null argument");
    try {
        ck(cudaMemcpyAsync(sam, h->sam, (size_t)h->g.nx * h->g.ny * sizeof(int), cudaMemcpyDeviceToHost, h->stream),
           "copy");
        ck(cudaStreamSynchronize(h->stream), "sync");
    } catch (const OversetError& e) {
        return report(e);
    }
    return CFD_OK;
}

int cfd_holemap_check(cfd_holemap_t h, long long n, const double* xy, int* inside) {
    if (!h || n < 0 || (n > 0 && (!xy || !inside))) return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_holemap_check: bad argument");
    if (n == 0) return CFD_OK;
    double* d_pts = nullptr;
    int* d_in = nullptr;
    int rc = CFD_OK;
    try {
        cudaStream_t s = h->stream;
        dalloc(&d_pts, 2 * n);
        dalloc(&d_in, n);
        ck(cudaMemcpyAsync(d_pts, xy, 2 * n * sizeof(double), cudaMemcpyHostToDevice, s), "copy");
        k_hole_check<<<blocks_for(n, 256), 256, 0, s>>>(n, d_pts, h->g, h->sam, d_in);
        ck(cudaGetLastError(), "k_hole_check");
        ck(cudaMemcpyAsync(inside, d_in, n * sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
        ck(cudaStreamSynchronize(s), "sync");
    } catch (const OversetError& e) {
        rc = report(e);
    }
    dfree(d_pts);
    dfree(d_in);
    return rc;
}

void cfd_holemap_free(cfd_holemap_t h) { delete h; }

int cfd_cell_iblank(cfd_block_t b, const int* node_iblank, int* cell_iblank) {
    if (!b || !node_iblank || !cell_iblank) return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_cell_iblank: null argument");
    int *d_n = nullptr, *d_c = nullptr;
    int rc = CFD_OK;
    try {
        cudaStream_t s = b->stream;
        dalloc(&d_n, b->nnode);
        dalloc(&d_c, b->ncell);
        ck(cudaMemcpyAsync(d_n, node_iblank, b->nnode * sizeof(int), cudaMemcpyHostToDevice, s), "copy");
        k_cell_iblank<<<blocks_for(b->ncell, 256), 256, 0, s>>>(b->ncell, b->cv, d_n, d_c);
        ck(cudaGetLastError(), "k_cell_iblank");
        ck(cudaMemcpyAsync(cell_iblank, d_c, b->ncell * sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
        ck(cudaStreamSynchronize(s), "sync");
    } catch (const OversetError& e) {
        rc = report(e);
    }
    dfree(d_n);
    dfree(d_c);
    return rc;
}

// ---------------------------------------------------------------------------
// Overset assembly of several blocks on one device: the sequence of
// tioga::performConnectivity (tioga.cpp:153-262) for one rank, with the
// searches, hole-map tests and cell volumes on the GPU and the bookkeeping
// (resolutions, donor lists, fringe choice, donor cancellation, fringe
// reduction) on the host in the reference's order.
//   profile      MeshBlock::preprocess / tagBoundary (MeshBlock.cpp:135-425):
//                cellRes = cell volume, nodeRes = mean of the node's cells'
//                cellRes (cells triangles first, then quadrilaterals, as
//                MeshBlock numbers them); nodes of cells touching an overset-
//                boundary node get nodeRes = BIGVALUE (mandatory receptors),
//                and mexclude layers of cells around them cellRes = BIGVALUE
//                (unacceptable donors)
//   search       every other block's nodes in each block (MeshBlock::search)
//   donor lists  MeshBlock::insertAndSort / insertInList (linkList.cpp:62-105):
//                ascending donor resolution, ties in block order
//   processDonors (bookkeeping.cpp:75-277): holes, nfringe layers of
//                mandatory receptors, then each remaining node with a donor
//                of finer resolution than its own becomes a receptor
//   findInterpData (bookkeeping.cpp:310-428): the donor rejects a receptor
//                when one of its cell's nodes is a mandatory or a receptor of
//                the receptor's own mesh; a mandatory receptor releases the
//                donor cell's receptor nodes
//   exchangeDonors (exchangeDonor.cpp:24-347) cancellations and final
//                receptors; tioga::reduce_fringes (tioga.cpp:474-600,
//                bookkeeping.cpp:572-652): receptors beyond nfringe+1 layers
//                from field nodes become holes; getCellIblanks.
// Coincident search points only merge within one receptor mesh
// (uniqNodesTree, utils.cpp:484-620), so with distinct node coordinates
// resetCoincident changes nothing and is not restated.  Distance-scaled
// resolutions (MeshBlock::reResolution) are off, as tioga's default.
struct cfd_connect_s {
    std::vector<std::vector<int>> ibl, iblc;
    struct Rec {
        int recv_block, recv_node, donor_cell, nw;
        int inode[4];
        double w[4];
    };
    std::vector<std::vector<Rec>> interps;  // per donor block, interpList order, not cancelled
};

namespace {
constexpr double kBig = 1.0e15;  // BIGVALUE (codetypes.h)

struct ConnDonor {
    int d;          // donor block
    int cell;       // donor cell
    double res;     // donor cellRes
    double rres;    // receptor resolution from the search (merged over coincident nodes)
};
}  // namespace

int cfd_overset_connect(int nblocks, const cfd_block_t* blocks, const cfd_holemap_t* maps, const int* const* obc_nodes,
                        const int* nobc, int nfringe, int mexclude, cfd_connect_t* out) {
    if (nblocks < 2 || nblocks > 64 || !blocks || !maps || !nobc || !obc_nodes || nfringe < 0 || mexclude < 0 || !out)
        return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_overset_connect: bad argument (2 to 64 blocks)");
    for (int b = 0; b < nblocks; b++) {
        if (!blocks[b]) return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_overset_connect: null block");
        if (nobc[b] < 0 || (nobc[b] > 0 && !obc_nodes[b]))
            return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_overset_connect: bad overset-boundary list");
        for (int k = 0; k < nobc[b]; k++)
            if (obc_nodes[b][k] < 0 || obc_nodes[b][k] >= blocks[b]->nnode)
                return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_overset_connect: overset-boundary node out of range");
        for (int c = 0; c < b; c++)
            if (blocks[c] == blocks[b]) return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_overset_connect: a block twice");
    }
    *out = nullptr;
    const int nb = nblocks;
    std::vector<std::vector<double>> hxy(nb), cellRes(nb), nodeRes(nb);
    std::vector<std::vector<int4>> hcv(nb);
    std::vector<std::vector<int>> tm(nb);  // MeshBlock cell order: triangles, then quadrilaterals
    // donor[d][r]: donor cell in block d of every node of block r (-1: none), with its weights
    std::vector<std::vector<std::vector<int>>> dcell(nb, std::vector<std::vector<int>>(nb));
    std::vector<std::vector<std::vector<double>>> dw(nb, std::vector<std::vector<double>>(nb));
    // rres[d][r][v]: the receptor resolution block d's search returns for node v of block r
    std::vector<std::vector<std::vector<double>>> rres(nb, std::vector<std::vector<double>>(nb));
    std::vector<std::vector<std::vector<int>>> inside(nb, std::vector<std::vector<int>>(nb));
    double* d_vol = nullptr;
    int *d_donor = nullptr, *d_in = nullptr;
    int rc = CFD_OK;
    cfd_connect_s* res = new cfd_connect_s;
    try {
        size_t nmax = 0;
        for (int b = 0; b < nb; b++) nmax = std::max(nmax, (size_t)std::max(blocks[b]->nnode, blocks[b]->ncell));
        dalloc(&d_vol, nmax);
        dalloc(&d_donor, nmax);
        dalloc(&d_in, nmax);
        for (int b = 0; b < nb; b++) {
            cfd_block_s* B = blocks[b];
            cudaStream_t s = B->stream;
            hxy[b].resize(2 * (size_t)B->nnode);
            hcv[b].resize(B->ncell);
            cellRes[b].resize(B->ncell);
            ck(cudaMemcpyAsync(hxy[b].data(), B->xy, hxy[b].size() * sizeof(double), cudaMemcpyDeviceToHost, s), "copy");
            ck(cudaMemcpyAsync(hcv[b].data(), B->cv, hcv[b].size() * sizeof(int4), cudaMemcpyDeviceToHost, s), "copy");
            k_cell_volume<<<blocks_for(B->ncell, 256), 256, 0, s>>>(B->ncell, B->xy, B->cv, d_vol);
            ck(cudaGetLastError(), "k_cell_volume");
            ck(cudaMemcpyAsync(cellRes[b].data(), d_vol, B->ncell * sizeof(double), cudaMemcpyDeviceToHost, s), "copy");
            ck(cudaStreamSynchronize(s), "sync");
            for (int pass = 0; pass < 2; pass++)
                for (int c = 0; c < B->ncell; c++)
                    if ((hcv[b][c].w < 0) == (pass == 0)) tm[b].push_back(c);
        }
        // ---- profile: resolutions, mandatory overset-boundary receptors, mexclude
        auto verts = [&](int b, int c, int* v) {
            const int4 q = hcv[b][c];
            v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
            return q.w < 0 ? 3 : 4;
        };
        for (int b = 0; b < nb; b++) {
            const int nn = blocks[b]->nnode;
            std::vector<int> cnt(nn, 0), iflag(nn, 0), iex(nn, 0), iex1(nn, 0);
            nodeRes[b].assign(nn, 0.0);
            int v[4];
            for (int c : tm[b]) {
                const int nv = verts(b, c, v);
                for (int m = 0; m < nv; m++) {
                    cnt[v[m]]++;
                    nodeRes[b][v[m]] += cellRes[b][c];
                }
            }
            for (int i = 0; i < nn; i++)
                if (cnt[i]) nodeRes[b][i] = nodeRes[b][i] / cnt[i];
            for (int k = 0; k < nobc[b]; k++) iflag[obc_nodes[b][k]] = 1;
            for (int c : tm[b]) {
                const int nv = verts(b, c, v);
                int itag = 0;
                for (int m = 0; m < nv; m++) itag |= iflag[v[m]];
                if (itag)
                    for (int m = 0; m < nv; m++) nodeRes[b][v[m]] = kBig, iex[v[m]] = iex1[v[m]] = 1;
            }
            for (int it = 0; it < mexclude; it++) {
                for (int c : tm[b]) {
                    const int nv = verts(b, c, v);
                    for (int m = 0; m < nv; m++)
                        if (iex[v[m]] == 1) {
                            cellRes[b][c] = kBig;
                            break;
                        }
                    if (cellRes[b][c] == kBig)
                        for (int m = 0; m < nv; m++)
                            if (iex[v[m]] != 1) iex1[v[m]] = 1;
                }
                iex = iex1;
            }
        }
        // searches and hole-map tests, all on the device: block d is searched
        // once for the nodes of every other block, in block order, each node
        // tagged with its block and carrying its resolution (exchangeSearchData)
        for (int d = 0; d < nb; d++) {
            long long ntot = 0;
            for (int r = 0; r < nb; r++)
                if (r != d) ntot += blocks[r]->nnode;
            std::vector<double> pts;
            std::vector<int> tags, xtag(ntot);
            std::vector<double> rsearch;
            pts.reserve(2 * ntot);
            tags.reserve(ntot);
            rsearch.reserve(ntot);
            DevBuf<double> d_pts(2 * ntot), d_wd(4 * ntot);
            DevBuf<int> d_dn(ntot);
            DevBuf<unsigned char> d_unacc(blocks[d]->ncell);
            long long off = 0;
            for (int r = 0; r < nb; r++) {
                if (r == d) continue;
                const int n = blocks[r]->nnode;
                ck(cudaStreamSynchronize(blocks[r]->stream), "sync");
                ck(cudaMemcpyAsync(d_pts.p + 2 * off, blocks[r]->xy, 2 * (size_t)n * sizeof(double),
                                   cudaMemcpyDeviceToDevice, blocks[d]->stream), "copy");
                pts.insert(pts.end(), hxy[r].begin(), hxy[r].end());
                tags.insert(tags.end(), n, r + 1);
                rsearch.insert(rsearch.end(), nodeRes[r].begin(), nodeRes[r].end());
                off += n;
            }
            std::vector<unsigned char> unacc(blocks[d]->ncell);
            for (int c = 0; c < blocks[d]->ncell; c++) unacc[c] = cellRes[d][c] == kBig;
            ck(cudaMemcpyAsync(d_unacc.p, unacc.data(), unacc.size(), cudaMemcpyHostToDevice, blocks[d]->stream), "copy");
            SearchQuery q;
            q.h_pts = pts.data();
            q.tags = tags.data();
            q.res = rsearch.data();
            q.d_unacc = d_unacc.p;
            q.xtag = xtag.data();
            search_device(blocks[d], ntot, d_pts.p, q, d_dn.p, nullptr, d_wd.p);
            std::vector<int> dn(ntot);
            std::vector<double> wd(4 * ntot);
            ck(cudaMemcpyAsync(dn.data(), d_dn.p, ntot * sizeof(int), cudaMemcpyDeviceToHost, blocks[d]->stream), "copy");
            ck(cudaMemcpyAsync(wd.data(), d_wd.p, 4 * ntot * sizeof(double), cudaMemcpyDeviceToHost, blocks[d]->stream),
               "copy");
            ck(cudaStreamSynchronize(blocks[d]->stream), "sync");
            off = 0;
            for (int r = 0; r < nb; r++) {
                if (r == d) continue;
                const int n = blocks[r]->nnode;
                dcell[d][r].assign(dn.begin() + off, dn.begin() + off + n);
                dw[d][r].assign(wd.begin() + 4 * off, wd.begin() + 4 * (off + n));
                rres[d][r].resize(n);
                for (int v = 0; v < n; v++) rres[d][r][v] = rsearch[xtag[off + v]];  // res_search[xtag[i]]
                off += n;
                if (maps[d]) {
                    k_hole_check<<<blocks_for(n, 256), 256, 0, maps[d]->stream>>>(n, blocks[r]->xy, maps[d]->g,
                                                                                  maps[d]->sam, d_in);
                    ck(cudaGetLastError(), "k_hole_check");
                    inside[d][r].resize(n);
                    ck(cudaMemcpyAsync(inside[d][r].data(), d_in, n * sizeof(int), cudaMemcpyDeviceToHost,
                                       maps[d]->stream), "copy");
                    ck(cudaStreamSynchronize(maps[d]->stream), "sync");
                }
            }
        }
        // ---- donor lists (ascending donor resolution, ties in block order)
        std::vector<std::vector<std::vector<ConnDonor>>> dl(nb);
        for (int r = 0; r < nb; r++) dl[r].resize(blocks[r]->nnode);
        for (int d = 0; d < nb; d++)
            for (int r = 0; r < nb; r++) {
                if (r == d) continue;
                for (int v = 0; v < blocks[r]->nnode; v++) {
                    const int c = dcell[d][r][v];
                    if (c < 0) continue;
                    auto& L = dl[r][v];
                    ConnDonor e{d, c, cellRes[d][c], rres[d][r][v]};
                    size_t at = 0;
                    while (at < L.size() && !(std::fabs(L[at].res) > e.res)) at++;
                    L.insert(L.begin() + at, e);
                }
            }
        // ---- processDonors
        std::vector<std::vector<int>>& ibl = res->ibl;
        ibl.resize(nb);
        struct Acc {
            int r, v;
            double rres;
        };
        std::vector<std::vector<Acc>> accepted(nb);  // records in receptor order, per receptor block
        std::vector<int> acc_donor;                   // donor block of each accepted record, in the same order
        for (int r = 0; r < nb; r++) {
            const int nn = blocks[r]->nnode;
            ibl[r].assign(nn, 1);
            for (int i = 0; i < nn; i++) {
                unsigned long long has = 0;  // blocks that gave node i a donor
                for (const auto& e : dl[r][i]) {
                    has |= 1ull << e.d;
                    // a coincident node of the same block may have brought a larger resolution
                    nodeRes[r][i] = nodeRes[r][i] > e.rres ? nodeRes[r][i] : e.rres;
                }
                for (int j = 0; j < nb; j++) {
                    if (j == r || !maps[j] || ((has >> j) & 1)) continue;
                    if (inside[j][r][i]) {
                        ibl[r][i] = 0;
                        break;
                    }
                }
            }
            std::vector<int> mtag(nn), mtag1(nn);
            for (int i = 0; i < nn; i++) mtag[i] = mtag1[i] = ibl[r][i] == 0;
            int v[4];
            for (int it = 0; it < nfringe; it++) {
                for (int c : tm[r]) {
                    const int nv = verts(r, c, v);
                    for (int m = 0; m < nv; m++)
                        if (mtag[v[m]] == 1)
                            for (int mm = 0; mm < nv; mm++)
                                if (m != mm && mtag[v[mm]] != 1) mtag1[v[mm]] = 1;
                }
                mtag = mtag1;
            }
            for (int i = 0; i < nn; i++)
                if (mtag1[i] && ibl[r][i]) nodeRes[r][i] = kBig;
            for (int i = 0; i < nn; i++) {
                if (dl[r][i].empty() || ibl[r][i] == 0) continue;
                for (const auto& e : dl[r][i])
                    if (e.res < nodeRes[r][i]) {
                        ibl[r][i] = -(e.d + 1);
                        accepted[r].push_back({r, i, nodeRes[r][i]});
                        break;
                    }
            }
        }
        // ---- findInterpData, in the order the receptor blocks send their records
        struct Interp {
            int r, v, cell, nw, cancel;
            int inode[4];
            double w[4];
        };
        std::vector<std::vector<Interp>> il(nb);
        // interp index of each (donor d, receptor r, node v), -1: none (interp2donor)
        std::vector<std::vector<std::vector<int>>> i2d(nb, std::vector<std::vector<int>>(nb));
        for (int d = 0; d < nb; d++)
            for (int r = 0; r < nb; r++)
                if (r != d) i2d[d][r].assign(blocks[r]->nnode, -1);
        std::vector<std::vector<int>> cancel_list(nb);
        for (int r = 0; r < nb; r++)
            for (const Acc& a : accepted[r]) {
                const ConnDonor& e = dl[r][a.v].front();  // the accepted donor heads the list
                const int d = e.d, c = e.cell;
                int v[4];
                const int nv = verts(d, c, v);
                int accept = 1;
                for (int m = 0; m < nv; m++) {
                    const int u = v[m];
                    if (ibl[d][u] <= 0 && a.rres > 0.0) {
                        if (nodeRes[d][u] == kBig) accept = 0;
                        if (std::abs(ibl[d][u]) == r + 1) accept = 0;
                    }
                }
                if (a.rres == kBig)
                    for (int m = 0; m < nv; m++) {
                        const int u = v[m];
                        if (ibl[d][u] <= 0 && nodeRes[d][u] != kBig) {
                            if (ibl[d][u] < 0) ibl[d][u] = 1;
                            cancel_list[d].push_back(u);
                        }
                    }
                Interp it{};
                it.r = r;
                it.v = a.v;
                it.cell = c;
                it.nw = nv;
                for (int m = 0; m < 4; m++) {
                    it.inode[m] = m < nv ? v[m] : -1;
                    it.w[m] = m < nv ? dw[d][r][4 * (size_t)a.v + m] : 0.0;
                }
                it.cancel = (accept == 0 && a.rres != kBig) ? 1 : 0;
                i2d[d][r][a.v] = (int)il[d].size();
                il[d].push_back(it);
            }
        auto cancel_donor_of = [&](int b, int u) {
            // the head of node u's donor list names the donor block and record
            if (dl[b][u].empty()) return;
            const int d = dl[b][u].front().d;
            const int k = i2d[d][b][u];
            if (k > -1) il[d][k].cancel = 1;
        };
        auto final_receptors = [&](const std::vector<std::vector<int>>* reduced) {
            for (int b = 0; b < nb; b++)
                for (int i = 0; i < blocks[b]->nnode; i++) {
                    if (ibl[b][i] < 0) ibl[b][i] = 1;
                    if (reduced && (*reduced)[b][i] == 0) ibl[b][i] = 0;
                }
            for (int d = 0; d < nb; d++)
                for (const Interp& it : il[d])
                    if (!it.cancel) ibl[it.r][it.v] = -1;
        };
        for (int b = 0; b < nb; b++)
            for (int u : cancel_list[b]) cancel_donor_of(b, u);
        final_receptors(nullptr);
        // ---- reduce_fringes
        std::vector<std::vector<int>> red(nb);
        for (int b = 0; b < nb; b++) {
            const int nn = blocks[b]->nnode;
            red[b].resize(nn);
            for (int i = 0; i < nn; i++) red[b][i] = ibl[b][i] > 0 ? ibl[b][i] : 0;
            std::vector<int> tmp = red[b];
            int v[4];
            for (int it = 0; it < nfringe + 1; it++) {
                for (int c : tm[b]) {
                    const int nv = verts(b, c, v);
                    int ncount = 0;
                    for (int m = 0; m < nv; m++) ncount += (red[b][v[m]] == 1 || red[b][v[m]] < 0);
                    if (ncount > 0 && ncount < nv)
                        for (int m = 0; m < nv; m++)
                            if (tmp[v[m]] == 0 && ibl[b][v[m]] < 0) tmp[v[m]] = ibl[b][v[m]];
                }
                red[b] = tmp;
            }
        }
        for (int b = 0; b < nb; b++)
            for (int i = 0; i < blocks[b]->nnode; i++)
                if (ibl[b][i] < 0 && red[b][i] == 0) cancel_donor_of(b, i);
        final_receptors(&red);
        // ---- outputs: cell iblanks on the device, surviving interpolations
        res->iblc.resize(nb);
        res->interps.resize(nb);
        for (int b = 0; b < nb; b++) {
            cfd_block_s* B = blocks[b];
            cudaStream_t s = B->stream;
            ck(cudaMemcpyAsync(d_in, ibl[b].data(), B->nnode * sizeof(int), cudaMemcpyHostToDevice, s), "copy");
            k_cell_iblank<<<blocks_for(B->ncell, 256), 256, 0, s>>>(B->ncell, B->cv, d_in, d_donor);
            ck(cudaGetLastError(), "k_cell_iblank");
            res->iblc[b].resize(B->ncell);
            ck(cudaMemcpyAsync(res->iblc[b].data(), d_donor, B->ncell * sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
            ck(cudaStreamSynchronize(s), "sync");
            for (const Interp& it : il[b]) {
                if (it.cancel) continue;
                cfd_connect_s::Rec q{};
                q.recv_block = it.r;
                q.recv_node = it.v;
                q.donor_cell = it.cell;
                q.nw = it.nw;
                for (int m = 0; m < 4; m++) q.inode[m] = it.inode[m], q.w[m] = it.w[m];
                res->interps[b].push_back(q);
            }
        }
    } catch (const OversetError& e) {
        rc = report(e);
    } catch (const std::bad_alloc&) {
        rc = cfdgb::set_last_error(CFD_ERR_CUDA, "cfd_overset_connect: host allocation failed");
    } catch (const std::system_error&) {
        rc = cfdgb::set_last_error(CFD_ERR_CUDA, "cfd_overset_connect: could not start a host thread");
    }
    dfree(d_vol);
    dfree(d_donor);
    dfree(d_in);
    if (rc != CFD_OK) {
        delete res;
        return rc;
    }
    *out = res;
    return CFD_OK;
}

int cfd_connect_iblank(cfd_connect_t c, int block, int* node_iblank, int* cell_iblank) {
    if (!c || block < 0 || block >= (int)c->ibl.size())
        return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_connect_iblank: bad argument");
    if (node_iblank) std::copy(c->ibl[block].begin(), c->ibl[block].end(), node_iblank);
    if (cell_iblank) std::copy(c->iblc[block].begin(), c->iblc[block].end(), cell_iblank);
    return CFD_OK;
}

int cfd_connect_interp_count(cfd_connect_t c, int donor_block, long long* n) {
    if (!c || !n || donor_block < 0 || donor_block >= (int)c->interps.size())
        return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_connect_interp_count: bad argument");
    *n = (long long)c->interps[donor_block].size();
    return CFD_OK;
}

int cfd_connect_interp_get(cfd_connect_t c, int donor_block, int* recv_block, int* recv_node, int* donor_cell,
                           int* nweights, int* inode, double* weights) {
    if (!c || donor_block < 0 || donor_block >= (int)c->interps.size())
        return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_connect_interp_get: bad argument");
    const auto& L = c->interps[donor_block];
    for (size_t i = 0; i < L.size(); i++) {
        if (recv_block) recv_block[i] = L[i].recv_block;
        if (recv_node) recv_node[i] = L[i].recv_node;
        if (donor_cell) donor_cell[i] = L[i].donor_cell;
        if (nweights) nweights[i] = L[i].nw;
        for (int m = 0; m < 4; m++) {
            if (inode) inode[4 * i + m] = L[i].inode[m];
            if (weights) weights[4 * i + m] = L[i].w[m];
        }
    }
    return CFD_OK;
}

void cfd_connect_free(cfd_connect_t c) { delete c; }

int cfd_overset_blank(cfd_block_t self, int nother, const cfd_block_t* others, const cfd_holemap_t* maps,
                      int nfringe, int* iblank, int* mandatory) {
    if (!self || nother < 0 || (nother > 0 && (!others || !maps)) || nfringe < 0 || !iblank)
        return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_overset_blank: bad argument");
    for (int j = 0; j < nother; j++)
        if (!others[j] || others[j] == self) return cfdgb::set_last_error(CFD_ERR_ARG, "cfd_overset_blank: bad other block");
    const int n = self->nnode;
    int *d_ib = nullptr, *d_donor = nullptr, *d_tag = nullptr, *d_tag1 = nullptr;
    int rc = CFD_OK;
    try {
        cudaStream_t s = self->stream;
        dalloc(&d_ib, n);
        dalloc(&d_donor, n);
        std::vector<int> ones(n, 1);
        ck(cudaMemcpyAsync(d_ib, ones.data(), n * sizeof(int), cudaMemcpyHostToDevice, s), "copy");
        for (int j = 0; j < nother; j++) {
            if (!maps[j]) continue;
            ck(cudaStreamSynchronize(s), "sync");
            SearchQuery q;
            q.h_pts = self->hxy.data();
            search_device(others[j], n, self->xy, q, d_donor, nullptr, nullptr);  // on the other block's stream
            ck(cudaStreamSynchronize(others[j]->stream), "sync");
            k_blank_nodes<<<blocks_for(n, 256), 256, 0, s>>>(n, self->xy, d_donor, maps[j]->g, maps[j]->sam, d_ib);
            ck(cudaGetLastError(), "k_blank_nodes");
        }
        ck(cudaMemcpyAsync(iblank, d_ib, n * sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
        if (mandatory) {
            dalloc(&d_tag, n);
            dalloc(&d_tag1, n);
            k_tag_holes<<<blocks_for(n, 256), 256, 0, s>>>(n, d_ib, d_tag);
            ck(cudaMemcpyAsync(d_tag1, d_tag, n * sizeof(int), cudaMemcpyDeviceToDevice, s), "copy");
            for (int it = 0; it < nfringe; it++) {
                k_fringe_layer<<<blocks_for(self->ncell, 256), 256, 0, s>>>(self->ncell, self->cv, d_tag, d_tag1);
                ck(cudaGetLastError(), "k_fringe_layer");
                ck(cudaMemcpyAsync(d_tag, d_tag1, n * sizeof(int), cudaMemcpyDeviceToDevice, s), "copy");
            }
            k_mandatory<<<blocks_for(n, 256), 256, 0, s>>>(n, d_ib, d_tag1, d_tag);
            ck(cudaGetLastError(), "k_mandatory");
            ck(cudaMemcpyAsync(mandatory, d_tag, n * sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
        }
        ck(cudaStreamSynchronize(s), "sync");
    } catch (const OversetError& e) {
        rc = report(e);
    } catch (const std::exception& e) {  // host allocation or thread start
        rc = cfdgb::set_last_error(CFD_ERR_CUDA, std::string("cfd_overset_blank: ") + e.what());
    }
    dfree(d_ib);
    dfree(d_donor);
    dfree(d_tag);
    dfree(d_tag1);
    return rc;
}

}  // extern "C"
