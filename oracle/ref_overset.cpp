// Test-oracle driver around the reference's own overset code (UniTioga and
// mathTools, compiled from their sources by oracle/build_ref.sh).  Test
// infrastructure only.  Run it in a scratch directory: the reference's search
// and data update write debug files into the working directory.
//
//   ref_overset weights IN OUT   computeNodalWeight2D (mathTools/math.cpp:229-312)
//     IN:  int32 n, then n records {int32 nvert, double xv[4][2], double xp[2]}
//     OUT: n records of double frac[4] (unused entries 0; -1e300 where it throws)
//   ref_overset search MESH PTS OUT   MeshBlock::search (UniTioga/search.cpp:81-270)
//     MESH: int32 nnode, ncell; double xy[2*nnode]; int32 nvert[ncell]; int32 verts[4*ncell] (0-based)
//     PTS:  int32 n; double xy[2*n]
//     OUT:  int32 donor[n] in the mesh's own cell numbering (-1: none)
//   ref_overset search2 MESH PTS OUT   the same search with per-point mesh tags and
//     resolutions and per-cell donor acceptance (cellRes = BIGVALUE where refused)
//     PTS:  int32 n; double xy[2*n]; int32 tag[n]; double res[n]; int32 unaccept[ncell] (mesh order)
//     OUT:  int32 donor[n] (mesh numbering, -1: none); int32 xtag[n]; double res[n] after the search
//   ref_overset interp LIST OUT   MeshBlock::getInterpolatedSolution + updateSolnData
//     (UniTioga/dataUpdate.cpp:6-132), ROW then COLUMN
//     LIST: int32 nnodes, nvar, ninterp, nrecv_nodes; double q[nnodes*nvar] (ROW);
//           ninterp records {int32 recv, int32 nw, int32 inode[4], double w[4]}
//     OUT:  for ROW then COLUMN: double recv_q[nrecv_nodes*nvar] in that layout,
//           starting from zeros and updated by every record in order
//   ref_overset holemap MESH WALL PTS OUT   tioga::getHoleMap (UniTioga/holeMap.cpp:7-180)
//     with MeshBlock::getWallBounds/markWallBoundary and fillHoleMap, then checkHoleMap
//     (utils.cpp:645-670) of the points
//     WALL: int32 isym, nwall; int32 wall_nodes[nwall] (0-based)
//     OUT:  int32 nx[2]; double extents[4]; int32 sam[nx*ny]; int32 inside[n]
//   ref_overset celliblank MESH IBL OUT   MeshBlock::getCellIblanks (UniTioga/bookkeeping.cpp:654-705)
//     IBL: int32 iblank[nnode];  OUT: int32 iblank_cell[ncell] in the mesh's own cell numbering
//   ref_overset connect CONN OUT   one rank's overset assembly (see do_connect)
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "tioga.h"  // also brings MeshBlock.h, which has no include guard

int checkHoleMap(int dim, double* x, int* nx, int* sam, double* extents);

void computeNodalWeight2D(double xv[8][3], double* xp, double* frac, int nvert);

template <class T>
static bool rd(FILE* f, T* p, size_t n) {
    return fread(p, sizeof(T), n, f) == n;
}

static int do_weights(const char* in, const char* out) {
    FILE* fi = fopen(in, "rb");
    if (!fi) return 3;
    int n = 0;
    if (!rd(fi, &n, 1)) return 3;
    std::vector<double> res(4 * (size_t)n, 0.0);
    for (int q = 0; q < n; q++) {
        int nv;
        double v[8], p[2];
        if (!rd(fi, &nv, 1) || !rd(fi, v, 8) || !rd(fi, p, 2)) return 3;
        double xv[8][3] = {{0}};
        for (int i = 0; i < 4; i++) {
            xv[i][0] = v[2 * i];
            xv[i][1] = v[2 * i + 1];
        }
        double frac[8] = {0};
        try {
            computeNodalWeight2D(xv, p, frac, nv);
        } catch (const std::exception&) {
            frac[0] = frac[1] = frac[2] = frac[3] = -1e300;
        }
        for (int i = 0; i < 4; i++) res[4 * (size_t)q + i] = frac[i];
    }
    fclose(fi);
    FILE* fo = fopen(out, "wb");
    if (!fo) return 4;
    fwrite(res.data(), 8, res.size(), fo);
    fclose(fo);
    return 0;
}

// A mesh as a MeshBlock (static storage: the driver makes one per run).
struct BlockData {
    int nnode = 0, ncell = 0;
    std::vector<double> xy;
    std::vector<int> nvert, verts, order, vtri, vquad;
    std::vector<double> cellres;
    int types_nv[2], types_nc[2];
    int* vconn[2] = {nullptr, nullptr};
};

static bool read_block(const char* meshf, BlockData& d) {
    FILE* fm = fopen(meshf, "rb");
    if (!fm) return false;
    if (!rd(fm, &d.nnode, 1) || !rd(fm, &d.ncell, 1)) return false;
    d.xy.resize(2 * (size_t)d.nnode);
    d.nvert.resize(d.ncell);
    d.verts.resize(4 * (size_t)d.ncell);
    if (!rd(fm, d.xy.data(), d.xy.size()) || !rd(fm, d.nvert.data(), d.ncell) || !rd(fm, d.verts.data(), d.verts.size()))
        return false;
    fclose(fm);
    return true;
}

// MeshBlock numbers cells type by type: triangles first, then quadrilaterals.
static MeshBlock* make_block(BlockData& d) {
    int ntri = 0;
    for (int pass = 0; pass < 2; pass++)
        for (int c = 0; c < d.ncell; c++)
            if (d.nvert[c] == (pass == 0 ? 3 : 4)) d.order.push_back(c);
    for (int c = 0; c < d.ncell; c++) ntri += d.nvert[c] == 3;
    const int nquad = d.ncell - ntri;
    MeshBlock* mb = new MeshBlock();
    mb->d_dim = 2;
    mb->nnodes = d.nnode;
    mb->ncells = d.ncell;
    mb->x = d.xy.data();
    for (int c : d.order) {
        auto& dst = d.nvert[c] == 3 ? d.vtri : d.vquad;
        for (int m = 0; m < d.nvert[c]; m++) dst.push_back(d.verts[4 * (size_t)c + m] + BASE);
    }
    int nt = 0;
    if (ntri) { d.types_nv[nt] = 3; d.types_nc[nt] = ntri; d.vconn[nt] = d.vtri.data(); nt++; }
    if (nquad) { d.types_nv[nt] = 4; d.types_nc[nt] = nquad; d.vconn[nt] = d.vquad.data(); nt++; }
    mb->ntypes = nt;
    mb->nv = d.types_nv;
    mb->nc = d.types_nc;
    mb->vconn = d.vconn;
    d.cellres.assign(d.ncell, 1.0);
    mb->cellRes = d.cellres.data();
    mb->ihigh = 0;
    mb->meshtag = 1;
    return mb;
}

static bool read_points(const char* ptsf, std::vector<double>& pts) {
    FILE* fp = fopen(ptsf, "rb");
    if (!fp) return false;
    int n;
    if (!rd(fp, &n, 1)) return false;
    pts.resize(2 * (size_t)n);
    if (!rd(fp, pts.data(), pts.size())) return false;
    fclose(fp);
    return true;
}

static int do_search(const char* meshf, const char* ptsf, const char* out) {
    static BlockData d;
    std::vector<double> pts;
    if (!read_block(meshf, d) || !read_points(ptsf, pts)) return 3;
    const int n = (int)(pts.size() / 2);
    MeshBlock* mb = make_block(d);
    const std::vector<int>& order = d.order;
    mb->nsearch = n;
    mb->xsearch = pts.data();
    std::vector<int> tags(n, 1);
    std::vector<double> res(n, 1.0);
    mb->tagsearch = tags.data();
    mb->res_search = res.data();
    mb->search();
    std::vector<int> donor(n, -1);
    for (int i = 0; i < n; i++) donor[i] = mb->donorId[i] < 0 ? -1 : order[mb->donorId[i]];
    FILE* fo = fopen(out, "wb");
    if (!fo) return 4;
    fwrite(donor.data(), 4, donor.size(), fo);
    fclose(fo);
    return 0;  // the block is left allocated: the driver exits next
}

static int do_holemap(const char* meshf, const char* wallf, const char* ptsf, const char* out) {
    static BlockData d;
    std::vector<double> pts;
    if (!read_block(meshf, d) || !read_points(ptsf, pts)) return 3;
    FILE* fw = fopen(wallf, "rb");
    if (!fw) return 3;
    int isym, nwall;
    if (!rd(fw, &isym, 1) || !rd(fw, &nwall, 1)) return 3;
    static std::vector<int> wall(nwall);
    if (!rd(fw, wall.data(), nwall)) return 3;
    fclose(fw);
    for (int& w : wall) w += BASE;
    MeshBlock* mb = make_block(d);
    mb->nwbc = nwall;
    mb->wbcnode = wall.data();
    TIOGA::tioga* tg = new TIOGA::tioga();
    tg->d_dim = 2;
    tg->isym = isym;
    tg->scomm = MPI_COMM_WORLD;
    tg->nblocks = 1;
    tg->mblocks.emplace_back(mb);
    tg->mtags.push_back(1);
    tg->getHoleMap();
    HOLEMAP& h = tg->holeMap[0];
    const int n = (int)(pts.size() / 2);
    std::vector<int> inside(n);
    for (int i = 0; i < n; i++) inside[i] = checkHoleMap(2, &pts[2 * (size_t)i], h.nx, h.sam, h.extents);
    FILE* fo = fopen(out, "wb");
    if (!fo) return 4;
    fwrite(h.nx, 4, 2, fo);
    fwrite(h.extents, 8, 4, fo);
    fwrite(h.sam, 4, (size_t)h.nx[0] * h.nx[1], fo);
    fwrite(inside.data(), 4, inside.size(), fo);
    fclose(fo);
    return 0;  // tg and the block are left allocated: the driver exits next
}

static int do_celliblank(const char* meshf, const char* iblf, const char* out) {
    static BlockData d;
    if (!read_block(meshf, d)) return 3;
    static std::vector<int> ibl(d.nnode);
    FILE* fi = fopen(iblf, "rb");
    if (!fi || !rd(fi, ibl.data(), ibl.size())) return 3;
    fclose(fi);
    MeshBlock* mb = make_block(d);
    mb->iblank = ibl.data();
    mb->iblank_reduced = nullptr;
    mb->iblank_cell = nullptr;
    mb->getCellIblanks();
    std::vector<int> res(d.ncell);
    for (int k = 0; k < d.ncell; k++) res[d.order[k]] = mb->iblank_cell[k];
    FILE* fo = fopen(out, "wb");
    if (!fo) return 4;
    fwrite(res.data(), 4, res.size(), fo);
    fclose(fo);
    return 0;
}

static int do_interp(const char* listf, const char* out) {
    FILE* fl = fopen(listf, "rb");
    if (!fl) return 3;
    int nnodes, nvar, ninterp, nrecv;
    if (!rd(fl, &nnodes, 1) || !rd(fl, &nvar, 1) || !rd(fl, &ninterp, 1) || !rd(fl, &nrecv, 1)) return 3;
    std::vector<double> qrow((size_t)nnodes * nvar);
    if (!rd(fl, qrow.data(), qrow.size())) return 3;
    std::vector<int> recv(ninterp), nw(ninterp), inode(4 * (size_t)ninterp);
    std::vector<double> w(4 * (size_t)ninterp);
    for (int i = 0; i < ninterp; i++)
        if (!rd(fl, &recv[i], 1) || !rd(fl, &nw[i], 1) || !rd(fl, &inode[4 * (size_t)i], 4) ||
            !rd(fl, &w[4 * (size_t)i], 4))
            return 3;
    fclose(fl);
    std::vector<double> qcol((size_t)nnodes * nvar);
    for (int i = 0; i < nnodes; i++)
        for (int k = 0; k < nvar; k++) qcol[(size_t)k * nnodes + i] = qrow[(size_t)i * nvar + k];

    MeshBlock* mb = new MeshBlock();
    mb->d_dim = 2;
    mb->nnodes = nnodes;
    mb->ninterp = ninterp;
    std::vector<double> xdummy(2 * (size_t)nnodes, 0.0);
    mb->x = xdummy.data();
    mb->interpList = new INTERPLIST[ninterp];
    for (int i = 0; i < ninterp; i++) {
        INTERPLIST& e = mb->interpList[i];
        e.cancel = 0;
        e.nweights = nw[i];
        e.receptorInfo[0] = 0;
        e.receptorInfo[1] = recv[i];
        e.receptorInfo[2] = 0;
        e.inode = new int[nw[i] + 1];
        e.weights = new double[nw[i] + 1];
        for (int m = 0; m < nw[i]; m++) {
            e.inode[m] = inode[4 * (size_t)i + m];
            e.weights[m] = w[4 * (size_t)i + m];
        }
    }
    FILE* fo = fopen(out, "wb");
    if (!fo) return 4;
    for (int layout = 0; layout < 2; layout++) {
        int nints = 0, nreals = 0;
        int* idata = nullptr;
        double* rdata = nullptr;
        mb->getInterpolatedSolution(&nints, &nreals, &idata, &rdata, layout == 0 ? qrow.data() : qcol.data(),
                                    nvar, layout);
        std::vector<double> target((size_t)nrecv * nvar, 0.0);
        const int save = mb->nnodes;
        mb->nnodes = nrecv;  // updateSolnData's COLUMN stride is the receiving block's node count
        for (int i = 0; i < nints; i++) mb->updateSolnData(idata[3 * i + 1], &rdata[(size_t)i * nvar], target.data(), nvar, layout);
        mb->nnodes = save;
        fwrite(target.data(), 8, target.size(), fo);
    }
    fclose(fo);
    return 0;
}

// One rank's overset assembly with the reference's own MeshBlock code, in the
// order tioga::performConnectivity runs it (tioga.cpp:153-262): profile
// (MeshBlock::preprocess: resolutions, overset-boundary receptors, mexclude),
// getHoleMap, search of every other block's nodes, then exchangeDonors
// (exchangeDonor.cpp:24-347) and tioga::reduce_fringes (tioga.cpp:474-600)
// with each packet exchange done as the single-rank loop it reduces to, and
// getCellIblanks.  Distance-scaled resolutions are off (the tioga default).
//   CONN: int32 nblocks, nfringe, mexclude, isym; per block: int32 nnode, ncell;
//         double xy[2*nnode]; int32 nvert[ncell]; int32 verts[4*ncell];
//         int32 nwall; int32 wall[nwall]; int32 nobc; int32 obc[nobc] (0-based)
//   OUT:  per block int32 iblank[nnode], int32 iblank_cell[ncell] (mesh cell order);
//         then per donor block int32 n and n records {int32 recv_block, recv_node,
//         donor_cell (mesh order), nweights, inode[4]; double w[4]} of its
//         interpolations that were not cancelled
static int do_connect(const char* inf, const char* out) {
    FILE* f = fopen(inf, "rb");
    if (!f) return 3;
    int nb, nfringe, mexclude, isym;
    if (!rd(f, &nb, 1) || !rd(f, &nfringe, 1) || !rd(f, &mexclude, 1) || !rd(f, &isym, 1) || nb < 1 || nb > 64)
        return 3;
    static std::vector<BlockData> bd(nb);
    static std::vector<std::vector<int>> wall(nb), obc(nb), ibl(nb), iblc(nb);
    std::vector<MeshBlock*> mbs(nb);
    for (int b = 0; b < nb; b++) {
        BlockData& d = bd[b];
        if (!rd(f, &d.nnode, 1) || !rd(f, &d.ncell, 1)) return 3;
        d.xy.resize(2 * (size_t)d.nnode);
        d.nvert.resize(d.ncell);
        d.verts.resize(4 * (size_t)d.ncell);
        if (!rd(f, d.xy.data(), d.xy.size()) || !rd(f, d.nvert.data(), d.ncell) || !rd(f, d.verts.data(), d.verts.size()))
            return 3;
        int nw, no;
        if (!rd(f, &nw, 1)) return 3;
        wall[b].resize(nw);
        if (nw && !rd(f, wall[b].data(), nw)) return 3;
        if (!rd(f, &no, 1)) return 3;
        obc[b].resize(no);
        if (no && !rd(f, obc[b].data(), no)) return 3;
        for (int& w : wall[b]) w += BASE;
        for (int& o : obc[b]) o += BASE;
        MeshBlock* mb = make_block(d);
        mb->meshtag = b + 1;
        mb->cellRes = nullptr;  // tagBoundary allocates its own
        mb->nodeRes = nullptr;
        mb->nwbc = nw;
        mb->wbcnode = wall[b].data();
        mb->nobc = no;
        mb->obcnode = obc[b].data();
        ibl[b].assign(d.nnode, 1);
        mb->iblank = ibl[b].data();
        mb->iblank_reduced = nullptr;
        mb->iblank_cell = nullptr;
        mb->mexclude = mexclude;
        mb->nfringe = nfringe;
        mb->preprocess();
        mbs[b] = mb;
    }
    fclose(f);
    TIOGA::tioga* tg = new TIOGA::tioga();
    tg->d_dim = 2;
    tg->isym = isym;
    tg->scomm = MPI_COMM_WORLD;
    tg->nblocks = nb;
    for (int b = 0; b < nb; b++) {
        tg->mblocks.emplace_back(mbs[b]);
        tg->mtags.push_back(b + 1);
    }
    tg->getHoleMap();
    const int nmesh = nb;
    // search: every other block's nodes, block by block, node by node (exchangeSearchData)
    static std::vector<std::vector<double>> xs(nb), rs(nb);
    static std::vector<std::vector<int>> is(nb), ts(nb);
    for (int d = 0; d < nb; d++) {
        for (int r = 0; r < nb; r++) {
            if (r == d) continue;
            for (int v = 0; v < bd[r].nnode; v++) {
                xs[d].push_back(bd[r].xy[2 * (size_t)v]);
                xs[d].push_back(bd[r].xy[2 * (size_t)v + 1]);
                is[d].push_back(0);
                is[d].push_back(v);
                is[d].push_back(r);
                ts[d].push_back(r + 1);
                rs[d].push_back(mbs[r]->nodeRes[v]);
            }
        }
        MeshBlock* mb = mbs[d];
        mb->nsearch = (int)ts[d].size();
        mb->xsearch = xs[d].data();
        mb->isearch = is[d].data();
        mb->tagsearch = ts[d].data();
        mb->res_search = rs[d].data();
        mb->search();
    }
    // exchangeDonors, comm 1: donors to the receptor blocks
    for (int b = 0; b < nb; b++) mbs[b]->initializeDonorList();
    for (int d = 0; d < nb; d++) {
        MeshBlock* mb = mbs[d];
        for (int i = 0; i < mb->nsearch; i++) {
            if (mb->donorId[i] < 0) continue;
            mbs[mb->isearch[3 * i + 2]]->insertAndSort(mb->isearch[3 * i + 1], 0, mb->meshtag, i,
                                                       mb->cellRes[mb->donorId[i]], mb->res_search[mb->xtag[i]]);
        }
    }
    std::vector<int> nrec(nb, 0);
    std::vector<int*> drec(nb, nullptr);
    std::vector<double*> rres(nb, nullptr);
    for (int b = 0; b < nb; b++) mbs[b]->processDonors(tg->holeMap, nmesh, &drec[b], &rres[b], &nrec[b]);
    // comm 2: accepted receptors to their donors
    std::vector<int> ninterp(nb, 0);
    for (int n = 0; n < nb; n++)
        for (int i = 0; i < nrec[n]; i++) ninterp[drec[n][3 * i + 2] - 1]++;
    for (int b = 0; b < nb; b++) mbs[b]->initializeInterpList(ninterp[b]);
    std::fill(ninterp.begin(), ninterp.end(), 0);
    for (int n = 0; n < nb; n++)
        for (int i = 0; i < nrec[n]; i++) {
            const int ib = drec[n][3 * i + 2] - 1;
            mbs[ib]->findInterpData(&ninterp[ib], drec[n][3 * i + 1], rres[n][i]);
        }
    for (int b = 0; b < nb; b++) mbs[b]->set_ninterp(ninterp[b]);
    // comm 3: cancellations, comm 4: final receptors
    auto cancel_and_set = [&](bool reduced) {
        for (int b = 0; b < nb; b++) {
            int nr = 0;
            int* rec = nullptr;
            if (reduced) mbs[b]->getCancellationReduce(&nr, &rec);
            else mbs[b]->getCancellationData(&nr, &rec);
            for (int i = 0; i < nr; i++) mbs[rec[3 * i + 2] - 1]->cancelDonor(rec[3 * i + 1]);
        }
        for (int b = 0; b < nb; b++) mbs[b]->resetCoincident();
        std::vector<std::vector<int>> fin(nb);
        for (int b = 0; b < nb; b++) {
            int nr = 0;
            int* rec = nullptr;
            mbs[b]->getInterpData(&nr, &rec);
            for (int i = 0; i < nr; i++) fin[b].push_back(rec[3 * i + 1]), fin[b].push_back(rec[3 * i + 2]);
        }
        for (int b = 0; b < nb; b++) mbs[b]->clearIblanks();
        for (int b = 0; b < nb; b++)
            for (size_t i = 0; i < fin[b].size(); i += 2) mbs[fin[b][i + 1]]->setIblanks(fin[b][i]);
    };
    cancel_and_set(false);
    for (int b = 0; b < nb; b++) mbs[b]->reduce_fringes();
    cancel_and_set(true);
    FILE* fo = fopen(out, "wb");
    if (!fo) return 4;
    for (int b = 0; b < nb; b++) {
        MeshBlock* mb = mbs[b];
        mb->getCellIblanks();
        std::vector<int> cres(bd[b].ncell);
        for (int k = 0; k < bd[b].ncell; k++) cres[bd[b].order[k]] = mb->iblank_cell[k];
        fwrite(mb->iblank, 4, bd[b].nnode, fo);
        fwrite(cres.data(), 4, cres.size(), fo);
    }
    for (int d = 0; d < nb; d++) {
        MeshBlock* mb = mbs[d];
        int n = 0;
        for (int i = 0; i < mb->ninterp; i++) n += !mb->interpList[i].cancel;
        fwrite(&n, 4, 1, fo);
        for (int i = 0; i < mb->ninterp; i++) {
            const INTERPLIST& e = mb->interpList[i];
            if (e.cancel) continue;
            int head[4] = {e.receptorInfo[2], e.receptorInfo[1], bd[d].order[e.inode[e.nweights]], e.nweights};
            int nodes[4] = {-1, -1, -1, -1};
            double w[4] = {0, 0, 0, 0};
            for (int m = 0; m < e.nweights; m++) nodes[m] = e.inode[m], w[m] = e.weights[m];
            fwrite(head, 4, 4, fo);
            fwrite(nodes, 4, 4, fo);
            fwrite(w, 8, 4, fo);
        }
    }
    fclose(fo);
    return 0;  // the blocks are left allocated: the driver exits next
}

static int do_search2(const char* meshf, const char* ptsf, const char* out) {
    static BlockData d;
    if (!read_block(meshf, d)) return 3;
    FILE* fp = fopen(ptsf, "rb");
    if (!fp) return 3;
    int n;
    if (!rd(fp, &n, 1) || n < 0) return 3;
    static std::vector<double> pts, res;
    static std::vector<int> tags, unacc;
    pts.resize(2 * (size_t)n);
    tags.resize(n);
    res.resize(n);
    unacc.resize(d.ncell);
    if (!rd(fp, pts.data(), pts.size()) || !rd(fp, tags.data(), n) || !rd(fp, res.data(), n) ||
        !rd(fp, unacc.data(), d.ncell))
        return 3;
    fclose(fp);
    MeshBlock* mb = make_block(d);
    for (int k = 0; k < d.ncell; k++)
        if (unacc[d.order[k]]) d.cellres[k] = BIGVALUE;
    mb->nsearch = n;
    mb->xsearch = pts.data();
    mb->tagsearch = tags.data();
    mb->res_search = res.data();
    mb->search();
    std::vector<int> donor(n, -1), xtag(n, 0);
    for (int i = 0; i < n; i++) {
        donor[i] = mb->donorId[i] < 0 ? -1 : d.order[mb->donorId[i]];
        xtag[i] = mb->xtag[i];
    }
    FILE* fo = fopen(out, "wb");
    if (!fo) return 4;
    fwrite(donor.data(), 4, donor.size(), fo);
    fwrite(xtag.data(), 4, xtag.size(), fo);
    fwrite(res.data(), 8, res.size(), fo);
    fclose(fo);
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: %s weights|search|interp ...\n", argv[0]);
        return 2;
    }
    const std::string mode = argv[1];
    if (mode == "weights" && argc == 4) return do_weights(argv[2], argv[3]);
    if (mode == "search" && argc == 5) return do_search(argv[2], argv[3], argv[4]);
    if (mode == "search2" && argc == 5) return do_search2(argv[2], argv[3], argv[4]);
    if (mode == "interp" && argc == 4) return do_interp(argv[2], argv[3]);
    if (mode == "holemap" && argc == 6) return do_holemap(argv[2], argv[3], argv[4], argv[5]);
    if (mode == "celliblank" && argc == 5) return do_celliblank(argv[2], argv[3], argv[4]);
    if (mode == "connect" && argc == 4) return do_connect(argv[2], argv[3]);
    fprintf(stderr, "bad arguments\n");
    return 2;
}
