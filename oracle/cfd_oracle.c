/*
 * CPU restatement of the reference solver's per-iteration path, in plain C.
 *
 * TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline leg use this library as the checker and as the reported CPU
 * baseline.  The product (tmp_gb300/libcfdgb.so) never links or calls it.
 *
 * Parity pin: tests/test_oracle_golden.py checks every array this oracle
 * produces against fixtures dumped by the reference's own code
 * (tests/golden/make_golden.py runs oracle/_ref/ref_driver, built from the
 * reference sources by oracle/build_ref.sh).
 *
 * Each routine follows the cited reference function with the same operation
 * order; compiled with -ffp-contract=off it reproduces the reference bit for
 * bit on x86-64 and aarch64.  Arrays use the reference's interleaved layout
 * [NEQU*cell + eq] with NEQU = 4, primitive [rho, p, u, v], conservative
 * [rho, rhoE, rhou, rhov].
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NEQU 4
#define BC_WALL (-2)
#define BC_FAR (-3)

typedef struct {
    int nnode, nedge, ncell;
    const double* xy;   /* 2*nnode */
    const int* en;      /* 2*nedge node ids (0-based, file order) */
    const int* lr;      /* 2*nedge left, right|BC */
    const int* cv;      /* 4*ncell vertex ids (-1 pad), cell3d order */
    const int* cnv;     /* ncell */
    const int* ce;      /* 4*ncell edge ids ascending (-1 pad) */
    const int* cne;     /* ncell */
    int viscous;
    /* freestream (nondimensional) and Sutherland constants */
    double rho_inf, p_inf, u_inf, v_inf, c_inf, mach, re, t_inf;
    /* geometry */
    double *vol, *cen, *nrm, *area, *ecen, *walld;
    /* state and intermediates */
    double *U, *Ue, *grad, *gradT, *specc, *specv, *R, *dt, *mu, *mue, *phi, *UL, *UR;
    double *umax, *umin;
    /* integrators */
    double *W, *Wnow, *D, *dW1, *dW;
    double force[2]; /* momentum flux through wall faces of the last residual */
    /* SST k-omega (allocated by orc_sst_enable): coupled = 1 when the model
     * runs inside every LU-SGS step (the build's turbulent path), 0 when its
     * functions are only evaluated one by one (the reference's own code) */
    int sst, coupled;
    double density, pressure;          /* dimensional freestream */
    double sst_k, sst_w, sst_mut;       /* nondimensional freestream k, omega, mu_t */
    double *T, *Tw, *Tf, *TG, *F1, *F2, *mut, *mutf, *Tfc, *Tfv, *TR, *TD, *TdW1, *TdW;
    /* analysis switches (no reference counterpart; off by default): limiter
     * factors held at the values they had when phi_hold was set, and the
     * turbulence state (k, omega, mu_t) held by skipping the model's sweeps
     * and update in the coupled step */
    double* phi_hold;
    int turb_hold;
    /* > 0: the k equation's production limited to plim * beta* rho k omega
     * (Menter's SST guard, absent from the reference's rans_P_Solver); 0: as
     * the reference computes it */
    double plim;
} orc_t;

static const double Gamma = 1.4;

static double dot2(double a0, double a1, double b0, double b1) {
    double r = 0;
    r += a0 * b0;
    r += a1 * b1;
    return r;
}
static double dmax(double a, double b) { return (a < b) ? b : a; }
static double dmin(double a, double b) { return (b < a) ? b : a; }

orc_t* orc_create(int nnode, const double* xy, int nedge, const int* en, const int* lr, int ncell, const int* cv,
                  const int* cnv, const int* ce, const int* cne) {
    orc_t* o = (orc_t*)calloc(1, sizeof(orc_t));
    o->nnode = nnode; o->nedge = nedge; o->ncell = ncell;
    o->xy = xy; o->en = en; o->lr = lr; o->cv = cv; o->cnv = cnv; o->ce = ce; o->cne = cne;
    size_t c = (size_t)ncell, e = (size_t)nedge;
    o->vol = calloc(c, 8); o->cen = calloc(2 * c, 8); o->nrm = calloc(2 * e, 8); o->area = calloc(e, 8);
    o->ecen = calloc(2 * e, 8); o->walld = calloc(c, 8);
    o->U = calloc(4 * c, 8); o->Ue = calloc(4 * e, 8); o->grad = calloc(8 * c, 8); o->gradT = calloc(2 * c, 8);
    o->specc = calloc(c, 8); o->specv = calloc(c, 8); o->R = calloc(4 * c, 8); o->dt = calloc(c, 8);
    o->mu = calloc(c, 8); o->mue = calloc(e, 8); o->phi = calloc(4 * c, 8); o->UL = calloc(4 * e, 8);
    o->UR = calloc(4 * e, 8); o->umax = calloc(4 * c, 8); o->umin = calloc(4 * c, 8);
    o->W = calloc(4 * c, 8); o->Wnow = calloc(4 * c, 8); o->D = calloc(c, 8); o->dW1 = calloc(4 * c, 8);
    o->dW = calloc(4 * c, 8);
    return o;
}

void orc_free(orc_t* o) {
    if (!o) return;
    double* p[] = {o->vol, o->cen, o->nrm, o->area, o->ecen, o->walld, o->U, o->Ue, o->grad, o->gradT, o->specc,
                   o->specv, o->R, o->dt, o->mu, o->mue, o->phi, o->UL, o->UR, o->umax, o->umin, o->W, o->Wnow,
                   o->D, o->dW1, o->dW, o->T, o->Tw, o->Tf, o->TG, o->F1, o->F2, o->mut, o->mutf, o->Tfc, o->Tfv,
                   o->TR, o->TD, o->TdW1, o->TdW, o->phi_hold};
    for (size_t i = 0; i < sizeof(p) / sizeof(p[0]); i++) free(p[i]);
    free(o);
}

/* triangle_area, mathTools/cellVolume.cpp:6-19 */
static double tri_area(const double* p1, const double* p2, const double* p3) {
    double a = 0.5 * ((p1[0] - p2[0]) * (p1[1] + p2[1]) + (p2[0] - p3[0]) * (p2[1] + p3[1]) +
                      (p3[0] - p1[0]) * (p3[1] + p1[1]));
    if (a < 0) a = -a;
    return a;
}

/* edge3d::find_area/find_normal/find_center (toolBox/edge3d_int.h:93-230),
 * computeCellVolume2D (mathTools/cellVolume.cpp:21-75), cell3d::find_center,
 * UnstructBlock2D::ComputeWallCellDistance (UnstructBlock.h:265-298). */
void orc_geometry(orc_t* o) {
    for (int k = 0; k < o->nedge; k++) {
        const double* p0 = o->xy + 2 * o->en[2 * k];
        const double* p1 = o->xy + 2 * o->en[2 * k + 1];
        double dx = p1[0] - p0[0], dy = p1[1] - p0[1];
        double l2 = 0;
        l2 += dx * dx;
        l2 += dy * dy;
        double A = sqrt(l2);
        o->area[k] = A;
        o->nrm[2 * k] = dy / A;
        o->nrm[2 * k + 1] = -dx / A;
        double cx = 0, cy = 0;
        cx = cx + p0[0]; cy = cy + p0[1];
        cx = cx + p1[0]; cy = cy + p1[1];
        o->ecen[2 * k] = cx / 2.0;
        o->ecen[2 * k + 1] = cy / 2.0;
    }
    for (int c = 0; c < o->ncell; c++) {
        int n = o->cnv[c];
        const double* p[4];
        for (int i = 0; i < n; i++) p[i] = o->xy + 2 * o->cv[4 * c + i];
        double area;
        if (n == 3) {
            area = tri_area(p[0], p[1], p[2]);
        } else {
            double abx = p[1][0] - p[0][0], aby = p[1][1] - p[0][1];
            double acx = p[2][0] - p[0][0], acy = p[2][1] - p[0][1];
            double adx = p[3][0] - p[0][0], ady = p[3][1] - p[0][1];
            double abac = abx * acy - aby * acx, abad = abx * ady - aby * adx, acad = acx * ady - acy * adx;
            area = 0;
            if (abac * abad > 0) {
                if (acad * abad > 0) { area += tri_area(p[0], p[2], p[1]); area += tri_area(p[0], p[2], p[3]); }
                else { area += tri_area(p[0], p[3], p[1]); area += tri_area(p[0], p[3], p[2]); }
            } else {
                area += tri_area(p[0], p[1], p[2]);
                area += tri_area(p[0], p[1], p[3]);
            }
        }
        o->vol[c] = area;
        double cx = 0, cy = 0;
        for (int i = 0; i < n; i++) { cx = cx + p[i][0]; cy = cy + p[i][1]; }
        o->cen[2 * c] = cx / (double)n;
        o->cen[2 * c + 1] = cy / (double)n;
    }
    /* the wall faces (ascending), then every cell's minimum over them */
    int nw = 0;
    for (int k = 0; k < o->nedge; k++) nw += o->lr[2 * k + 1] == BC_WALL;
    int* wf = (int*)malloc(sizeof(int) * (size_t)(nw > 0 ? nw : 1));
    nw = 0;
    for (int k = 0; k < o->nedge; k++)
        if (o->lr[2 * k + 1] == BC_WALL) wf[nw++] = k;
    for (int c = 0; c < o->ncell; c++) {
        double d = 100000000000.0;
        for (int q = 0; q < nw; q++) {
            int k = wf[q];
            double x = o->cen[2 * c] - o->ecen[2 * k], y = o->cen[2 * c + 1] - o->ecen[2 * k + 1];
            d = dmin(d, fabs(dot2(x, y, o->nrm[2 * k], o->nrm[2 * k + 1])));
        }
        o->walld[c] = d;
    }
    free(wf);
}

/* TopologyHolderStrategy::set_fs_variable2 + update_nondim_variable
 * (TopologyHolderStrategy.cpp:325-396). */
void orc_set_freestream(orc_t* o, double Ma, double AOA, double Re, double density, double pressure, int viscous) {
    const double R = 287.0, PI = 3.141593;
    double aoa = PI * AOA / 180;
    double c = sqrt(Gamma * pressure / density);
    double T = pressure / (R * density);
    double vm = c * Ma;
    double u = vm * cos(aoa), v = vm * sin(aoa);
    o->u_inf = u / (c / sqrt(Gamma));
    o->v_inf = v / (c / sqrt(Gamma));
    o->p_inf = pressure / pressure;
    o->rho_inf = density / density;
    o->c_inf = sqrt(Gamma);
    o->mach = Ma;
    o->re = Re;
    o->t_inf = T;
    o->viscous = viscous;
    o->density = density;
    o->pressure = pressure;
}

void orc_init_freestream(orc_t* o) {
    for (int k = 0; k < o->ncell; k++) {
        o->U[4 * k] = o->rho_inf; o->U[4 * k + 1] = o->p_inf;
        o->U[4 * k + 2] = o->u_inf; o->U[4 * k + 3] = o->v_inf;
    }
}

/* initializeConsData / initializePrimData / UpdatePrimitiveVariables
 * (TopologyHolderStrategy.cpp:48-109) */
static void cons_from_prim(const double* u, double* w) {
    double vm = 0;
    vm += u[2] * u[2]; w[2] = u[0] * u[2];
    vm += u[3] * u[3]; w[3] = u[0] * u[3];
    w[0] = u[0];
    w[1] = u[1] / (Gamma - 1) + 0.5 * u[0] * vm;
}
static void prim_from_cons(const double* w, double* u) {
    double vm = 0;
    u[0] = w[0];
    u[2] = w[2] / u[0]; vm += u[2] * u[2];
    u[3] = w[3] / u[0]; vm += u[3] * u[3];
    u[1] = (Gamma - 1) * (w[1] - 0.5 * u[0] * vm);
}

void orc_cons_from_U(orc_t* o) {
    for (int k = 0; k < o->ncell; k++) cons_from_prim(o->U + 4 * k, o->W + 4 * k);
}

static double sutherland(const orc_t* o, double T) {
    double cc = 110.5 / o->t_inf;
    return (1.0 + cc) / (T + cc) * pow(T, 1.5) * sqrt(Gamma) * o->mach / o->re;
}

/* mu/Pr at a face and a cell (getMuOverPrEdge / getMuOverPrCell): laminar,
 * plus mu_t / Prt when the SST model is coupled (ViscousFlow2D.h:138-154 with
 * isLaminar() false; Pr = 0.72, Prt = 0.9, TopologyHolderStrategy.h:40-41). */
static int turb(const orc_t* o) { return o->sst && o->coupled; }
static double mpr_face(const orc_t* o, int k) {
    return turb(o) ? o->mue[k] / 0.72 + o->mutf[k] / 0.9 : o->mue[k] / 0.72;
}
static double mpr_cell(const orc_t* o, int c) {
    return turb(o) ? o->mu[c] / 0.72 + o->mut[c] / 0.9 : o->mu[c] / 0.72;
}
static void sst_equation(orc_t* o);

/* BoundaryStrategy::HandleInvicidBoundary / HandleViscousBoundary
 * (BoundaryStrategy.h:73-335).  Returns 1 when the slip-wall check fails. */
static int face_states(orc_t* o) {
    int bad = 0;
    for (int k = 0; k < o->nedge; k++) {
        int l = o->lr[2 * k], r = o->lr[2 * k + 1];
        double* ue = o->Ue + 4 * k;
        const double* ul = o->U + 4 * l;
        double nx = o->nrm[2 * k], ny = o->nrm[2 * k + 1];
        if (r >= 0) {
            for (int j = 0; j < 4; j++) ue[j] = (ul[j] + o->U[4 * r + j]) / 2;
        } else if (r == BC_WALL) {
            if (o->viscous) {
                ue[0] = ul[0]; ue[1] = ul[1]; ue[2] = 0; ue[3] = 0;
            } else {
                double vn = dot2(ul[2], ul[3], nx, ny);
                double t0 = ul[2] - nx * vn, t1 = ul[3] - ny * vn;
                if (dot2(t0, t1, nx, ny) > 1.0e-7) bad = 1;
                ue[0] = ul[0]; ue[1] = ul[1]; ue[2] = t0; ue[3] = t1;
            }
        } else {
            double vnl = dot2(ul[2], ul[3], nx, ny);
            double tl0 = ul[2] - nx * vnl, tl1 = ul[3] - ny * vnl;
            double vnr = dot2(o->u_inf, o->v_inf, nx, ny);
            double tr0 = o->u_inf - nx * vnr, tr1 = o->v_inf - ny * vnr;
            double rl = ul[0], pl = ul[1];
            if (fabs(vnr) < o->c_inf) {
                double cl = sqrt(Gamma * pl / rl);
                double vnb = (vnl + vnr + 2 * (cl - o->c_inf) / (Gamma - 1)) / 2;
                double cb = (vnl - vnr + 2 * (o->c_inf + cl) / (Gamma - 1)) * (Gamma - 1) / 4;
                double sb, e0, e1;
                if (vnr >= 0) { sb = (pl / pow(rl, Gamma)); e0 = tl0 + nx * vnb; e1 = tl1 + ny * vnb; }
                else { sb = (o->p_inf / pow(o->rho_inf, Gamma)); e0 = tr0 + nx * vnb; e1 = tr1 + ny * vnb; }
                ue[0] = pow((cb * cb / (Gamma * sb)), (1.0 / (Gamma - 1)));
                ue[1] = ue[0] * cb * cb / Gamma;
                ue[2] = e0; ue[3] = e1;
            } else if (vnr >= 0) {
                for (int j = 0; j < 4; j++) ue[j] = ul[j];
            } else {
                ue[0] = o->rho_inf; ue[1] = o->p_inf; ue[2] = o->u_inf; ue[3] = o->v_inf;
            }
        }
    }
    return bad;
}

/* HLLCFluxStrategy::computeFlux inner-face branch (HLLCFluxStrategy.cpp:40-133).
 * Returns 1 when the p* consistency check fails. */
static int hllc(const double* ql, const double* qr, double nx, double ny, double A, double* F) {
    double dl = ql[0], pl = ql[1], ul = ql[2], vl = ql[3];
    double vnl = dot2(ul, vl, nx, ny);
    double cl = sqrt(Gamma * pl / dl);
    double hl = pl * Gamma / ((Gamma - 1) * dl) + 0.5 * dot2(ul, vl, ul, vl);
    double dr = qr[0], pr = qr[1], ur = qr[2], vr = qr[3];
    double vnr = dot2(ur, vr, nx, ny);
    double cr = sqrt(Gamma * pr / dr);
    double hr = pr * Gamma / ((Gamma - 1) * dr) + 0.5 * dot2(ur, vr, ur, vr);
    double el = sqrt(dl) / (sqrt(dl) + sqrt(dr));
    double er = 1 - el;
    double ht = el * hl + er * hr;
    double vnt = el * vnl + er * vnr;
    double ct = sqrt((Gamma - 1) * (ht - 0.5 * (vnt * vnt)));
    double sl = dmin(vnl - cl, vnt - ct);
    double sr = dmax(vnt + ct, vnr + cr);
    double sm = (dr * vnr * (sr - vnr) - dl * vnl * (sl - vnl) + pl - pr) / (dr * (sr - vnr) - dl * (sl - vnl));
    double ps = dl * (vnl - sl) * (vnl - sm) + pl;
    double ps2 = dr * (vnr - sr) * (vnr - sm) + pr;
    int bad = !(fabs(ps2 - ps) < 1e-10);
    if (sl > 0.0) {
        double re = pl / (Gamma - 1) + 0.5 * dl * dot2(ul, vl, ul, vl);
        F[0] = vnl * dl * A; F[1] = vnl * (re + pl) * A;
        F[2] = (vnl * dl * ul + pl * nx) * A; F[3] = (vnl * dl * vl + pl * ny) * A;
    } else if (sr < 0.0) {
        double re = pr / (Gamma - 1) + 0.5 * dr * dot2(ur, vr, ur, vr);
        F[0] = vnr * dr * A; F[1] = vnr * (re + pr) * A;
        F[2] = (vnr * dr * ur + pr * nx) * A; F[3] = (vnr * dr * vr + pr * ny) * A;
    } else {
        double s, vn, d, p, u, v;
        if (sm < 0.0) { s = sr; vn = vnr; d = dr; p = pr; u = ur; v = vr; }
        else { s = sl; vn = vnl; d = dl; p = pl; u = ul; v = vl; }
        double re = p / (Gamma - 1) + 0.5 * d * dot2(u, v, u, v);
        double f0 = (s - vn) * d / (s - sm);
        double f1 = ((s - vn) * re - p * vn + ps * sm) / (s - sm);
        double f2 = ((s - vn) * d * u + (ps - p) * nx) / (s - sm);
        double f3 = ((s - vn) * d * v + (ps - p) * ny) / (s - sm);
        F[0] = f0 * sm * A; F[1] = (f1 + ps) * sm * A;
        F[2] = (f2 * sm + ps * nx) * A; F[3] = (f3 * sm + ps * ny) * A;
    }
    return bad;
}

static double venkat(double d2, double d1max, double d1min, double eps2) {
    if (d2 > 0) return (d1max * d1max + eps2 + 2 * d2 * d1max) / (d1max * d1max + 2 * d2 * d2 + d1max * d2 + eps2);
    if (d2 < 0) return (d1min * d1min + eps2 + 2 * d2 * d1min) / (d1min * d1min + 2 * d2 * d2 + d1min * d2 + eps2);
    return 1;
}

/* One residual evaluation, preprocessAdvanceSerial of Euler2D (Euler2D.h:133-140)
 * or ViscousFlow2D (ViscousFlow2D.h:192-212), with the reference's own face-loop
 * scatter order.  Returns a bit mask: 1 = p* check failed, 4 = wall check failed. */
int orc_residual(orc_t* o, int first_order) {
    int nc = o->ncell, ne = o->nedge, err = 0;
    memset(o->grad, 0, 8 * 8 * (size_t)nc);
    memset(o->gradT, 0, 2 * 8 * (size_t)nc);
    memset(o->specc, 0, 8 * (size_t)nc);
    memset(o->specv, 0, 8 * (size_t)nc);
    memset(o->R, 0, 4 * 8 * (size_t)nc);
    if (face_states(o)) err |= 4;
    o->force[0] = 0;
    o->force[1] = 0;
    /* solveGradient */
    for (int k = 0; k < ne; k++) {
        int l = o->lr[2 * k], r = o->lr[2 * k + 1];
        double nx = o->nrm[2 * k], ny = o->nrm[2 * k + 1], A = o->area[k];
        const double* ue = o->Ue + 4 * k;
        if (o->viscous) {
            double et = ue[1] / ue[0];
            o->gradT[2 * l] = o->gradT[2 * l] + nx * (A * et);
            o->gradT[2 * l + 1] = o->gradT[2 * l + 1] + ny * (A * et);
        }
        for (int j = 0; j < 4; j++) {
            o->grad[8 * l + 2 * j] = o->grad[8 * l + 2 * j] + nx * (A * ue[j]);
            o->grad[8 * l + 2 * j + 1] = o->grad[8 * l + 2 * j + 1] + ny * (A * ue[j]);
        }
        if (r >= 0) {
            if (o->viscous) {
                double et = ue[1] / ue[0];
                o->gradT[2 * r] = o->gradT[2 * r] - nx * (A * et);
                o->gradT[2 * r + 1] = o->gradT[2 * r + 1] - ny * (A * et);
            }
            for (int j = 0; j < 4; j++) {
                o->grad[8 * r + 2 * j] = o->grad[8 * r + 2 * j] - nx * (A * ue[j]);
                o->grad[8 * r + 2 * j + 1] = o->grad[8 * r + 2 * j + 1] - ny * (A * ue[j]);
            }
        }
    }
    for (int c = 0; c < nc; c++) {
        for (int j = 0; j < 8; j++) o->grad[8 * c + j] = o->grad[8 * c + j] / o->vol[c];
        if (o->viscous) { o->gradT[2 * c] = o->gradT[2 * c] / o->vol[c]; o->gradT[2 * c + 1] = o->gradT[2 * c + 1] / o->vol[c]; }
    }
    /* LaminarFluxStrategy::computeMu (LaminarFluxStrategy.h:76-96) */
    if (o->viscous) {
        for (int c = 0; c < nc; c++) o->mu[c] = sutherland(o, o->U[4 * c + 1] / o->U[4 * c]);
        for (int k = 0; k < ne; k++) o->mue[k] = sutherland(o, o->Ue[4 * k + 1] / o->Ue[4 * k]);
    }
    /* the turbulence equation's residual, between computeMu and the spectral
     * radii as in ViscousFlow2D::preprocessAdvance (ViscousFlow2D.h:163-190) */
    if (turb(o)) sst_equation(o);
    /* solveSpectralRadius */
    for (int k = 0; k < ne; k++) {
        int l = o->lr[2 * k], r = o->lr[2 * k + 1];
        const double* ue = o->Ue + 4 * k;
        double nx = o->nrm[2 * k], ny = o->nrm[2 * k + 1], A = o->area[k];
        double c = sqrt(Gamma * ue[1] / ue[0]);
        double vn = dot2(ue[2], ue[3], nx, ny);
        double s = (fabs(vn) + c) * A;
        o->specc[l] += s;
        if (r >= 0) o->specc[r] += s;
        if (o->viscous) {
            s = dmax(4 / (3.0 * ue[0]), Gamma / ue[0]) * mpr_face(o, k) * A * A;
            o->specv[l] += s / o->vol[l];
            if (r >= 0) o->specv[r] += s / o->vol[r];
        }
    }
    /* Vankatakrishnan_Limiter::init + computeLimiter (Vankatakrishnan_Limiter.hpp:69-177,186-200) */
    for (int i = 0; i < 4 * nc; i++) { o->umax[i] = o->U[i]; o->umin[i] = o->U[i]; o->phi[i] = 1.0; }
    for (int k = 0; k < ne; k++) {
        int l = o->lr[2 * k], r = o->lr[2 * k + 1];
        if (r < 0) continue;
        for (int j = 0; j < 4; j++) {
            o->umax[4 * l + j] = dmax(o->umax[4 * l + j], o->U[4 * r + j]);
            o->umin[4 * l + j] = dmin(o->umin[4 * l + j], o->U[4 * r + j]);
            o->umax[4 * r + j] = dmax(o->umax[4 * r + j], o->U[4 * l + j]);
            o->umin[4 * r + j] = dmin(o->umin[4 * r + j], o->U[4 * l + j]);
        }
    }
    for (int i = 0; i < 4 * nc; i++) { o->umax[i] = o->umax[i] - o->U[i]; o->umin[i] = o->umin[i] - o->U[i]; }
    for (int k = 0; k < ne; k++) {
        int l = o->lr[2 * k], r = o->lr[2 * k + 1];
        double eps2 = pow(5, 3) * pow(o->vol[l], 1);
        for (int side = 0; side < 2; side++) {
            int c = side ? r : l;
            if (c < 0) continue;
            double vx = o->ecen[2 * k] - o->cen[2 * c], vy = o->ecen[2 * k + 1] - o->cen[2 * c + 1];
            double* dst = side ? o->UR : o->UL;
            for (int j = 0; j < 4; j++) {
                double d2 = dot2(o->grad[8 * c + 2 * j], o->grad[8 * c + 2 * j + 1], vx, vy);
                dst[4 * k + j] = d2;
                double lim = venkat(d2, o->umax[4 * c + j], o->umin[4 * c + j], eps2);
                o->phi[4 * c + j] = dmin(o->phi[4 * c + j], lim);
            }
        }
    }
    if (first_order)
        for (int i = 0; i < 4 * nc; i++) o->phi[i] = 0.0;
    if (o->phi_hold) memcpy(o->phi, o->phi_hold, 4 * 8 * (size_t)nc);
    /* updateLeftRight + flux loop (HLLCFluxStrategy.h:35-100, HLLCFluxStrategy.cpp:4-170) */
    for (int k = 0; k < ne; k++) {
        int l = o->lr[2 * k], r = o->lr[2 * k + 1];
        double nx = o->nrm[2 * k], ny = o->nrm[2 * k + 1], A = o->area[k];
        double* ql = o->UL + 4 * k;
        double* qr = o->UR + 4 * k;
        double F[4];
        if (r >= 0) {
            for (int j = 0; j < 4; j++) {
                if (first_order) { ql[j] = 0; qr[j] = 0; }
                ql[j] = ql[j] * o->phi[4 * l + j] + o->U[4 * l + j];
                qr[j] = qr[j] * o->phi[4 * r + j] + o->U[4 * r + j];
            }
            if (hllc(ql, qr, nx, ny, A, F)) err |= 1;
        } else {
            for (int j = 0; j < 4; j++) ql[j] = qr[j] = o->Ue[4 * k + j];
            if (r == BC_WALL) {
                F[0] = 0 * A; F[1] = 0 * A; F[2] = ql[1] * nx * A; F[3] = ql[1] * ny * A;
            } else {
                double d = ql[0], p = ql[1], u = ql[2], v = ql[3];
                double re = p / (Gamma - 1) + 0.5 * d * dot2(u, v, u, v);
                double vn = dot2(u, v, nx, ny);
                F[0] = vn * d * A; F[1] = vn * (re + p) * A;
                F[2] = (vn * d * u + p * nx) * A; F[3] = (vn * d * v + p * ny) * A;
            }
        }
        for (int j = 0; j < 4; j++) o->R[4 * l + j] += F[j];
        if (r >= 0)
            for (int j = 0; j < 4; j++) o->R[4 * r + j] -= F[j];
        if (r == BC_WALL) { o->force[0] += F[2]; o->force[1] += F[3]; }
    }
    /* LaminarFluxStrategy::computeFlux(int) (LaminarFluxStrategy.h:110-216) */
    if (o->viscous) {
        for (int k = 0; k < ne; k++) {
            int l = o->lr[2 * k], r = o->lr[2 * k + 1];
            double nx = o->nrm[2 * k], ny = o->nrm[2 * k + 1], A = o->area[k];
            double mu = turb(o) ? o->mue[k] + o->mutf[k] : o->mue[k], eff = 2.0 / 3.0 * mu;
            double g[3][2];
            if (r >= 0) {
                double lx = o->cen[2 * r] - o->cen[2 * l], ly = o->cen[2 * r + 1] - o->cen[2 * l + 1];
                double l2 = dot2(lx, ly, lx, ly);
                for (int j = 0; j < 2; j++) {
                    double ax = (o->grad[8 * l + 2 * (2 + j)] + o->grad[8 * r + 2 * (2 + j)]) * 0.5;
                    double ay = (o->grad[8 * l + 2 * (2 + j) + 1] + o->grad[8 * r + 2 * (2 + j) + 1]) * 0.5;
                    double kk = (o->U[4 * r + 2 + j] - o->U[4 * l + 2 + j] - dot2(ax, ay, lx, ly)) / l2;
                    g[j][0] = ax + lx * kk; g[j][1] = ay + ly * kk;
                }
                double ax = (o->gradT[2 * l] + o->gradT[2 * r]) * 0.5, ay = (o->gradT[2 * l + 1] + o->gradT[2 * r + 1]) * 0.5;
                double rt = o->U[4 * r + 1] / o->U[4 * r], lt = o->U[4 * l + 1] / o->U[4 * l];
                double kk = (rt - lt - dot2(ax, ay, lx, ly)) / l2;
                g[2][0] = ax + lx * kk; g[2][1] = ay + ly * kk;
            } else {
                for (int j = 0; j < 2; j++) { g[j][0] = o->grad[8 * l + 2 * (2 + j)]; g[j][1] = o->grad[8 * l + 2 * (2 + j) + 1]; }
                if (r == BC_WALL) { g[2][0] = 0; g[2][1] = 0; }
                else { g[2][0] = o->gradT[2 * l]; g[2][1] = o->gradT[2 * l + 1]; }
            }
            double ve0 = o->Ue[4 * k + 2], ve1 = o->Ue[4 * k + 3];
            double txx = eff * (2.0 * g[0][0] - g[1][1]);
            double tyy = eff * (2.0 * g[1][1] - g[0][0]);
            double txy = mu * (g[0][1] + g[1][0]);
            double qx = -Gamma / (Gamma - 1) * mpr_face(o, k) * g[2][0];
            double qy = -Gamma / (Gamma - 1) * mpr_face(o, k) * g[2][1];
            double Fv[4];
            Fv[0] = 0.0;
            Fv[1] = ((ve0 * txx + ve1 * txy - qx) * nx + (ve0 * txy + ve1 * tyy - qy) * ny) * A;
            Fv[2] = (txx * nx + txy * ny) * A;
            Fv[3] = (txy * nx + tyy * ny) * A;
            for (int j = 0; j < 4; j++) o->R[4 * l + j] -= Fv[j];
            if (r >= 0)
                for (int j = 0; j < 4; j++) o->R[4 * r + j] += Fv[j];
            if (r == BC_WALL) { o->force[0] -= Fv[2]; o->force[1] -= Fv[3]; }
        }
    }
    return err;
}

/* Euler2D/ViscousFlow2D::SolveTime (Euler2D.h:67-77, ViscousFlow2D.h:223-242):
 * the laminar branch, or with the SST model coupled the turbulent one,
 * dt = CFL vol / (spec_c + 4 spec_v). */
void orc_solve_time(orc_t* o, double cfl) {
    for (int c = 0; c < o->ncell; c++)
        o->dt[c] = turb(o) ? cfl * o->vol[c] / (o->specc[c] + 4.0 * o->specv[c]) : cfl * o->vol[c] / o->specc[c];
}

/* RungeKuttaStrategy::singleStepSerial (RungeKuttaStrategy.h:74-86,39-72). */
int orc_rk_step(orc_t* o, int first_order) {
    static const double a[5] = {1.0 / 4, 1.0 / 6, 3.0 / 8, 1.0 / 2, 1.0};
    int err = 0;
    orc_cons_from_U(o);
    for (int s = 0; s < 5; s++) {
        err |= orc_residual(o, first_order);
        if (s == 0) orc_solve_time(o, 0.8);
        for (int k = 0; k < o->ncell; k++) {
            for (int j = 0; j < 4; j++)
                o->Wnow[4 * k + j] = o->W[4 * k + j] + a[s] * o->dt[k] * (-o->R[4 * k + j]) / o->vol[k];
            prim_from_cons(o->Wnow + 4 * k, o->U + 4 * k);
        }
    }
    return err;
}

/* ConservativeParam2ConvectiveFlux (TopologyHolderStrategy.cpp:129-141) */
static void conv_flux(const double* w, double nx, double ny, double* F) {
    double u = w[2] / w[0], v = w[3] / w[0];
    double vn = dot2(u, v, nx, ny);
    double d = w[0];
    double p = (Gamma - 1) * (w[1] - 0.5 * d * dot2(u, v, u, v));
    F[0] = w[0] * vn; F[1] = (w[1] + p) * vn; F[2] = w[2] * vn + p * nx; F[3] = w[3] * vn + p * ny;
}

static void sst_step_sweeps(orc_t* o);
static void sst_step_update(orc_t* o);

/* SolveDF + SolveViscousFlux (TopologyHolderStrategy.cpp:143-323) for cell i,
 * face k, forward (fb = 1) or backward (fb = 0), increment array dWx. */
static void solve_df(const orc_t* o, int i, int k, const double* dWx, int fb, double* DF) {
    int l = o->lr[2 * k], r = o->lr[2 * k + 1];
    int j, left;
    for (int m = 0; m < 4; m++) DF[m] = 0;
    if (i == l) {
        if (!(r >= 0 && (int)(r < l) == fb)) return;
        j = r; left = 1;
    } else {
        if (!((int)(l < r) == fb)) return;
        j = l; left = 0;
    }
    double w0[4], dw[4], wp[4], fc[4], fcp[4];
    for (int m = 0; m < 4; m++) { w0[m] = o->W[4 * j + m]; dw[m] = dWx[4 * j + m]; wp[m] = w0[m] + dw[m]; }
    double nx = o->nrm[2 * k], ny = o->nrm[2 * k + 1], A = o->area[k];
    conv_flux(w0, nx, ny, fc);
    conv_flux(wp, nx, ny, fcp);
    const double* uj = o->U + 4 * j;
    double lx = o->cen[2 * j] - o->cen[2 * i], ly = o->cen[2 * j + 1] - o->cen[2 * i + 1];
    double vn = dot2(uj[2], uj[3], nx, ny);
    double c = sqrt(Gamma * uj[1] / uj[0]);
    double rA = 1.5 * (fabs(vn) + c);
    if (o->viscous) rA += dmax(4 / (3 * uj[0]), Gamma / uj[0]) * mpr_cell(o, i) / sqrt(dot2(lx, ly, lx, ly));
    for (int m = 0; m < 4; m++) {
        double fv = rA * dw[m];
        double dfc = left ? (fcp[m] - fc[m]) : (fc[m] - fcp[m]);
        DF[m] = 0.5 * (dfc - fv) * A;
    }
}

/* LUSGSIntegrator::UpdateSerial (LUSGS_Integrator.cpp:228-240): residual,
 * SolveTime, SolveDiag, serial forward and backward sweeps, W += dW. */
int orc_lusgs_step(orc_t* o, double cfl, int first_order) {
    int err = orc_residual(o, first_order);
    orc_solve_time(o, cfl);
    for (int c = 0; c < o->ncell; c++) {
        double OMEGAN = 1.5;
        double d = o->vol[c] / o->dt[c] + 0.5 * OMEGAN * o->specc[c];
        if (o->viscous) d += o->specv[c];
        o->D[c] = d;
    }
    double DF[4];
    for (int c = 0; c < o->ncell; c++) {
        double s[4] = {0, 0, 0, 0};
        for (int e = 0; e < o->cne[c]; e++) {
            solve_df(o, c, o->ce[4 * c + e], o->dW1, 1, DF);
            for (int m = 0; m < 4; m++) s[m] += DF[m];
        }
        for (int m = 0; m < 4; m++) o->dW1[4 * c + m] = (-o->R[4 * c + m] - s[m]) / o->D[c];
    }
    for (int c = o->ncell - 1; c >= 0; c--) {
        double s[4] = {0, 0, 0, 0};
        for (int e = 0; e < o->cne[c]; e++) {
            solve_df(o, c, o->ce[4 * c + e], o->dW, 0, DF);
            for (int m = 0; m < 4; m++) s[m] += DF[m];
        }
        for (int m = 0; m < 4; m++) o->dW[4 * c + m] = o->dW1[4 * c + m] - s[m] / o->D[c];
    }
    if (turb(o) && !o->turb_hold) sst_step_sweeps(o);
    for (int c = 0; c < o->ncell; c++) {
        for (int m = 0; m < 4; m++) o->W[4 * c + m] = o->W[4 * c + m] + o->dW[4 * c + m];
        prim_from_cons(o->W + 4 * c, o->U + 4 * c);
    }
    if (turb(o) && !o->turb_hold) sst_step_update(o);
    return err;
}

/* ------------------------------------------------------------------------
 * SST k-omega (SSTkomegaModel, UnstructSolver/SSTKWStrategy.h).
 *
 * The functions below restate the model's residual (:615-1013), diagonal
 * (:170-192) and eddy-viscosity update (:194-223) in the reference's operation
 * order; they are pinned to the reference's own outputs by
 * tests/test_oracle_sst.py.  The reference never runs the model (isLaminar()
 * is true), and its turbulence LU-SGS step cannot run as written, so the
 * coupled step (orc_sst_enable with coupled = 1) is the build's definition,
 * with these departures from the written code, each a defect of the dead path:
 *   - the residual is sum(Fc - Fv) - Q vol: SolveTotalTFlux (:969-1013) adds
 *     +Q vol, which with LU-SGS's dW = -R/D turns production into destruction;
 *   - SolveDF (:251-474) reads the neighbour's k, omega and their increments at
 *     [j + 2 cell] for j = 4, 5 (past the cell's own pair); the cell's pair is
 *     used;
 *   - in its right-cell branch SolveDF passes the current cell as the
 *     neighbour to SolveViscousFlux (:377), whose centre line is then zero
 *     (r_A divides by sqrt(0)); the left neighbour is passed;
 *   - k and omega are kept above 1e-4 of their freestream values after each
 *     update (the reference's clip at :206-215 is commented out);
 *   - the flow state and flow increments SolveDF reads (its extern pointers,
 *     never set by any caller) are the flow's W before the update and the
 *     flow's dW1 / dW of the same step, so the turbulence sweep follows the
 *     flow's sweeps and the update of k, omega follows the flow's update, as
 *     UpdatePrimitiveVariables asks (:196).
 * ------------------------------------------------------------------------ */
static const double sst_beta1 = 0.075, sst_beta2 = 0.0828, sst_sk1 = 0.85, sst_sk2 = 1.0, sst_sw1 = 0.5,
                    sst_sw2 = 0.856, sst_cw1 = 0.533, sst_cw2 = 0.440, sst_a1 = 0.31, sst_bstar = 0.09;

/* InitializeturbulenceVariable (:582-613) with the turbulence intensity tu
 * (the reference: 0.01) and eddy-viscosity ratio (the reference: 0.035) as
 * parameters: k = 1.5 (tu |V|)^2, omega = rho k / (ratio mu), mu_t = ratio mu. */
void orc_sst_enable(orc_t* o, int coupled, double tu, double ratio) {
    size_t c = (size_t)o->ncell, e = (size_t)o->nedge;
    if (!o->sst) {
        o->T = calloc(2 * c, 8); o->Tw = calloc(2 * c, 8); o->Tf = calloc(2 * e, 8); o->TG = calloc(4 * c, 8);
        o->F1 = calloc(c, 8); o->F2 = calloc(c, 8); o->mut = calloc(c, 8); o->mutf = calloc(e, 8);
        o->Tfc = calloc(2 * e, 8); o->Tfv = calloc(2 * e, 8); o->TR = calloc(2 * c, 8); o->TD = calloc(2 * c, 8);
        o->TdW1 = calloc(2 * c, 8); o->TdW = calloc(2 * c, 8);
    }
    o->sst = 1;
    o->coupled = coupled;
    const double R = 287.0, L = 1.0;
    double cs = sqrt(Gamma * o->pressure / o->density);
    double T = o->pressure / (R * o->density);
    double mu = 1.458e-6 * pow(T, 1.5) / (T + 110.5);
    double fs_mut = mu * ratio;
    o->sst_mut = fs_mut / mu * sqrt(Gamma) * o->mach / o->re;
    double k = 1.5 * o->mach * cs * tu * o->mach * cs * tu;
    double w = o->density * k / (ratio * mu);
    o->sst_k = Gamma * k / (cs * cs);
    o->sst_w = sqrt(Gamma) * L * w / cs;
    for (int i = 0; i < o->ncell; i++) {
        o->T[2 * i] = o->sst_k;
        o->T[2 * i + 1] = o->sst_w;
        o->mut[i] = o->sst_mut;
    }
}

/* initializeConsData (:97-109): conservative rho k, rho omega from the flow's rho */
void orc_sst_cons(orc_t* o) {
    for (int i = 0; i < o->ncell; i++) {
        double rho = o->U[4 * i];
        o->Tw[2 * i] = o->T[2 * i] * rho;
        o->Tw[2 * i + 1] = o->T[2 * i + 1] * rho;
    }
}

/* SolveTurbulenceEquation (:515-524): ComputeFaceTValue, ComputeCellTGradient,
 * ComputeSSTf1f2, ComputeTurbulenceViscousCoefficient (face loop),
 * SolveConvectiveTFlux, SolveViscousTFlux, SolveTotalTFlux, on the flow's
 * face states, gradients and laminar viscosities of the current residual. */
static void sst_equation(orc_t* o) {
    int nc = o->ncell, ne = o->nedge;
    for (int k = 0; k < ne; k++) { /* :615-659 */
        int l = o->lr[2 * k], r = o->lr[2 * k + 1];
        if (r >= 0) {
            o->Tf[2 * k] = 0.5 * (o->T[2 * l] + o->T[2 * r]);
            o->Tf[2 * k + 1] = 0.5 * (o->T[2 * l + 1] + o->T[2 * r + 1]);
        } else if (r == BC_WALL) {
            double dis = o->walld[l];
            o->Tf[2 * k] = 0.0;
            o->Tf[2 * k + 1] = 10.0 * 6.0 * o->mue[k] / (o->Ue[4 * k] * sst_beta1 * dis * dis);
        } else {
            double vn = dot2(o->Ue[4 * k + 2], o->Ue[4 * k + 3], o->nrm[2 * k], o->nrm[2 * k + 1]);
            o->Tf[2 * k] = vn > 0.0 ? o->T[2 * l] : o->sst_k;
            o->Tf[2 * k + 1] = vn > 0.0 ? o->T[2 * l + 1] : o->sst_w;
        }
    }
    memset(o->TG, 0, 4 * 8 * (size_t)nc); /* :662-692 */
    for (int k = 0; k < ne; k++) {
        int l = o->lr[2 * k], r = o->lr[2 * k + 1];
        double nx = o->nrm[2 * k], ny = o->nrm[2 * k + 1], A = o->area[k];
        for (int q = 0; q < 2; q++) {
            double a = A * o->Tf[2 * k + q];
            o->TG[4 * l + 2 * q] = o->TG[4 * l + 2 * q] + nx * a;
            o->TG[4 * l + 2 * q + 1] = o->TG[4 * l + 2 * q + 1] + ny * a;
            if (r >= 0) {
                o->TG[4 * r + 2 * q] = o->TG[4 * r + 2 * q] - nx * a;
                o->TG[4 * r + 2 * q + 1] = o->TG[4 * r + 2 * q + 1] - ny * a;
            }
        }
    }
    for (int c = 0; c < nc; c++)
        for (int q = 0; q < 4; q++) o->TG[4 * c + q] = o->TG[4 * c + q] / o->vol[c];
    for (int c = 0; c < nc; c++) { /* :695-722 */
        double gv = dot2(o->TG[4 * c], o->TG[4 * c + 1], o->TG[4 * c + 2], o->TG[4 * c + 3]);
        double rho = o->U[4 * c], dis = o->walld[c], K = o->T[2 * c], w = o->T[2 * c + 1], muL = o->mu[c];
        double cdkw = dmax(2.0 * rho * sst_sw2 / w * gv, 1.0e-20);
        double arg1 = dmax(sqrt(K) / (0.09 * w * dis), 500.0 * muL / (rho * w * dis * dis));
        arg1 = dmin(arg1, 4.0 * rho * sst_sw2 * K / (cdkw * dis * dis));
        double arg2 = dmax(2.0 * sqrt(K) / (0.09 * w * dis), 500.0 * muL / (rho * w * dis * dis));
        o->F1[c] = tanh(arg1 * arg1 * arg1 * arg1);
        o->F2[c] = tanh(arg2 * arg2);
    }
    for (int k = 0; k < ne; k++) { /* :749-777 */
        int l = o->lr[2 * k], r = o->lr[2 * k + 1];
        if (r >= 0) o->mutf[k] = 0.5 * (o->mut[l] + o->mut[r]);
        else if (r == BC_WALL) o->mutf[k] = 0.0;
        else {
            double vn = dot2(o->Ue[4 * k + 2], o->Ue[4 * k + 3], o->nrm[2 * k], o->nrm[2 * k + 1]);
            o->mutf[k] = vn > 0.0 ? o->mut[l] : o->sst_mut;
        }
    }
    for (int k = 0; k < ne; k++) { /* :783-831 and :834-920 */
        int l = o->lr[2 * k], r = o->lr[2 * k + 1];
        double nx = o->nrm[2 * k], ny = o->nrm[2 * k + 1], A = o->area[k];
        double vn = dot2(o->Ue[4 * k + 2], o->Ue[4 * k + 3], nx, ny);
        double g[2][2], ff1;
        if (r >= 0) {
            double vp = 0.5 * (vn + fabs(vn)), vs = 0.5 * (vn - fabs(vn));
            double rl = o->U[4 * l], rr = o->U[4 * r];
            o->Tfc[2 * k] = o->T[2 * l] * rl * vp * A + o->T[2 * r] * rr * vs * A;
            o->Tfc[2 * k + 1] = o->T[2 * l + 1] * rl * vp * A + o->T[2 * r + 1] * rr * vs * A;
            double l0 = o->cen[2 * r] - o->cen[2 * l], l1 = o->cen[2 * r + 1] - o->cen[2 * l + 1];
            double L2 = dot2(l0, l1, l0, l1);
            ff1 = 0.5 * (o->F1[l] + o->F1[r]);
            for (int q = 0; q < 2; q++) {
                g[q][0] = (o->TG[4 * l + 2 * q] + o->TG[4 * r + 2 * q]) * 0.5;
                g[q][1] = (o->TG[4 * l + 2 * q + 1] + o->TG[4 * r + 2 * q + 1]) * 0.5;
                double dq = o->T[2 * r + q] - o->T[2 * l + q];
                /* x first, then y with the corrected x (:857-861) */
                g[q][0] = g[q][0] + ((dq) - (g[q][0] * l0 + g[q][1] * l1)) * l0 / L2;
                g[q][1] = g[q][1] + ((dq) - (g[q][0] * l0 + g[q][1] * l1)) * l1 / L2;
            }
        } else {
            o->Tfc[2 * k] = vn * o->Ue[4 * k] * o->Tf[2 * k] * A;
            o->Tfc[2 * k + 1] = vn * o->Ue[4 * k] * o->Tf[2 * k + 1] * A;
            ff1 = o->F1[l];
            for (int q = 0; q < 2; q++) { g[q][0] = o->TG[4 * l + 2 * q]; g[q][1] = o->TG[4 * l + 2 * q + 1]; }
        }
        double sk = ff1 * sst_sk1 + (1 - ff1) * sst_sk2;
        double sw = ff1 * sst_sw1 + (1 - ff1) * sst_sw2;
        double ml = o->mue[k], mt = o->mutf[k];
        double txk = (ml + sk * mt) * g[0][0], tyk = (ml + sk * mt) * g[0][1];
        double txw = (ml + sw * mt) * g[1][0], tyw = (ml + sw * mt) * g[1][1];
        double v0 = txk * nx + tyk * ny, v1 = txw * nx + tyw * ny;
        o->Tfv[2 * k] = v0 * A;
        o->Tfv[2 * k + 1] = v1 * A;
    }
    for (int c = 0; c < nc; c++) { /* rans_P_Solver (:923-966) and SolveTotalTFlux (:969-1013) */
        const double* gr = o->grad + 8 * c;
        double ux = gr[4], uy = gr[5], vx = gr[6], vy = gr[7];
        double f1 = o->F1[c];
        double rdiv = dot2(o->TG[4 * c], o->TG[4 * c + 1], o->TG[4 * c + 2], o->TG[4 * c + 3]);
        double cw = f1 * sst_cw1 + (1.0 - f1) * sst_cw2;
        double beta = f1 * sst_beta1 + (1.0 - f1) * sst_beta2;
        double rho = o->U[4 * c], k = o->T[2 * c], w = o->T[2 * c + 1], mt = o->mut[c];
        double d0 = 2.0 / 3.0 * ((ux - vy) * (ux - vy));
        double d1 = (uy + vx) * (uy + vx);
        double d2 = 2.0 / 3.0 * rho * k * (ux + vy);
        double P = (d0 + d1) * mt - d2;
        if (o->plim > 0) P = dmin(P, o->plim * sst_bstar * rho * k * w);
        double q0 = P - sst_bstar * rho * k * w;
        double q1 = cw * rho * P / mt - beta * rho * w * w + 2 * (1 - f1) * rho * sst_sw2 / w * rdiv;
        if (o->coupled) { /* sum(Fc - Fv) - Q vol: the source with the sign of dW = -R/D */
            o->TR[2 * c] = -(q0 * o->vol[c]);
            o->TR[2 * c + 1] = -(q1 * o->vol[c]);
        } else { /* as written (:1001-1002) */
            o->TR[2 * c] = q0 * o->vol[c];
            o->TR[2 * c + 1] = q1 * o->vol[c];
        }
    }
    for (int k = 0; k < ne; k++) {
        int l = o->lr[2 * k], r = o->lr[2 * k + 1];
        for (int q = 0; q < 2; q++) {
            o->TR[2 * l + q] += o->Tfc[2 * k + q] - o->Tfv[2 * k + q];
            if (r >= 0) o->TR[2 * r + q] -= o->Tfc[2 * k + q] - o->Tfv[2 * k + q];
        }
    }
}

/* The reference's functions one by one (no coupling): SolveTurbulenceEquation
 * on the current residual's arrays. */
void orc_sst_equation(orc_t* o) { sst_equation(o); }

/* SSTkomegaModel::SolveDiag (:170-192), after SolveTime */
void orc_sst_diag(orc_t* o) {
    for (int c = 0; c < o->ncell; c++) {
        double OMEGAN = 1.5, vol = o->vol[c];
        double diag = vol / o->dt[c] + 0.5 * OMEGAN * o->specc[c] + o->specv[c];
        o->TD[2 * c] = diag + 2.0 * sst_bstar * o->T[2 * c + 1] * vol;
        double gv = dot2(o->TG[4 * c], o->TG[4 * c + 1], o->TG[4 * c + 2], o->TG[4 * c + 3]);
        double f1 = o->F1[c];
        double beta = f1 * sst_beta1 + (1 - f1) * sst_beta2;
        double w = o->T[2 * c + 1];
        o->TD[2 * c + 1] = diag + vol * fabs(2.0 * beta * w + 2.0 * sst_sw2 * (1 - f1) * gv / (w * w));
    }
}

/* initializeConsData + UpdatePrimitiveVariables (:97-109, :194-223) as the
 * reference runs them on its own conservative copy: k, omega = W / rho and
 * mu_t = a1 W_k / max(a1 W_omega / rho, F2 |dv/dx - du/dy|). */
void orc_sst_update_mut(orc_t* o) {
    for (int c = 0; c < o->ncell; c++) {
        double rho = o->U[4 * c];
        double w0 = o->T[2 * c] * rho, w1 = o->T[2 * c + 1] * rho;
        o->T[2 * c] = w0 / rho;
        o->T[2 * c + 1] = w1 / rho;
        double curl = fabs(o->grad[8 * c + 6] - o->grad[8 * c + 5]);
        double h = dmax(sst_a1 * w1 / rho, o->F2[c] * curl);
        o->mut[c] = sst_a1 * w0 / h;
    }
}

/* SSTkomegaModel::SolveDF + ConservativeParam2ConvectiveFlux + SolveViscousFlux
 * (:251-474) for cell i, face k, with the departures listed above: the
 * neighbour's flow state W_j + dW_j, its k, omega pair and increment, and the
 * neighbour passed to the viscous part on both sides. */
static void sst_solve_df(const orc_t* o, int i, int k, const double* dWf, const double* dWt, int fb, double* DF) {
    int l = o->lr[2 * k], r = o->lr[2 * k + 1];
    int j, left;
    DF[0] = 0; DF[1] = 0;
    if (i == l) {
        if (!(r >= 0 && (int)(r < l) == fb)) return;
        j = r; left = 1;
    } else {
        if (!((int)(l < r) == fb)) return;
        j = l; left = 0;
    }
    double w0[4], wp[4], t0[2], dt[2], tp[2];
    for (int m = 0; m < 4; m++) { w0[m] = o->W[4 * j + m]; wp[m] = w0[m] + dWf[4 * j + m]; }
    for (int m = 0; m < 2; m++) { t0[m] = o->Tw[2 * j + m]; dt[m] = dWt[2 * j + m]; tp[m] = t0[m] + dt[m]; }
    double nx = o->nrm[2 * k], ny = o->nrm[2 * k + 1], A = o->area[k];
    double vn0 = dot2(w0[2] / w0[0], w0[3] / w0[0], nx, ny);
    double vnp = dot2(wp[2] / wp[0], wp[3] / wp[0], nx, ny);
    const double* uj = o->U + 4 * j;
    double lx = o->cen[2 * j] - o->cen[2 * i], ly = o->cen[2 * j + 1] - o->cen[2 * i + 1];
    double vn = dot2(uj[2], uj[3], nx, ny);
    double c = sqrt(Gamma * uj[1] / uj[0]);
    double rA = 1.5 * (fabs(vn) + c);
    rA += dmax(4 / (3 * uj[0]), Gamma / uj[0]) * mpr_cell(o, i) / sqrt(dot2(lx, ly, lx, ly));
    for (int m = 0; m < 2; m++) {
        double fc = t0[m] * vn0, fcp = tp[m] * vnp;
        double dfc = left ? (fcp - fc) : (fc - fcp);
        DF[m] = 0.5 * (dfc - rA * dt[m]) * A;
    }
}

/* The turbulence LU-SGS sweeps of a coupled step (LUSGSIntegrator's serial
 * sweeps, LUSGS_Integrator.cpp:492-560, with two equations), after the flow's
 * sweeps and before its update. */
static void sst_step_sweeps(orc_t* o) {
    orc_sst_diag(o);
    double DF[2];
    for (int c = 0; c < o->ncell; c++) {
        double s[2] = {0, 0};
        for (int e = 0; e < o->cne[c]; e++) {
            sst_solve_df(o, c, o->ce[4 * c + e], o->dW1, o->TdW1, 1, DF);
            s[0] += DF[0]; s[1] += DF[1];
        }
        for (int m = 0; m < 2; m++) o->TdW1[2 * c + m] = (-o->TR[2 * c + m] - s[m]) / o->TD[2 * c + m];
    }
    for (int c = o->ncell - 1; c >= 0; c--) {
        double s[2] = {0, 0};
        for (int e = 0; e < o->cne[c]; e++) {
            sst_solve_df(o, c, o->ce[4 * c + e], o->dW, o->TdW, 0, DF);
            s[0] += DF[0]; s[1] += DF[1];
        }
        for (int m = 0; m < 2; m++) o->TdW[2 * c + m] = o->TdW1[2 * c + m] - s[m] / o->TD[2 * c + m];
    }
}

/* W_t += dW_t, then k, omega = W_t / rho with the flow's updated rho, floored
 * at 1e-4 of the freestream values, and mu_t from them (:194-223). */
static void sst_step_update(orc_t* o) {
    const double kmin = 1e-4 * o->sst_k, wmin = 1e-4 * o->sst_w;
    for (int c = 0; c < o->ncell; c++) {
        double rho = o->U[4 * c];
        double w0 = o->Tw[2 * c] + o->TdW[2 * c], w1 = o->Tw[2 * c + 1] + o->TdW[2 * c + 1];
        double k = w0 / rho, w = w1 / rho;
        if (!(k >= kmin)) { k = kmin; w0 = rho * kmin; }
        if (!(w >= wmin)) { w = wmin; w1 = rho * wmin; }
        o->Tw[2 * c] = w0;
        o->Tw[2 * c + 1] = w1;
        o->T[2 * c] = k;
        o->T[2 * c + 1] = w;
        double curl = fabs(o->grad[8 * c + 6] - o->grad[8 * c + 5]);
        double h = dmax(sst_a1 * w1 / rho, o->F2[c] * curl);
        o->mut[c] = sst_a1 * w0 / h;
    }
}

/* SST arrays by id (the CFD_FIELD_SST_* numbering of include/cfdgb.h) */
double* orc_sst_field(orc_t* o, int which) {
    switch (which) {
        case 21: return o->T;
        case 22: return o->Tf;
        case 23: return o->TG;
        case 24: return o->F1;
        case 25: return o->F2;
        case 26: return o->mut;
        case 27: return o->mutf;
        case 28: return o->Tfc;
        case 29: return o->Tfv;
        case 30: return o->TR;
        case 31: return o->TD;
        case 40: return o->Tw;
        case 41: return o->TdW1;
        case 42: return o->TdW;
        default: return 0;
    }
}

/* Wall force of the last residual evaluation (Fx, Fy): not in the reference,
 * which integrates Cp only (Euler2D.cpp:392-618). */
void orc_wall_force(orc_t* o, double* f) {
    f[0] = o->force[0];
    f[1] = o->force[1];
}

/* Field access by name id (same ids as CFD_FIELD_* in include/cfdgb.h where shared). */
double* orc_field(orc_t* o, int which) {
    switch (which) {
        case 0: return o->U;
        case 1: return o->W;
        case 2: return o->R;
        case 3: return o->grad;
        case 4: return o->phi;
        case 5: return o->specc;
        case 6: return o->specv;
        case 7: return o->dt;
        case 8: return o->D;
        case 9: return o->dW1;
        case 10: return o->dW;
        case 11: return o->gradT;
        case 12: return o->mu;
        case 13: return o->Ue;
        case 14: return o->mue;
        case 15: return o->vol;
        case 16: return o->cen;
        case 17: return o->nrm;
        case 18: return o->area;
        case 19: return o->ecen;
        case 20: return o->walld;
        case 21: return o->UL;
        case 22: return o->UR;
        case 23: return o->Wnow;
        default: return 0;
    }
}

/* ------------------------------------------------------------------------
 * Overset: interpolation weights, donor search, fringe data update.
 * ------------------------------------------------------------------------ */
#define OVS_TOL 1.0e-10 /* TOL, UniTioga/codetypes.h:54 */

/* solvec for n = 2 (mathTools/math.cpp:4-60): elimination with a row exchange
 * when the pivot is below 1e-8, then back substitution; 0 = singular. */
static int ovs_solvec2(double* a00, double* a01, double* a10, double* a11, double* b0, double* b1) {
    const double eps = 1e-8;
    double fact, sum, t;
    if (fabs(*a00) < eps) {
        if (fabs(*a10) < eps) return 0;
        t = *a00; *a00 = *a10; *a10 = t;
        t = *a01; *a01 = *a11; *a11 = t;
        t = *b0; *b0 = *b1; *b1 = t;
    }
    fact = -*a10 / *a00;
    *a10 += fact * *a00;
    *a11 += fact * *a01;
    *b1 += fact * *b0;
    if (fabs(*a11) < eps) return 0;
    sum = 0;
    *b1 = (*b1 - sum) / *a11;
    sum = 0;
    sum += *a01 * *b1;
    *b0 = (*b0 - sum) / *a00;
    return 1;
}

/* computeNodalWeight2D (math.cpp:229-312) with findClockWise (:190-227) and
 * newtonSolve2D (:126-187).  x[8] = (x0,y0,..,x3,y3).  Returns 0 for a
 * singular triangle (the reference throws). */
static int ovs_weights(int nvert, const double* x, double px, double py, double* frac) {
    int mp[4] = {0, 1, 2, 3};
    double f[4][2], p[2], u, v, uv, r0, r1, l00, l01, l10, l11, norm;
    int i, iter, ok = 1;
    frac[0] = frac[1] = frac[2] = frac[3] = 0.0;
    if (nvert == 3) {
        double a00 = x[0] - x[4], a01 = x[2] - x[4], a10 = x[1] - x[5], a11 = x[3] - x[5];
        double b0 = px - x[4], b1 = py - x[5];
        if (!ovs_solvec2(&a00, &a01, &a10, &a11, &b0, &b1)) return 0;
        frac[0] = b0;
        frac[1] = b1;
        frac[2] = 1. - frac[0] - frac[1];
        return 1;
    }
    {
        double abx = x[2] - x[0], aby = x[3] - x[1], acx = x[4] - x[0], acy = x[5] - x[1];
        double adx = x[6] - x[0], ady = x[7] - x[1];
        double zabac = abx * acy - aby * acx, zabad = abx * ady - aby * adx;
        if (zabac * zabad > 0) {
            double zacad = acx * ady - acy * adx;
            if (!(zacad * zabad > 0)) { mp[2] = 3; mp[3] = 2; }
        } else {
            mp[1] = 2;
            mp[2] = 1;
        }
    }
    p[0] = px;
    p[1] = py;
    for (i = 0; i < 2; i++) {
        f[0][i] = x[2 * mp[0] + i] - p[i];
        f[1][i] = x[2 * mp[1] + i] - x[2 * mp[0] + i];
        f[2][i] = x[2 * mp[3] + i] - x[2 * mp[0] + i];
        f[3][i] = x[2 * mp[0] + i] - x[2 * mp[1] + i] + x[2 * mp[2] + i] - x[2 * mp[3] + i];
    }
    u = v = 0.5;
    for (iter = 0; iter < 500; iter++) {
        uv = u * v;
        r0 = f[0][0] + f[1][0] * u + f[2][0] * v + f[3][0] * uv;
        r1 = f[0][1] + f[1][1] * u + f[2][1] * v + f[3][1] * uv;
        norm = r0 * r0 + r1 * r1;
        if (sqrt(norm) <= 1e-14) break;
        l00 = f[1][0] + f[3][0] * v;
        l01 = f[2][0] + f[3][0] * u;
        l10 = f[1][1] + f[3][1] * v;
        l11 = f[2][1] + f[3][1] * u;
        if (!ovs_solvec2(&l00, &l01, &l10, &l11, &r0, &r1)) { ok = 0; break; }
        u -= r0 * 1.0;
        v -= r1 * 1.0;
    }
    if (iter == 500 || !ok) { u = 2.0; v = 0.0; }
    frac[mp[0]] = (1 - u) * (1 - v);
    frac[mp[1]] = u * (1 - v);
    frac[mp[2]] = u * v;
    frac[mp[3]] = (1 - u) * v;
    return 1;
}

/* Weights of n (cell, point) pairs; returns the number of singular triangles
 * (their frac is -1e300). */
long orc_nodal_weights(long n, const int* nvert, const double* xv, const double* xp, double* frac) {
    long i, bad = 0;
    for (i = 0; i < n; i++) {
        if (!ovs_weights(nvert[i], xv + 8 * i, xp[2 * i], xp[2 * i + 1], frac + 4 * i)) {
            frac[4 * i] = frac[4 * i + 1] = frac[4 * i + 2] = frac[4 * i + 3] = -1e300;
            bad++;
        }
    }
    return bad;
}

/* Containment of MeshBlock::search by brute force: for every point, every cell
 * whose TOL-widened box holds it (recursiveADT.cpp:117-124) and whose weights
 * lie in [-TOL, 1+TOL] (checkContainment.cpp:41-46) contains it.  donor[i] =
 * the lowest such cell (-1 if none), ncontain[i] = how many there are,
 * w[4*i] = the donor's weights.  cverts[4*c] are 0-based, -1 padded. */
void orc_donor_search(const double* xy, int ncell, const int* cverts, const int* nvert, long npts,
                      const double* pts, int* donor, int* ncontain, double* w) {
    long i;
    int c, m;
    for (i = 0; i < npts; i++) {
        double px = pts[2 * i], py = pts[2 * i + 1];
        donor[i] = -1;
        ncontain[i] = 0;
        w[4 * i] = w[4 * i + 1] = w[4 * i + 2] = w[4 * i + 3] = 0.0;
        for (c = 0; c < ncell; c++) {
            double x[8], f[4], xmin = 1.0e15, ymin = 1.0e15, xmax = -1.0e15, ymax = -1.0e15;
            int nv = nvert[c], inside = 1;
            for (m = 0; m < 4; m++) {
                int id = m < nv ? cverts[4 * c + m] : cverts[4 * c + 2];
                x[2 * m] = xy[2 * id];
                x[2 * m + 1] = xy[2 * id + 1];
                if (m < nv) {
                    xmin = xmin < x[2 * m] ? xmin : x[2 * m];
                    ymin = ymin < x[2 * m + 1] ? ymin : x[2 * m + 1];
                    xmax = xmax > x[2 * m] ? xmax : x[2 * m];
                    ymax = ymax > x[2 * m + 1] ? ymax : x[2 * m + 1];
                }
            }
            if (!(px >= xmin - OVS_TOL && py >= ymin - OVS_TOL && px <= xmax + OVS_TOL && py <= ymax + OVS_TOL))
                continue;
            if (!ovs_weights(nv, x, px, py, f)) continue;
            for (m = 0; m < nv; m++)
                if ((f[m] + OVS_TOL) * (f[m] - 1.0 - OVS_TOL) > 0) inside = 0;
            if (!inside) continue;
            if (donor[i] < 0) {
                donor[i] = c;
                for (m = 0; m < 4; m++) w[4 * i + m] = f[m];
            }
            ncontain[i]++;
        }
    }
}

/* ---- MeshBlock::search as the reference runs it (UniTioga/search.cpp:81-270),
 * for the parity of the donor choice where several cells contain a point.
 * Literal restatement: the oriented box of the query points (findOBB,
 * UniTioga/utils.cpp:43-291, with Kaiser's eigen-solver, mathTools/kaiser.cpp:
 * 9-160), the cells whose boxes cross it pushed on a LIFO list, the
 * alternating digital tree over their axis-aligned boxes (ADT::buildADT,
 * ADT.cpp:15-91, buildADTrecursion, recursiveADT.cpp:8-109, median split of
 * mathTools/median.cpp:5-240), the coincident-point hash (uniquenodes_octree,
 * utils.cpp:484-643) and the recursive walk (searchIntersections,
 * recursiveADT.cpp:111-156, with checkContainment, checkContainment.cpp:4-62).
 * 2D only (d_dim = 2, ndim = 4). */
#define OVS_BIG 1.0e+15 /* BIGVALUE, UniTioga/codetypes.h:52 */

/* Jacobi rotations of kaiser() for a 2x2 matrix a (columns rotated in place),
 * then the columns normalised by their lengths. */
static void ovs_kaiser2(double a[2][2]) {
    const int n = 2;
    double ss = 0, eps, ev[2];
    int i, j, k, it;
    for (i = 0; i < n; i++)
        for (j = 0; j < n; j++) ss += a[i][j] * a[i][j];
    eps = 1.0e-12 * ss / n;
    for (it = 0; it < 100; it++) {
        int skip = 0;
        for (i = 0; i < n - 1; i++)
            for (j = i + 1; j < n; j++) {
                double halfp = 0, q = 0, p, absp, absq, t, c, s, tmp;
                for (k = 0; k < n; k++) {
                    halfp += a[k][i] * a[k][j];
                    q += (a[k][i] + a[k][j]) * (a[k][i] - a[k][j]);
                }
                p = 2 * halfp;
                absp = fabs(p);
                if (absp < eps && q >= 0) {
                    skip++;
                    continue;
                }
                absq = fabs(q);
                if (absp <= absq) {
                    t = absp / absq;
                    c = 1 / sqrt(1 + t * t);
                    s = t * c;
                } else {
                    t = absq / absp;
                    s = 1 / sqrt(1 + t * t);
                    c = s * t;
                }
                c = sqrt((1 + c) / 2);
                s = s / (2 * c);
                if (q < 0) {
                    tmp = c;
                    c = s;
                    s = tmp;
                }
                if (p < 0) s = -s;
                for (k = 0; k < n; k++) {
                    tmp = a[k][i];
                    a[k][i] = tmp * c + a[k][j] * s;
                    a[k][j] = -tmp * s + a[k][j] * c;
                }
            }
        if (skip == 0.5 * n * (n - 1)) break;
    }
    for (i = 0; i < n; i++) {
        double t = 0;
        for (j = 0; j < n; j++) t += a[j][i] * a[j][i];
        ev[i] = sqrt(t);
    }
    for (i = 0; i < n; i++)
        for (j = 0; j < n; j++) a[j][i] = ev[i] > 0 ? a[j][i] / ev[i] : 0;
}

/* findOBB in 2D: centre xc, half extents dxc, basis vec (rows). */
static void ovs_find_obb(const double* x, long nn, double xc[2], double dxc[2], double vec[2][2]) {
    double aa[2][2] = {{0, 0}, {0, 0}}, xmin[2], xmax[2], xd[2];
    long i;
    int j, k;
    xc[0] = xc[1] = 0;
    for (i = 0; i < nn; i++)
        for (j = 0; j < 2; j++) xc[j] += x[2 * i + j];
    for (j = 0; j < 2; j++) xc[j] = xc[j] / nn;
    if (nn <= 2) {
        vec[0][0] = vec[1][1] = 1;
        vec[0][1] = vec[1][0] = 0;
        for (j = 0; j < 2; j++) {
            if (nn == 1) {
                dxc[j] = 1e-3;
            } else {
                /* TIOGA_MAX(1e-3, d) * 0.5 expands to 1e-3 > d ? 1e-3 : d * 0.5 (the macro has no outer
                 * parentheses) */
                double d = fabs(x[2 + j] - x[j]);
                dxc[j] = 1e-3 > d ? 1e-3 : d * 0.5;
            }
        }
        return;
    }
    for (i = 0; i < nn; i++)
        for (j = 0; j < 2; j++)
            for (k = j; k < 2; k++) aa[j][k] += (x[2 * i + j] - xc[j]) * (x[2 * i + k] - xc[k]);
    aa[1][0] = aa[0][1];
    ovs_kaiser2(aa);
    for (j = 0; j < 2; j++) {
        vec[j][0] = aa[j][0];
        vec[j][1] = aa[j][1];
        xmax[j] = -OVS_BIG;
        xmin[j] = OVS_BIG;
    }
    for (i = 0; i < nn; i++) {
        xd[0] = xd[1] = 0;
        for (j = 0; j < 2; j++)
            for (k = 0; k < 2; k++) xd[j] += (x[2 * i + k] - xc[k]) * vec[j][k];
        for (j = 0; j < 2; j++) {
            xmax[j] = xmax[j] > xd[j] ? xmax[j] : xd[j];
            xmin[j] = xmin[j] < xd[j] ? xmin[j] : xd[j];
        }
    }
    for (j = 0; j < 2; j++) {
        dxc[j] = (xmax[j] - xmin[j]) * 0.5 * 1.01;
        xd[j] = (xmax[j] + xmin[j]) * 0.5;
    }
    for (j = 0; j < 2; j++)
        for (k = 0; k < 2; k++) xc[j] += xd[k] * vec[k][j];
}

static void ovs_swap(int* ix, double* x, int a, int b) {
    double t = x[a];
    int u = ix[a];
    x[a] = x[b];
    x[b] = t;
    ix[a] = ix[b];
    ix[b] = u;
}

/* find_median (mathTools/median.cpp:5-190): partial partition of x[*ilow..*ihigh]
 * about a clamped middle value, recursing on the side that holds the median
 * position; *ilow / *ihigh are updated as the reference's references are. */
static void ovs_find_median(int* ix, double* x, int n, int* ilow, int* ihigh) {
    int low = *ilow, high = *ihigh, mid = (low + high) / 2, nby2 = (n - 1) / 2, nby2p1 = (n - 1) / 2 + 1;
    int odd = n % 2 == 1, i, j, signal = 1;
    double xlow = x[low], xhigh = x[high], xmed = x[mid];
    if (xlow > xhigh) {
        double t = xlow;
        xlow = xhigh;
        xhigh = t;
    }
    if (xmed > xhigh) xmed = xhigh;
    else if (xmed < xlow) xmed = xlow;
    i = low;
    j = high;
    while (signal) {
        signal = 0;
        while (!(x[i] >= xmed)) ++i;
        while (!(x[j] <= xmed)) --j;
        if (i < j) {
            ovs_swap(ix, x, i, j);
            i = i + 1;
            j = j - 1;
            if (i <= j) signal = 1;
        }
    }
    if (!odd) {
        if (j == nby2 && i == nby2p1) {
            int idx = j, k;
            for (k = 0; k < nby2; k++)
                if (x[k] > x[idx]) idx = k;
            if (idx != j) ovs_swap(ix, x, idx, j);
            return;
        }
        if (j < nby2) low = i;
        if (i > nby2p1) high = j;
        if (i != j) {
            if (low < high - 1) ovs_find_median(ix, x, n, &low, &high);
            return;
        }
        if (i == nby2) low = nby2;
        if (j == nby2p1) high = nby2p1;
    } else {
        if (j < nby2) low = i;
        if (i > nby2) high = j;
        if (i != j) {
            if (low < high - 1) ovs_find_median(ix, x, n, &low, &high);
            *ilow = low;
            *ihigh = high;
            return;
        }
        if (i == nby2) {
            *ilow = low;
            *ihigh = high;
            return;
        }
    }
    if (low < high - 1) {
        *ilow = low;
        *ihigh = high;
        ovs_find_median(ix, x, n, &low, &high);
    }
}

/* find_median_wrap (median.cpp:192-240) */
static void ovs_median_wrap(int* ix, double* x, int n) {
    int ilow = 0, ihigh = n - 1, nby2 = (n - 1) / 2;
    if (n <= 2) {
        if (n == 2 && x[0] > x[1]) ovs_swap(ix, x, 0, 1);
        return;
    }
    ovs_find_median(ix, x, n, &ilow, &ihigh);
    if (n % 2 == 0) {
        if (x[nby2] > x[nby2 + 1]) ovs_swap(ix, x, nby2, nby2 + 1);
    } else if (x[ilow] > x[ihigh]) {
        ovs_swap(ix, x, ilow, ihigh);
    }
}

typedef struct {
    int ndim, nelem;
    const double* coord; /* per element: min x, min y, max x, max y */
    int* ints;           /* 4 per node: element, left child element, right child element, (node of element) */
    double* reals;       /* ndim per node: the subtree's box */
    double ext[4];       /* adtExtents: min x, max x, min y, max y, widened by 1% */
    int count;
} OvsAdt;

/* buildADTrecursion */
static void ovs_adt_rec(OvsAdt* t, double* work, int* avail, int side, int parent, int level, int nav) {
    const int ndim = t->ndim, nd = ndim / 2;
    int i, j;
    if (nav > 1) {
        int dimcut = level % ndim, nleft, node;
        for (i = 0; i < nav; i++) work[i] = t->coord[ndim * avail[i] + dimcut];
        ovs_median_wrap(avail, work, nav);
        nleft = (nav + 1) / 2;
        node = ++t->count;
        t->ints[4 * node] = avail[nleft - 1];
        t->ints[4 * node + 1] = t->ints[4 * node + 2] = t->ints[4 * node + 3] = -1;
        for (j = 0; j < nd; j++) {
            t->reals[ndim * node + j] = OVS_BIG;
            t->reals[ndim * node + j + nd] = -OVS_BIG;
        }
        for (i = 0; i < nav; i++)
            for (j = 0; j < nd; j++) {
                double lo = t->coord[ndim * avail[i] + j], hi = t->coord[ndim * avail[i] + j + nd];
                double* r = t->reals + ndim * node;
                r[j] = r[j] < lo ? r[j] : lo;
                r[j + nd] = r[j + nd] > hi ? r[j + nd] : hi;
            }
        if (side > 0) t->ints[4 * parent + side] = avail[nleft - 1];
        if (nleft > 1) ovs_adt_rec(t, work, avail, 1, node, level + 1, nleft - 1);
        ovs_adt_rec(t, work, avail + nleft, 2, node, level + 1, nav - nleft);
    } else if (nav == 1) {
        int node = ++t->count;
        t->ints[4 * node] = avail[0];
        t->ints[4 * node + 1] = t->ints[4 * node + 2] = t->ints[4 * node + 3] = -1;
        for (j = 0; j < ndim; j++) t->reals[ndim * node + j] = t->coord[ndim * avail[0] + j];
        if (side > 0) t->ints[4 * parent + side] = avail[0];
    }
}

/* ADT::buildADT */
static void ovs_adt_build(OvsAdt* t, int nelem, const double* coord) {
    int i, j;
    int* avail = (int*)malloc(sizeof(int) * (size_t)(nelem > 0 ? nelem : 1));
    double* work = (double*)malloc(sizeof(double) * (size_t)(nelem > 0 ? nelem : 1));
    t->ndim = 4;
    t->nelem = nelem;
    t->coord = coord;
    t->ints = (int*)malloc(sizeof(int) * 4 * (size_t)(nelem > 0 ? nelem : 1));
    t->reals = (double*)malloc(sizeof(double) * 4 * (size_t)(nelem > 0 ? nelem : 1));
    for (i = 0; i < 2; i++) {
        t->ext[2 * i] = OVS_BIG;
        t->ext[2 * i + 1] = -OVS_BIG;
    }
    for (j = 0; j < nelem; j++)
        for (i = 0; i < 2; i++) {
            double lo = coord[4 * j + i], hi = coord[4 * j + i + 2];
            t->ext[2 * i] = t->ext[2 * i] < lo ? t->ext[2 * i] : lo;
            t->ext[2 * i + 1] = t->ext[2 * i + 1] > hi ? t->ext[2 * i + 1] : hi;
        }
    for (i = 0; i < 2; i++) {
        double delta = 0.01 * (t->ext[2 * i + 1] - t->ext[2 * i]);
        t->ext[2 * i] -= delta;
        t->ext[2 * i + 1] += delta;
    }
    for (i = 0; i < nelem; i++) avail[i] = i;
    t->count = -1;
    ovs_adt_rec(t, work, avail, 0, 0, 0, nelem);
    for (i = 0; i < nelem; i++) t->ints[4 * t->ints[4 * i] + 3] = i;
    free(avail);
    free(work);
}

typedef struct {
    const double* xy;
    const int* cverts;   /* mesh cell order, 4 per cell, 0-based */
    const int* nvert;
    const int* order;    /* MeshBlock cell -> mesh cell (triangles first, then quadrilaterals) */
    const unsigned char* unaccept; /* per mesh cell: cellRes == BIGVALUE */
    const int* elist;    /* ADT element -> MeshBlock cell */
} OvsBlk;

/* checkContainment: ci[0] = the MeshBlock cell or -1, ci[1] = 1 for a
 * containing cell with a vanishing weight that may not donate. */
static void ovs_check(const OvsBlk* b, int* ci, int elem, const double* p) {
    const int icell = b->elist[elem], c = b->order[icell], nv = b->nvert[c];
    double x[8], f[4];
    int m;
    for (m = 0; m < 4; m++) {
        const int id = m < nv ? b->cverts[4 * c + m] : b->cverts[4 * c + 2];
        x[2 * m] = b->xy[2 * id];
        x[2 * m + 1] = b->xy[2 * id + 1];
    }
    ci[0] = icell;
    ci[1] = 0;
    if (!ovs_weights(nv, x, p[0], p[1], f)) { /* the reference throws here; taken as no containment */
        ci[0] = -1;
        return;
    }
    for (m = 0; m < nv; m++) {
        if ((f[m] + OVS_TOL) * (f[m] - 1.0 - OVS_TOL) > 0) {
            ci[0] = -1;
            return;
        }
        if (fabs(f[m]) < OVS_TOL && b->unaccept[c]) ci[1] = 1;
    }
}

static int ovs_in_box(const double* p, const double* e) {
    return p[0] >= e[0] - OVS_TOL && p[1] >= e[1] - OVS_TOL && p[0] <= e[2] + OVS_TOL && p[1] <= e[3] + OVS_TOL;
}

/* searchIntersections */
static void ovs_adt_walk(const OvsAdt* t, const OvsBlk* b, int* ci, int node, const double* p) {
    int d;
    if (ovs_in_box(p, t->coord + 4 * t->ints[4 * node])) {
        ovs_check(b, ci, t->ints[4 * node], p);
        if (ci[0] > -1 && ci[1] == 0) return;
    }
    for (d = 1; d < 3; d++) {
        int child = t->ints[4 * node + d];
        if (child > -1) {
            child = t->ints[4 * child + 3];
            if (ovs_in_box(p, t->reals + 4 * child)) {
                ovs_adt_walk(t, b, ci, child, p);
                if (ci[0] > -1 && ci[1] == 0) return;
            }
        }
    }
}

/* uniqNodesTree: coincident points (L1 distance below TOL, same tag) share
 * one itag; rtag takes the larger resolution. */
static void ovs_uniq_tree(const double* x, int* itag, double* rtag, const int* tag, int* avail, int nav) {
    int icheck = 1, i, j;
    if (nav > 20) {
        double xmin[2] = {OVS_BIG, OVS_BIG}, xmax[2] = {-OVS_BIG, -OVS_BIG}, xmid[2], dx[2];
        int npts[4] = {0, 0, 0, 0}, cft[5];
        icheck = 0;
        for (i = 0; i < nav; i++)
            for (j = 0; j < 2; j++) {
                const double v = x[2 * avail[i] + j];
                xmin[j] = xmin[j] < v ? xmin[j] : v;
                xmax[j] = xmax[j] > v ? xmax[j] : v;
            }
        for (j = 0; j < 2; j++) {
            xmid[j] = (xmax[j] + xmin[j]) * 0.5;
            dx[j] = (xmax[j] - xmin[j]) * 0.5 + OVS_TOL;
        }
#define OVS_IBOX(q) (2 * ((int)floor((x[2 * (q)] - xmid[0]) / dx[0]) + 1) + ((int)floor((x[2 * (q) + 1] - xmid[1]) / dx[1]) + 1))
        for (i = 0; i < nav; i++) npts[OVS_IBOX(avail[i])]++;
        for (j = 0; j < 4; j++)
            if (npts[j] == nav) icheck = 1;
        if (!icheck) {
            int* tmp = (int*)malloc(sizeof(int) * (size_t)nav);
            cft[0] = 0;
            for (j = 0; j < 4; j++) cft[j + 1] = cft[j] + npts[j];
            for (i = 0; i < nav; i++) {
                const int ib = OVS_IBOX(avail[i]);
                npts[ib]--;
                tmp[npts[ib] + cft[ib]] = avail[i];
            }
            memcpy(avail, tmp, sizeof(int) * (size_t)nav);
            free(tmp);
            for (j = 0; j < 4; j++)
                if (cft[j + 1] > cft[j]) ovs_uniq_tree(x, itag, rtag, tag, avail + cft[j], cft[j + 1] - cft[j]);
        }
#undef OVS_IBOX
    }
    if (icheck)
        for (i = 0; i < nav; i++) {
            const int p1 = avail[i];
            for (j = i + 1; j < nav; j++) {
                const int p2 = avail[j];
                if (fabs(x[2 * p1] - x[2 * p2]) + fabs(x[2 * p1 + 1] - x[2 * p2 + 1]) < OVS_TOL && tag[p1] == tag[p2]) {
                    if (p1 > p2) {
                        rtag[p2] = rtag[p1] > rtag[p2] ? rtag[p1] : rtag[p2];
                        itag[p1] = itag[p2];
                    } else {
                        rtag[p1] = rtag[p1] > rtag[p2] ? rtag[p1] : rtag[p2];
                        itag[p2] = itag[p1];
                    }
                }
            }
        }
}

/* MeshBlock::search of npts points (tags per point, resolutions rtag merged in
 * place over coincident points) in a block whose cells are given in mesh
 * order; unaccept[c] marks the cells whose cellRes is BIGVALUE.  donor[i] =
 * the mesh cell (-1: none), xtag[i] = the point whose search it took. */
void orc_adt_search(const double* xy, int ncell, const int* cverts, const int* nvert, const unsigned char* unaccept,
                    long npts, const double* pts, const int* tags, double* rtag, int* donor, int* xtag) {
    OvsBlk b;
    OvsAdt t;
    double xc[2], dxc[2], vec[2][2], *bbox;
    int *order, *icell, *elist, *avail, iptr = -1, count = 0, p, k, l, nt = 0;
    long i;
    if (npts <= 0) return;
    order = (int*)malloc(sizeof(int) * (size_t)(ncell > 0 ? ncell : 1));
    for (k = 0; k < 2; k++)
        for (p = 0; p < ncell; p++)
            if ((nvert[p] == 3) == (k == 0)) order[nt++] = p;
    ovs_find_obb(pts, npts, xc, dxc, vec);
    icell = (int*)malloc(sizeof(int) * (size_t)(ncell > 0 ? ncell : 1));
    for (p = 0; p < ncell; p++) {
        const int c = order[p], nv = nvert[c];
        double xmn[2] = {OVS_BIG, OVS_BIG}, xmx[2] = {-OVS_BIG, -OVS_BIG}, xd[2] = {0, 0}, dx[2] = {0, 0};
        int m, j, q, cross = 1;
        icell[p] = -1;
        for (m = 0; m < nv; m++) {
            const int id = cverts[4 * c + m];
            for (j = 0; j < 2; j++) {
                xd[j] = 0;
                for (q = 0; q < 2; q++) xd[j] += (xy[2 * id + q] - xc[q]) * vec[j][q];
                xmn[j] = xmn[j] < xd[j] ? xmn[j] : xd[j];
                xmx[j] = xmx[j] > xd[j] ? xmx[j] : xd[j];
            }
            for (j = 0; j < 2; j++) {
                xd[j] = (xmx[j] + xmn[j]) * 0.5;
                dx[j] = (xmx[j] - xmn[j]) * 0.5;
            }
        }
        for (j = 0; j < 2; j++) cross = cross && (fabs(xd[j]) <= dx[j] + dxc[j]);
        if (cross) {
            icell[p] = iptr;
            iptr = p;
            count++;
        }
    }
    bbox = (double*)malloc(sizeof(double) * 4 * (size_t)(count > 0 ? count : 1));
    elist = (int*)malloc(sizeof(int) * (size_t)(count > 0 ? count : 1));
    for (k = iptr, l = 0; k != -1; k = icell[k], l++) {
        const int c = order[k], nv = nvert[c];
        double xmn[2] = {OVS_BIG, OVS_BIG}, xmx[2] = {-OVS_BIG, -OVS_BIG};
        int m, j;
        for (m = 0; m < nv; m++)
            for (j = 0; j < 2; j++) {
                const double v = xy[2 * cverts[4 * c + m] + j];
                xmn[j] = xmn[j] < v ? xmn[j] : v;
                xmx[j] = xmx[j] > v ? xmx[j] : v;
            }
        bbox[4 * l] = xmn[0];
        bbox[4 * l + 1] = xmn[1];
        bbox[4 * l + 2] = xmx[0];
        bbox[4 * l + 3] = xmx[1];
        elist[l] = k;
    }
    ovs_adt_build(&t, count, bbox);
    b.xy = xy;
    b.cverts = cverts;
    b.nvert = nvert;
    b.order = order;
    b.unaccept = unaccept;
    b.elist = elist;
    avail = (int*)malloc(sizeof(int) * (size_t)npts);
    for (i = 0; i < npts; i++) avail[i] = (int)i, xtag[i] = (int)i;
    ovs_uniq_tree(pts, xtag, rtag, tags, avail, (int)npts);
    for (i = 0; i < npts; i++) {
        if (xtag[i] == i) {
            int ci[2] = {-1, 0};
            const double* q = pts + 2 * i;
            if (q[0] >= t.ext[0] - OVS_TOL && q[1] >= t.ext[2] - OVS_TOL && q[0] <= t.ext[1] + OVS_TOL &&
                q[1] <= t.ext[3] + OVS_TOL && count > 0)
                ovs_adt_walk(&t, &b, ci, 0, q);
            donor[i] = ci[0] < 0 ? -1 : order[ci[0]];
        } else {
            donor[i] = donor[xtag[i]];
        }
    }
    free(avail);
    free(t.ints);
    free(t.reals);
    free(bbox);
    free(elist);
    free(icell);
    free(order);
}

/* getInterpolatedSolution + updateSolnData (UniTioga/dataUpdate.cpp:6-132):
 * receptor i gets sum_m q[inode[4i+m]] * w[4i+m] (m < nw[i], from 0, in list
 * order) and writes it to node recv[i] of qr, records in list order; layout 0
 * = ROW q[node*nvar+k], 1 = COLUMN q[k*nnodes+node]. */
void orc_interp_update(long n, const int* recv, const int* nw, const int* inode, const double* w,
                       const double* q, long nnodes, double* qr, long nnodes_recv, int nvar, int layout) {
    long i;
    int k, m;
    double* vals = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1) * (size_t)nvar);
    for (i = 0; i < n; i++)
        for (k = 0; k < nvar; k++) {
            double qq = 0;
            for (m = 0; m < nw[i]; m++) {
                long node = inode[4 * i + m];
                double qv = layout == 0 ? q[node * nvar + k] : q[(long)k * nnodes + node];
                qq += qv * w[4 * i + m];
            }
            vals[i * nvar + k] = qq;
        }
    for (i = 0; i < n; i++)
        for (k = 0; k < nvar; k++) {
            if (layout == 0) qr[(long)recv[i] * nvar + k] = vals[i * nvar + k];
            else qr[(long)k * nnodes_recv + recv[i]] = vals[i * nvar + k];
        }
    free(vals);
}

/* Hole map of one block's walls, 2D: tioga::getHoleMap (holeMap.cpp:7-180)
 * for a single block, MeshBlock::getWallBounds (MeshBlock.cpp:653-685),
 * markWallBoundary (:687-778) and fillHoleMap2D (utils.cpp:782-860).
 * wall_nodes: 0-based ids.  geo[4] = {xmin, ymin, xmax, ymax} of the map,
 * nxy[2] its size; sam (capacity cap) receives nx*ny ints.  Returns 0, or -1
 * when sam is too small. */
int orc_holemap(const double* xy, int ncell, const int* cverts, const int* nvert, int nwall, const int* wall_nodes,
                int isym, int* nxy, double* geo, int* sam, long cap) {
    double wb[4] = {1.0e15, 1.0e15, -1.0e15, -1.0e15}, ds[2], dsmax, dsbox;
    int i, j, k, c, m, jj, nx[2];
    unsigned char* isw;
    long n, nnode_max = 0;
    for (i = 0; i < nwall; i++) {
        const double* p = xy + 2 * wall_nodes[i];
        for (j = 0; j < 2; j++) {
            wb[j] = wb[j] < p[j] ? wb[j] : p[j];
            wb[2 + j] = wb[2 + j] > p[j] ? wb[2 + j] : p[j];
        }
        if (wall_nodes[i] + 1 > nnode_max) nnode_max = wall_nodes[i] + 1;
    }
    for (j = 0; j < 2; j++) ds[j] = wb[2 + j] - wb[j];
    dsmax = ds[0] > ds[1] ? ds[0] : ds[1];
    dsbox = dsmax / 192;
    for (j = 0; j < 2; j++) {
        double r;
        wb[j] -= (2 * dsbox);
        wb[2 + j] += (2 * dsbox);
        r = (wb[2 + j] - wb[j]) / dsbox;
        nx[j] = (int)floor(r > 1 ? r : 1);
    }
    nxy[0] = nx[0];
    nxy[1] = nx[1];
    for (j = 0; j < 4; j++) geo[j] = wb[j];
    n = (long)nx[0] * nx[1];
    if (n > cap) return -1;
    for (i = 0; i < n; i++) sam[i] = 0;
    for (c = 0; c < ncell; c++)
        for (m = 0; m < nvert[c]; m++)
            if (cverts[4 * c + m] + 1 > nnode_max) nnode_max = cverts[4 * c + m] + 1;
    isw = (unsigned char*)calloc((size_t)nnode_max, 1);
    for (i = 0; i < nwall; i++) isw[wall_nodes[i]] = 1;
    for (k = 0; k < 2; k++) ds[k] = (wb[2 + k] - wb[k]) / nx[k];
    for (c = 0; c < ncell; c++) {
        int wall = 0, imin[2] = {2147483647, 2147483647}, imax[2] = {-2147483647, -2147483647}, ii;
        for (m = 0; m < nvert[c]; m++)
            if (isw[cverts[4 * c + m]]) { wall = 1; break; }
        if (!wall) continue;
        for (m = 0; m < nvert[c]; m++)
            for (k = 0; k < 2; k++) {
                int iv = (int)floor((xy[2 * cverts[4 * c + m] + k] - wb[k]) / ds[k]);
                imin[k] = imin[k] < iv ? imin[k] : iv;
                imax[k] = imax[k] > iv ? imax[k] : iv;
            }
        for (k = 0; k < 2; k++) {
            imin[k] = imin[k] > 0 ? imin[k] : 0;
            imax[k] = imax[k] < nx[k] - 1 ? imax[k] : nx[k] - 1;
        }
        for (jj = imin[1]; jj < imax[1] + 1; jj++)
            for (ii = imin[0]; ii < imax[0] + 1; ii++) sam[jj * nx[0] + ii] = 2;
    }
    free(isw);
    /* flood fill from the border, sweep by sweep in row order */
    for (jj = 0; jj < nx[1]; jj += nx[1] - 1)
        for (i = 0; i < nx[0]; i++) sam[jj * nx[0] + i] = 1;
    for (jj = 0; jj < nx[1]; jj++)
        for (i = 0; i < nx[0]; i += nx[0] - 1) sam[jj * nx[0] + i] = 1;
    {
        long npaint = 1;
        while (npaint > 0) {
            npaint = 0;
            for (j = 1; j < nx[1] - 1; j++)
                for (i = 1; i < nx[0] - 1; i++) {
                    int mm = j * nx[0] + i, p;
                    if (sam[mm] != 0) continue;
                    if (isym == 1) p = sam[mm - nx[0]] == 1 || sam[mm + nx[0]] == 1;
                    else if (isym == 2) p = sam[mm - 1] == 1 || sam[mm + 1] == 1;
                    else p = sam[mm - nx[0]] == 1 || sam[mm + nx[0]] == 1 || sam[mm - 1] == 1 || sam[mm + 1] == 1;
                    if (p) { sam[mm] = 1; npaint++; }
                }
        }
    }
    for (i = 0; i < n; i++) sam[i] = (sam[i] == 0 || sam[i] == 2);
    return 0;
}

/* checkHoleMap (utils.cpp:645-670) for n points. */
void orc_holemap_check(const int* nxy, const double* geo, const int* sam, long n, const double* pts, int* inside) {
    long i;
    int k;
    double dx[2];
    for (k = 0; k < 2; k++) dx[k] = (geo[2 + k] - geo[k]) / nxy[k];
    for (i = 0; i < n; i++) {
        int ix[2], out = 0;
        for (k = 0; k < 2; k++) {
            ix[k] = (int)((pts[2 * i + k] - geo[k]) / dx[k]);
            if (ix[k] < 0 || ix[k] > nxy[k] - 1) out = 1;
        }
        inside[i] = out ? 0 : sam[ix[1] * nxy[0] + ix[0]];
    }
}

/* Analysis switches, for separating what keeps an iteration from converging:
 * orc_hold_limiter(o, 1) freezes the Venkatakrishnan factors at their current
 * values (every later residual uses them; 0 releases them), and
 * orc_hold_turbulence(o, 1) freezes k, omega and mu_t (the coupled step skips
 * the model's sweeps and update; the flow still sees the held mu_t). */
void orc_hold_limiter(orc_t* o, int on) {
    if (on) {
        if (!o->phi_hold) o->phi_hold = malloc(4 * 8 * (size_t)o->ncell);
        if (o->phi_hold) memcpy(o->phi_hold, o->phi, 4 * 8 * (size_t)o->ncell);
    } else {
        free(o->phi_hold);
        o->phi_hold = NULL;
    }
}

void orc_hold_turbulence(orc_t* o, int on) { o->turb_hold = on != 0; }

/* The k equation's production limited to factor * beta* rho k omega (Menter's
 * SST guard at stagnation points; factor 0 restores the reference's unlimited
 * production).  Analysis only: it departs from the reference's model. */
void orc_sst_production_limit(orc_t* o, double factor) { o->plim = factor > 0 ? factor : 0; }
