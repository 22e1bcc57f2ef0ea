/*
 * cfdgb.h - C ABI of the GB300 (sm_103a) unstructured finite-volume hot path.
 *
 * The library replaces the per-iteration path of the reference solver
 * (SenhuWong/tmp, src/UnstructSolver + the per-iteration part of src/UniTioga):
 * residual evaluation, local time step, 5-stage Runge-Kutta and LU-SGS
 * stepping, residual norms, and the overset fringe data update.  Every
 * function returns an int status (CFD_OK == 0, negative on error) and leaves
 * a message for cfd_last_error().  All device memory belongs to the handles.
 * Calls on one case handle are issued on that case's stream and are not
 * thread-safe for the same handle; different handles may be used from
 * different threads.  No signature uses a framework type.
 */
#ifndef CFDGB_H
#define CFDGB_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define CFD_OK               0
#define CFD_ERR_ARG         -1  /* bad argument (null pointer, size, enum)         */
#define CFD_ERR_IO          -2  /* mesh file missing or unreadable                  */
#define CFD_ERR_MESH        -3  /* topology the solver cannot use (bad BC tag ...)  */
#define CFD_ERR_CUDA        -4  /* CUDA runtime failure; message has the CUDA text  */
#define CFD_ERR_PSTAR       -5  /* HLLC |p*_L - p*_R| >= 1e-10 on some face         */
#define CFD_ERR_NONPHYSICAL -6  /* NaN or non-positive density/pressure             */
#define CFD_ERR_TIMEOUT     -7  /* a bounded device wait gave up                    */
#define CFD_ERR_STATE       -8  /* call not valid in the handle's current state     */
#define CFD_ERR_WALLTAN     -9  /* slip-wall tangential velocity check failed       */

/* ---- boundary codes (the reference's edge3d<2>::BoundaryType) ------------ */
#define CFD_BC_WALL     -2
#define CFD_BC_FARFIELD -3

/* ---- enums --------------------------------------------------------------- */
#define CFD_FLOW_EULER    0   /* Euler2D                                   */
#define CFD_FLOW_LAMINAR  1   /* ViscousFlow2D (laminar branch)            */
#define CFD_FLOW_SST      2   /* ViscousFlow2D with the SST k-omega model
                                 coupled into every LU-SGS step (the
                                 isLaminar() == false branch, which the
                                 reference never runs): mu + mu_t in the
                                 viscous flux and radii, dt = CFL vol /
                                 (spec_c + 4 spec_v), a two-equation
                                 turbulence sweep beside or after the
                                 flow's.  LU-SGS with the FP64, MIXED or
                                 MIXFF form (MIXFF: the model's residual
                                 passes in float-float as well)            */
#define CFD_ADV_RK5       0   /* RungeKuttaStrategy(5)                     */
#define CFD_ADV_LUSGS     1   /* LUSGSIntegrator                           */
#define CFD_PREC_FP64     0   /* plain: every kernel in binary64           */
#define CFD_PREC_FP32     1   /* fast form: face states, gradients, limiter,
                                 fluxes and the LU-SGS sweep combination in
                                 binary32; residual sums, update, norms and
                                 the LU-SGS diagonal in binary64 (converges
                                 to the binary32 discretisation, ~1e-4)   */
#define CFD_PREC_MIXED    2   /* defect correction: binary64 residual (as
                                 CFD_PREC_FP64) with the binary32 LU-SGS
                                 sweep as the implicit operator; converges
                                 to the binary64 solution                 */
#define CFD_PREC_MIXFF    3   /* CFD_PREC_MIXED with the residual's face
                                 states, gradients, limiter and fluxes in
                                 float-float pairs (48-bit significands on
                                 the binary32 pipe) summed per cell into a
                                 binary64 residual; converges to the
                                 binary64 solution within ~1e-14 relative.
                                 LU-SGS sweep modes 0, 3, 4, 5, 6 only    */

/* Field selectors for cfd_get_field / cfd_put_field.  Cell fields use the
 * reference's interleaved layout [NEQU*cell + eq]; face fields [4*face + eq]. */
#define CFD_FIELD_U        0  /* primitive [rho, p, u, v], 4/cell (getU)            */
#define CFD_FIELD_W        1  /* conservative [rho, rhoE, rhou, rhov], 4/cell       */
#define CFD_FIELD_R        2  /* residual, 4/cell (getResidual)                     */
#define CFD_FIELD_GRAD     3  /* Green-Gauss gradient of U, 8/cell [eq][x,y]        */
#define CFD_FIELD_PHI      4  /* Venkatakrishnan limiter, 4/cell                    */
#define CFD_FIELD_SPEC_C   5  /* convective spectral radius, 1/cell                 */
#define CFD_FIELD_SPEC_V   6  /* viscous spectral radius, 1/cell                    */
#define CFD_FIELD_DT       7  /* local time step, 1/cell (getStableTime)           */
#define CFD_FIELD_DIAG     8  /* LU-SGS scalar diagonal, 1/cell                     */
#define CFD_FIELD_DW1      9  /* LU-SGS forward-sweep increment, 4/cell             */
#define CFD_FIELD_DW      10  /* LU-SGS backward-sweep increment, 4/cell            */
#define CFD_FIELD_GRADT   11  /* gradient of T = p/rho, 2/cell                      */
#define CFD_FIELD_MU      12  /* laminar viscosity per cell, 1/cell                 */
#define CFD_FIELD_UEDGE   13  /* face state, 4/face (getUEdge)                      */
#define CFD_FIELD_MUEDGE  14  /* laminar viscosity per face, 1/face                 */
#define CFD_FIELD_VOL     15  /* cell area, 1/cell (read only)                      */
#define CFD_FIELD_CENTER  16  /* cell centre, 2/cell (read only)                    */
#define CFD_FIELD_NORMAL  17  /* unit face normal, 2/face (read only)               */
#define CFD_FIELD_AREA    18  /* face length, 1/face (read only)                    */
#define CFD_FIELD_ECENTER 19  /* face centre, 2/face (read only)                    */
#define CFD_FIELD_WALLDIST 20 /* projected wall distance, 1/cell (read only)        */
/* SST k-omega fields (after cfd_sst_enable); T and MUT are writable. */
#define CFD_FIELD_SST_T     21 /* k, omega, 2/cell (turbulenceCellValue)           */
#define CFD_FIELD_SST_TFACE 22 /* face k, omega, 2/face (turbulenceFaceValue)      */
#define CFD_FIELD_SST_TGRAD 23 /* grad k, grad omega, 4/cell [kx, ky, wx, wy]      */
#define CFD_FIELD_SST_F1    24 /* blending function F1, 1/cell                      */
#define CFD_FIELD_SST_F2    25 /* blending function F2, 1/cell                      */
#define CFD_FIELD_SST_MUT   26 /* eddy viscosity, 1/cell (vCellMut)                 */
#define CFD_FIELD_SST_MUTF  27 /* face eddy viscosity, 1/face (vFaceMut)            */
#define CFD_FIELD_SST_FCONV 28 /* convective face flux of k, omega, 2/face          */
#define CFD_FIELD_SST_FVISC 29 /* viscous face flux of k, omega, 2/face             */
#define CFD_FIELD_SST_R     30 /* residual of k, omega, 2/cell (CellTotalTFlux)     */
#define CFD_FIELD_SST_DIAG  31 /* LU-SGS diagonal of k, omega, 2/cell (SolveDiag)   */
/* Limited face states of the last residual (HLLCFluxStrategy UL / UR after
 * updateLeftRight), 4/face; formed on request from the binary64 residual's
 * arrays (FP64 and MIXED forms; read only). */
#define CFD_FIELD_UL        32
#define CFD_FIELD_UR        33

/* Residual-norm selectors for cfd_residual_norm. */
#define CFD_NORM_DW_RHO2   0  /* sum dW_rho^2 (LUSGSIntegrator::postprocessUpdate) */
#define CFD_NORM_RK_DRHO   1  /* sum |rho - rho0| (RungeKuttaStrategy::converged)  */
#define CFD_NORM_L2_R_RHO  2  /* sqrt(sum R_rho^2 / ncell)                         */

typedef struct cfd_mesh_s* cfd_mesh_t;
typedef struct cfd_case_s* cfd_case_t;

/* Per-mesh physical parameters; the first four mirror WrapSolver::setParams
 * (UnstructSolver/SolverWrapper.h:27-56), which calls
 * set_fs_variable2(Ma, AoA, 1.225, 101325, Re). */
typedef struct {
    double mach;
    double aoa_deg;
    double reynolds;
    double density;   /* dimensional freestream density  (reference: 1.225)  */
    double pressure;  /* dimensional freestream pressure (reference: 101325) */
} cfd_freestream_t;

typedef struct {
    int flow;          /* CFD_FLOW_*                                              */
    int advance;       /* CFD_ADV_*                                               */
    int precision;     /* CFD_PREC_*                                              */
    int first_order;   /* 1: limiter forced to 0 (piecewise-constant faces)       */
    double cfl;        /* LU-SGS CFL (LUSGSIntegrator::d_CFL_number); RK uses 0.8 */
    int sweep_mode;    /* LU-SGS schedule: 0 dataflow (one cooperative launch per sweep),
                          1 one launch per level, one thread per cell,
                          2 one launch per level, 16 lanes per cell,
                          3 dataflow with two cells per warp (binary64 form;
                          measured 6% slower per step than 0 on C2),
                          4 binary32 dataflow whose two half-warps wait and
                          exchange independently (measured 7-10% slower per step
                          than 0: the diverged halves issue one after the other),
                          5 binary32 forms: dataflow over a chain schedule (each
                          warp runs its own list of cells and passes the
                          increment of its previous cell in registers; the
                          binary64 form runs mode 0),
                          6 binary32 forms: the chain schedule with groups of
                          four consecutive lists in one block (one per SM
                          sub-partition), a slot whose producer runs in the
                          same block waiting on a shared-memory table instead
                          of global memory (the table capped to the block's
                          first positions when the whole range would not
                          leave the grid co-resident).
                          All modes give the same bits */
    int sweep_blocks_per_sm; /* dataflow sweep residency (0 = default 2; capped at
                                the occupancy limit)                             */
    int sweep_poll_ns; /* dataflow sweep: pause between polls of a neighbour's
                          increment in ns (__nanosleep; 0 = spin)                */
    int sweep_threads; /* round-robin dataflow sweeps (modes 0, 3, 4 and the
                          SST turbulence sweeps): threads per block, 64, 128 or
                          256 (0 = 256); fewer warps per block put fewer cells
                          on one SM sub-partition's pipes at a time            */
    int sst_sequential; /* CFD_FLOW_SST with the round-robin schedule (mode 0):
                           0 = the turbulence sweep of each direction runs in
                           the flow's sweep launch, on its own blocks, taking
                           each slot's updated face velocity from the flow's
                           sweep as it is formed; 1 = the turbulence sweeps run
                           after the flow's.  Both give the same bits        */
    int sst_sweep_share; /* overlapped sweeps: percent of the launch's blocks that
                            run the turbulence sweep (0 = 50; 10..90)         */
    int chain_table_cap; /* sweep mode 6: at most this many shared-memory
                            hand-off entries per block, covering the block's
                            first positions (0 = the whole range, or the
                            largest count that keeps the grid co-resident)   */
    int reserved[1];
} cfd_params_t;

/* ---- errors -------------------------------------------------------------- */
/* Last error message of the calling thread ("" when none). */
const char* cfd_last_error(void);
/* ABI version: major*10000 + minor*100 + patch. */
int cfd_version(void);

/* ---- meshes (UnstructReader / UnstructTopologyHolder) -------------------- */
/* Read a 2D .grd file (UnstructReader::readForUnstruct, reader/UnstructReader.h:124-272).
 * wall_tag / far_tag are the file's negative right-cell codes that map to the
 * wall and far-field boundary types (UnstructReader::setWallSign/setOverSign). */
int cfd_mesh_load_grd(const char* path, int wall_tag, int far_tag, cfd_mesh_t* out);
/* Same mesh from arrays in .grd order: xy[2*nnode]; edge_nodes[2*nedge] (1-based
 * node ids); edge_cells[2*nedge] (1-based left/right cell ids, right may be a tag). */
int cfd_mesh_from_arrays(int nnode, const double* xy, int nedge, const int* edge_nodes,
                         const int* edge_cells, int ncell, int wall_tag, int far_tag,
                         cfd_mesh_t* out);
int cfd_mesh_info(cfd_mesh_t mesh, int* nnode, int* nedge, int* ncell);
/* Topology as the reference builds it: lr[2*nedge] (0-based, or CFD_BC_*),
 * cell_edges[4*ncell] and cell_verts[4*ncell] (0-based, -1 padded; cell3d
 * edgeInd / pointInd order), cell_sizes[2*ncell] = {nverts, nedges}. Any
 * output pointer may be NULL. */
int cfd_mesh_topology(cfd_mesh_t mesh, int* lr, int* cell_edges, int* cell_verts, int* cell_sizes);
/* LU-SGS level schedule of the reference's cell order: number of forward and
 * backward levels (cells in one level have no dependency on each other). */
int cfd_mesh_levels(cfd_mesh_t mesh, int* n_forward, int* n_backward);
void cfd_mesh_free(cfd_mesh_t mesh);

/* ---- cases (TopologyHolderStrategy + TimeIntegrator) --------------------- */
/* One case = nmesh meshes packed into one set of device arrays (overset
 * components or independent batched cases).  fs[nmesh] gives each mesh's
 * freestream.  stream: a cudaStream_t to issue on, or NULL for the library's
 * own non-blocking stream. */
int cfd_case_create(const cfd_mesh_t* meshes, int nmesh, const cfd_freestream_t* fs,
                    const cfd_params_t* params, void* stream, cfd_case_t* out);
void cfd_case_free(cfd_case_t c);
int cfd_case_info(cfd_case_t c, int* nmesh, int* ncell_total, int* nedge_total);
/* cudaStream_t the case issues on. */
int cfd_case_stream(cfd_case_t c, void** stream);
int cfd_set_cfl(cfd_case_t c, double cfl);
/* Switch a live case between precision forms, keeping its state (for example
 * binary32 while the residual is far from converged, then the binary64
 * residual).  A case created in the FP64 form cannot switch to a form with the
 * binary32 LU-SGS sweep (CFD_ERR_MESH); FP32 and MIXED cases can switch to any
 * form.  Drops the captured step graph. */
int cfd_set_precision(cfd_case_t c, int precision);
/* Uniform freestream initial state (Euler2D/ViscousFlow2D::initializeData and
 * the integrator's initializeData). */
int cfd_init_freestream(cfd_case_t c);
/* One residual evaluation from the current U (preprocessAdvanceSerial):
 * face states, gradients, limiter, spectral radii, HLLC (+ laminar) fluxes. */
int cfd_residual(cfd_case_t c, int stage);
/* dt = CFL*vol/spec_c (SolveTime). */
int cfd_local_dt(cfd_case_t c, double cfl);
/* nsteps iterations of the case's integrator (singleStepSerial). */
int cfd_step(cfd_case_t c, int nsteps);
int cfd_rk_step(cfd_case_t c);
int cfd_lusgs_step(cfd_case_t c);
/* Capture one integrator step in a CUDA graph and replay it nsteps times. */
int cfd_step_graph(cfd_case_t c, int nsteps);
/* Norm of the last step for one mesh (synchronises; also reports device-side
 * error flags as CFD_ERR_PSTAR / CFD_ERR_NONPHYSICAL / CFD_ERR_WALLTAN). */
int cfd_residual_norm(cfd_case_t c, int mesh, int which, double* out);
/* One call for a host-driven loop (no reference counterpart): optionally the
 * whole case's primitive field from host memory (host_u[4*ncell_total], the
 * meshes one after another; pinned memory makes the copy asynchronous), then
 * nsteps graph-replayed steps (cfd_step_graph), then, if host_norms is not
 * NULL, every mesh's norm `which` into host_norms[nmesh], and, if host_u_out
 * is not NULL, the updated primitive field into host_u_out[4*ncell_total]
 * (the same layout as host_u; it may be the same buffer); synchronises once
 * and reports device errors as cfd_sync does. */
int cfd_step_io(cfd_case_t c, const double* host_u, int nsteps, int which, double* host_norms, double* host_u_out);
/* Copy a field of one mesh to / from host memory (layout above). */
int cfd_get_field(cfd_case_t c, int mesh, int which, double* host);
int cfd_put_field(cfd_case_t c, int mesh, int which, const double* host);
/* Force on the walls of one mesh from the current state (evaluates the
 * fluxes first): out4 = {Fx, Fy, CL, CD}, coefficients on 0.5*rho*V^2*ref_length
 * in the freestream direction.  No reference counterpart: the reference
 * integrates only Cp (Euler2D.cpp:392-618). */
int cfd_wall_force(cfd_case_t c, int mesh, double ref_length, double* out4);
/* Per-cell CFL multipliers of one mesh for LU-SGS (dt_i = CFL * mult_i * vol_i /
 * spec_c,i).  The reference uses one constant CFL (LUSGS_Integrator.h:18); the
 * multipliers are the hook of local-CFL controllers.  NULL removes them. */
int cfd_set_cell_cfl(cfd_case_t c, int mesh, const double* mult);
/* Wait for the case's stream and report any device-side error flag. */
int cfd_sync(cfd_case_t c);
/* Number of kernel launches the library issued on this case so far. */
long long cfd_launch_count(cfd_case_t c);
/* Measurement helper (no reference counterpart; the reference only has a
 * scope timer, toolBox/Timer.h:5-20): run one pass reps times on the case's
 * stream, each bracketed by CUDA events, writing flush_bytes to a scratch
 * buffer before each rep to evict L2, and return the mean duration in ms.
 * pass: 0 face_state, 1 cell_grad, 2 face_flux, 3 cell_update, 4 forward sweep
 * (all levels), 5 backward sweep (all levels), 6 LU-SGS update, 7 whole step;
 * coupled SST cases: 8 the model's residual passes, 9 the turbulence sweeps
 * (constants, forward, backward), 10 the k, omega, mu_t update; connected
 * overset cases: 11 the fringe exchange; SST cases that overlap their sweeps
 * (cfd_params_t.sst_sequential 0, sweep mode 0): 12 both directions' flow and
 * turbulence sweeps with their per-step constants, as a step runs them. */
int cfd_bench_pass(cfd_case_t c, int pass, int reps, long long flush_bytes, double* avg_ms);
/* Autotuner of the dataflow sweeps' launch shape (no reference counterpart):
 * times `reps` whole LU-SGS steps for each co-resident block count per SM
 * (1, 2, ... up to the occupancy limit), keeps the fastest for the case and
 * reports it; the case's state is restored afterwards.  For the binary32-sweep
 * forms of a case created with sweep_mode 0, 5 or 6 it also picks among those
 * three schedules, and for the round-robin ones among 256, 128 and 64 threads
 * per block, with and without the look-ahead loads (cfd_case_sweep reads the
 * choice). */
int cfd_autotune(cfd_case_t c, int reps, int* best_blocks_per_sm, double* best_ms);
/* Host-side chain schedule of the binary32 LU-SGS sweep (sweep modes 5 and 6)
 * for one mesh, as a case holding that mesh builds it (no reference
 * counterpart; needs no GPU).  forward: 1 forward sweep, 0 backward; nlists:
 * warps of the launch (a multiple of 8); local: mode 6's block-local list
 * numbering; table: 0 no shared-memory table, else its cap in entries per
 * block (INT_MAX: the block's whole range) -- a dependency on a producer of
 * the same block at a position below the cap is encoded as a table entry.
 * Outputs: hptr[nlists+1] each list's range of positions; cells[2*ncell]
 * per position (cell, bits 2s..2s+1 = 1/2 when slot s waits for the list's
 * previous cell / the one before); rec[8*ncell] per position and face slot
 * (neighbour waited for or -1, signed face code); jenc[4*ncell] the
 * dependency as the sweep reads it (-1 none, -2/-3 registers, -4-t table entry
 * t, else the cell id); *table_entries the table's entries per block. */
int cfd_chain_schedule(cfd_mesh_t mesh, int forward, int nlists, int local, int table, int* hptr,
                       int* cells, int* rec, int* jenc, int* table_entries);
/* The case's current LU-SGS schedule: sweep_mode, blocks per SM, threads per
 * block of the round-robin dataflow sweeps and whether they load the next
 * position's inputs while waiting (lookahead 1: more registers per thread,
 * fewer resident warps; after cfd_autotune, the ones it chose); any pointer
 * may be NULL. No reference counterpart. */
int cfd_case_sweep(cfd_case_t c, int* sweep_mode, int* blocks_per_sm, int* threads, int* lookahead);
/* 1 if the case's LU-SGS step runs its turbulence sweeps in the flow's sweep
 * launches (CFD_FLOW_SST, sweep mode 0, sst_sequential 0; cfd_autotune sets
 * sst_sequential by timing both), else 0. */
int cfd_case_sst_overlap(cfd_case_t c, int* overlapped);
/* Failure-detection self-test (no reference counterpart): launch a kernel that
 * waits, at most `polls` polls, on a device flag nothing sets, exactly as the
 * dataflow LU-SGS sweep waits on its neighbours.  Returns CFD_ERR_TIMEOUT when
 * the bounded wait gave up (the expected outcome) and leaves the case usable. */
int cfd_selftest_bounded_wait(cfd_case_t c, long long polls);
/* Measurement helper: the latency floor of the dataflow sweeps' hand-off.  A
 * cooperative chain of `hops` one-warp blocks, each waiting (bounded) for the
 * previous block's value in global memory, running fp64_ops dependent binary64
 * FMAs on it and publishing its own; us_per_hop = best of 4 timed chains /
 * (hops - 1).  2 <= hops <= 1024.  stream may be NULL. */
int cfd_measure_hop_latency(void* stream, int hops, int fp64_ops, double* us_per_hop);

/* ---- field dumps (TopologyHolderStrategyOutput.cpp) ---------------------- */
/* Tecplot files in the reference's layouts, byte for byte: node coordinates,
 * the data, each cell's 1-based vertices padded to four; numbers in the C++
 * stream's default format.
 * cfd_write_cell_data: writeCellData (:466-554) of mesh `mesh` of the case
 *   (density, pressure, u, v, Cp, Mach per cell; Cp and Mach formed on the
 *   device), file filename_<mesh+1>_<proc+1>; m must be that mesh.
 * cfd_write_node_data: writeNOdeData (:556-630), node_q[4*node + k] (host).
 * cfd_write_tioga_format: writeTiogaFormat (:410-464), one int per cell
 *   (host), file filename<mesh><proc>. */
int cfd_write_cell_data(cfd_case_t c, int mesh, cfd_mesh_t m, const char* filename, int proc);
int cfd_write_node_data(cfd_mesh_t m, int mesh, const char* filename, int proc, const double* node_q);
int cfd_write_tioga_format(cfd_mesh_t m, int mesh, const char* filename, int proc, const int* cell_data);

/* ---- overset connectivity and fringe exchange (UniTioga MeshBlock) ------- */
/* Layouts of a node array for the fringe update (dataUpdate.cpp:4-5). */
#define CFD_LAYOUT_ROW     0  /* q[node*nvar + k]   */
#define CFD_LAYOUT_COLUMN  1  /* q[k*nnodes + node] */

typedef struct cfd_block_s* cfd_block_t;    /* one mesh on the device as a donor (MeshBlock) */
typedef struct cfd_interp_s* cfd_interp_t;  /* an interpolation list (MeshBlock::interpList)  */

/* Interpolation weights of n (cell, point) pairs, evaluated on the device:
 * computeNodalWeight2D (mathTools/math.cpp:229-312) with solvec and
 * newtonSolve2D.  nvert[i] is 3 or 4; xv[8*i ..] holds the cell's vertices
 * (x0,y0,..,x3,y3); xp[2*i ..] the point; frac[4*i ..] receives the weights
 * (vertex order of xv; 0 in the unused slot of a triangle).  A triangle whose
 * 2x2 system is singular returns CFD_ERR_MESH (the reference throws).  All
 * arrays are host memory. */
int cfd_nodal_weights(long long n, const int* nvert, const double* xv, const double* xp, double* frac);
/* Upload one mesh's nodes and cells and build its donor-search bins on the
 * device (the block a MeshBlock registers, tioga::registerGridData). */
int cfd_block_create(cfd_mesh_t mesh, void* stream, cfd_block_t* out);
void cfd_block_free(cfd_block_t b);
/* Donor search for npts points (host xy[2*npts]), as MeshBlock::search
 * (search.cpp:81-270) chooses: the cells whose boxes cross the oriented box of
 * the points form the reference's alternating digital tree, and each point
 * takes the first cell of that tree's walk whose box holds it within
 * TOL = 1e-10 and whose weights all lie in [-TOL, 1+TOL] (checkContainment.cpp:
 * 4-62), else -1; where several cells contain a point (a shared edge or
 * vertex) the donor is the reference's.  Points closer than TOL (L1) to an
 * earlier point take that point's donor (uniquenodes_octree).  donor_nodes[4*i]
 * / weights[4*i] (may be NULL) get the donor's vertices and the point's weights
 * in it (-1 / 0 when not found or in a triangle's unused slot). */
int cfd_block_search(cfd_block_t b, long long npts, const double* xy, int* donor_cell, int* donor_nodes,
                     double* weights);
/* The same search with the rest of MeshBlock::search's inputs: tags[i] the
 * point's mesh tag (coincident points merge only within one tag; NULL: all 1),
 * res[i] its resolution, merged in place over coincident points as the
 * reference merges res_search (NULL: not used), cell_unaccept[c] = 1 for a
 * cell whose cellRes is BIGVALUE (such a cell does not stop the walk where one
 * of the point's weights vanishes; NULL: none), xtag[i] (may be NULL) the
 * point whose search point i took. */
int cfd_block_search_ex(cfd_block_t b, long long npts, const double* xy, const int* tags, double* res,
                        const unsigned char* cell_unaccept, int* donor_cell, int* donor_nodes, double* weights,
                        int* xtag);
/* Cell values as the mean of their nodes' values (Orchestra.cpp:270-291), on
 * device arrays in ROW layout: q_cell[c*nvar + k] = (sum_j q_node[v_j*nvar + k]) / nvert. */
int cfd_block_node_to_cell(cfd_block_t b, const double* d_q_node, int nvar, double* d_q_cell, void* stream);
/* Interpolation list for the receptor points xy[2*n] (host), found in the donor
 * block: receptor i writes node recv_node[i] of the receiving array.  Points
 * without a donor are left out of the list (n_found counts those kept). */
int cfd_interp_create(cfd_block_t donor, long long n, const double* xy, const int* recv_node, cfd_interp_t* out);
/* Interpolation list from explicit entries (as findInterpData fills interpList,
 * bookkeeping.cpp:396-424): nweights[i] in {3,4}, inode[4*i], weights[4*i].
 * A weight outside [-TOL, 1+TOL] returns CFD_ERR_MESH: getInterpolatedSolution
 * throws "weights are not convex" (dataUpdate.cpp:52-55); the weights of a
 * list never change, so the check is made once, here. */
int cfd_interp_create_list(long long n, const int* recv_node, const int* nweights, const int* inode,
                           const double* weights, void* stream, cfd_interp_t* out);
int cfd_interp_info(cfd_interp_t it, long long* n_found, long long* n_requested);
/* Host copies of the list: recv_node[n], donor_cell[n] (-1 for an explicit
 * list), inode[4n], weights[4n]; any pointer may be NULL. */
int cfd_interp_get(cfd_interp_t it, int* recv_node, int* donor_cell, int* inode, double* weights);
/* Fringe exchange on device arrays: every receptor's value is interpolated
 * from q_donor (getInterpolatedSolution, dataUpdate.cpp:6-111) and then written
 * into q_recv (updateSolnData, dataUpdate.cpp:113-132), in `layout` with nvar
 * values per node, asynchronously on `stream` (NULL: the list's stream).  All
 * values are interpolated before any is written, so the two arrays may be the
 * same; where several receptors name one node the last in the list wins, as
 * in the reference's update loop.  Node indices are checked on the host
 * against nnodes_donor / nnodes_recv (CFD_ERR_ARG). */
int cfd_interp_update(cfd_interp_t it, const double* d_q_donor, long long nnodes_donor, double* d_q_recv,
                      long long nnodes_recv, int nvar, int layout, void* stream);
void cfd_interp_free(cfd_interp_t it);

/* Hole cutting.  A hole map is the Cartesian map of one block's walls
 * (tioga::getHoleMap, holeMap.cpp:7-180): the box of the wall nodes
 * (MeshBlock::getWallBounds, MeshBlock.cpp:653-685), 192 map cells along its
 * longer side plus 2 cells of padding, the cells touched by the boxes of
 * wall-adjacent mesh cells marked (MeshBlock::markWallBoundary,
 * MeshBlock.cpp:687-778), then a flood fill from the map's border
 * (fillHoleMap2D, utils.cpp:782-860): map cells the fill cannot reach are
 * inside the body.  isym: 3 = four neighbours (tioga's default), 1 = only
 * the y neighbours, 2 = only the x neighbours.  The wall nodes are the ends
 * of the block's wall faces.  A block without walls returns CFD_ERR_MESH. */
typedef struct cfd_holemap_s* cfd_holemap_t;
int cfd_holemap_create(cfd_block_t b, int isym, cfd_holemap_t* out);
/* nx[2] map cells and extents[4] = {xmin, ymin, xmax, ymax}. */
int cfd_holemap_info(cfd_holemap_t h, int* nx, double* extents);
/* Host copy of the map, nx[0]*nx[1] ints (1 = inside), row y*nx[0] + x. */
int cfd_holemap_get(cfd_holemap_t h, int* sam);
/* checkHoleMap (utils.cpp:645-670) for n host points: inside[i] = 1 or 0. */
int cfd_holemap_check(cfd_holemap_t h, long long n, const double* xy, int* inside);
void cfd_holemap_free(cfd_holemap_t h);
/* Node blanking of one block against others (MeshBlock::processDonors,
 * bookkeeping.cpp:88-186): iblank[i] = 0 where some other block j that has a
 * hole map (maps[j] != NULL) gives node i no donor cell and its map holds the
 * node, else 1; mandatory[i] = 1 for an unblanked node within nfringe layers
 * of cells of a blanked node (a mandatory receptor, nodeRes = BIGVALUE), else
 * 0.  Host output arrays of the block's node count; mandatory may be NULL. */
int cfd_overset_blank(cfd_block_t self, int nother, const cfd_block_t* others, const cfd_holemap_t* maps,
                      int nfringe, int* iblank, int* mandatory);
/* Overset assembly of nblocks (2 to 64) blocks on this device (one rank's
 * tioga::performConnectivity, tioga.cpp:153-262, with MeshBlock::preprocess,
 * MeshBlock.cpp:135-425; processDonors / findInterpData / cancellation /
 * reduce_fringes, bookkeeping.cpp:75-705; exchangeDonors' order,
 * exchangeDonor.cpp:24-347).  maps[b]: block b's hole map or NULL (no walls);
 * obc_nodes[b][nobc[b]]: block b's overset-boundary nodes (host, 0-based;
 * they and their cells' nodes become mandatory receptors, and mexclude layers
 * of cells around them unacceptable donors); nfringe: layers of mandatory
 * receptors around holes and, plus one, receptors kept by the fringe
 * reduction (tioga defaults: nfringe 1, mexclude 3).  Distance-scaled
 * resolutions (MeshBlock::reResolution) are not applied, as tioga's default.
 * Each block is searched once for the nodes of all other blocks, in block
 * order, tagged by block and carrying their resolutions, as exchangeSearchData
 * hands them to MeshBlock::search (cfd_block_search_ex). */
typedef struct cfd_connect_s* cfd_connect_t;
int cfd_overset_connect(int nblocks, const cfd_block_t* blocks, const cfd_holemap_t* maps, const int* const* obc_nodes,
                        const int* nobc, int nfringe, int mexclude, cfd_connect_t* out);
/* Final node iblank (1 field, 0 hole, -1 receptor) and cell iblank
 * (getCellIblanks) of one block; host arrays, either may be NULL. */
int cfd_connect_iblank(cfd_connect_t c, int block, int* node_iblank, int* cell_iblank);
/* The interpolations a donor block serves (interpList entries not cancelled,
 * in the reference's order): count, then host arrays of that length
 * (inode / weights: 4 per entry, -1 / 0 in a triangle's unused slot); any
 * pointer may be NULL.  cfd_interp_create_list builds the exchange. */
int cfd_connect_interp_count(cfd_connect_t c, int donor_block, long long* n);
int cfd_connect_interp_get(cfd_connect_t c, int donor_block, int* recv_block, int* recv_node, int* donor_cell,
                           int* nweights, int* inode, double* weights);
void cfd_connect_free(cfd_connect_t c);
/* Cell blanking from node blanking (MeshBlock::getCellIblanks,
 * bookkeeping.cpp:654-705): cell_iblank[c] = 0 if any of its nodes is 0 (hole),
 * -1 if all of its nodes are -1 (receptors), else 1.  Host arrays of the
 * block's node / cell counts. */
int cfd_cell_iblank(cfd_block_t b, const int* node_iblank, int* cell_iblank);

/* ---- overset components of one case ---------------------------------------- */
/* Connectivity of a case whose meshes are overset components: one rank's
 * tioga::performConnectivity over them (tioga.cpp:153-262; the assembly of
 * cfd_overset_connect with hole maps of the meshes that have wall faces, isym
 * 3).  meshes[] are the handles the case was created from, in the same order;
 * obc_nodes[m][nobc[m]] the overset-boundary nodes of mesh m (0-based; either
 * array may be NULL for none).  Afterwards every LU-SGS step updates only the
 * field cells (cell iblank 1) and ends with the fringe exchange below, so a
 * captured step (cfd_step_graph) holds the whole coupled iteration.  LU-SGS
 * cases, 2 to 64 meshes; re-run it when the grids move. */
int cfd_connectivity(cfd_case_t c, const cfd_mesh_t* meshes, const int* const* obc_nodes, const int* nobc,
                     int nfringe, int mexclude);
/* The fringe exchange of a connected case (tioga::dataUpdate between its
 * components, tioga.cpp:326-471, dataUpdate.cpp:6-132, on node values as
 * Orchestra::init registers them, Orchestra.cpp:201-291): the donor nodes get
 * the mean of their cells' primitive state, every receptor node is
 * interpolated from its donor cell (all values formed before any is written),
 * and every receptor cell (iblank -1) takes the mean of its nodes.  nvar must
 * be 4 (the primitive state).  Asynchronous on the case's stream. */
int cfd_fringe_update(cfd_case_t c, int nvar);
/* Cell iblank of one mesh of a connected case (1 field, 0 hole, -1 receptor). */
int cfd_case_iblank(cfd_case_t c, int mesh, int* cell_iblank);

/* ---- SST k-omega (SSTkomegaModel, UnstructSolver/SSTKWStrategy.h) -------- */
/* The reference builds this model but never runs it (ViscousFlow2D's serial
 * residual skips it and isLaminar() is true); these calls evaluate its
 * functions on the device from the laminar residual's arrays.
 * cfd_sst_enable: allocate the k-omega arrays of a laminar case (binary64
 * residual: FP64 or MIXED) and set k, omega and mu_t to the freestream values
 * (InitializeturbulenceVariable, :582-613).  cfd_sst_freestream: out3 = {k,
 * omega, mu_t} of that freestream.  cfd_sst_residual: SolveTurbulenceEquation
 * (:515-524) and SolveDiag (:170-192) from the current face states,
 * gradients, viscosities, spectral radii and time steps (call cfd_residual and
 * cfd_local_dt first).  cfd_sst_update_mut: the eddy viscosity update of
 * UpdatePrimitiveVariables (:194-223) from W = rho (k, omega). */
int cfd_sst_enable(cfd_case_t c);
/* Freestream turbulence of the model: intensity tu and eddy-viscosity ratio
 * mu_t / mu (InitializeturbulenceVariable, SSTKWStrategy.h:582-613, fixes them
 * at 0.01 and 0.035): k = 1.5 (tu |V|)^2, omega = rho k / (ratio mu), mu_t =
 * ratio mu.  Sets the far-field values (and the floors of the coupled model);
 * cfd_init_freestream then starts from them.  No reference counterpart. */
int cfd_sst_set_inflow(cfd_case_t c, double intensity, double viscosity_ratio);
int cfd_sst_freestream(cfd_case_t c, int mesh, double* out3);
int cfd_sst_residual(cfd_case_t c);
int cfd_sst_update_mut(cfd_case_t c);

/* ---- learned relaxation (no reference counterpart) ------------------------- */
/* A 12-64-64-2 perceptron (relu, bf16 weights, fp32 arithmetic) that maps 12
 * features of a cell after its LU-SGS sweeps to o = (o0, o1): the cell's update
 * is W += omega * dW with omega = 1 + 0.6*sigmoid(o0), and, when enabled, its
 * next time step is multiplied by 2^(2*tanh(o1)).  The reference uses one
 * constant CFL and omega = 1 (LUSGS_Integrator.h:18, .cpp:242-255), which stay
 * the fallback; neither output changes the fixed point (dW = 0 there).
 * Parameters, fp32, in this order: W1[64][12], b1[64], W2[64][64], b2[64],
 * W3[2][64], b3[2]; the input transform norm[24] = mean[12], scale[12]
 * (x^ = (x - mean) * scale).  Features, per cell (dW scaled per equation by
 * rho, |rhoE|, rho(|u|+c), rho(|u|+c)): 0 log10|dW|, 1 log10|dW_prev|,
 * 2 (dW.dW_prev)/|dW_prev|^2 clipped to [-4, 4], 3 cos(dW, dW_prev),
 * 4 log10(|R_rho| dt/(vol rho)), 5 log10(spec_v/spec_c + 1e-12), 6 Mach,
 * 7 min limiter, 8 log10(D dt/vol), 9 log10(wall distance/sqrt(vol) + 1e-6),
 * 10 rho - 1, 11 p - 1.  The learned update is three launches: the network per
 * cell, the mean factor per mesh, and the bounded update. */
#define CFD_MLP_INPUTS  12
#define CFD_MLP_OUTPUTS 2
#define CFD_MLP_PARAMS  5122
typedef struct cfd_mlp_s* cfd_mlp_t;
/* He-uniform weights from a seed; b3[0] = -4 (omega ~ 1.01 untrained). */
int cfd_mlp_create(unsigned long long seed, cfd_mlp_t* out);
void cfd_mlp_free(cfd_mlp_t m);
/* Host copies of the fp32 parameters and the input transform (either may be NULL). */
int cfd_mlp_get_params(cfd_mlp_t m, float* params, float* norm);
int cfd_mlp_set_params(cfd_mlp_t m, const float* params, const float* norm);
/* Raw outputs y[2n] for inputs x[12n] (device arrays). */
int cfd_mlp_forward(cfd_mlp_t m, const float* d_x, long long n, float* d_y, void* stream);
/* Loss (1/n) sum_i sum_o m_io (y_io - t_io)^2 over all n <= 2^20 rows and its
 * gradient with respect to the bf16-rounded parameters (host grad[CFD_MLP_PARAMS],
 * may be NULL).  d_m (per-output weights) may be NULL (all 1). */
int cfd_mlp_loss_grad(cfd_mlp_t m, const float* d_x, const float* d_t, const float* d_m, long long n, double* loss,
                      float* grad);
/* `steps` Adam steps (beta 0.9 / 0.999) on minibatches of `batch` rows drawn
 * from the n rows with a seeded counter hash; loss_hist[steps] (host, may be
 * NULL) receives each minibatch's loss. */
int cfd_mlp_train(cfd_mlp_t m, const float* d_x, const float* d_t, const float* d_m, long long n, int steps,
                  int batch, float lr, unsigned long long seed, float* loss_hist);
/* Keep each LU-SGS step's previous increment on the device (the features need it). */
int cfd_case_track(cfd_case_t c, int on);
/* Features of every cell (device x[12 * ncell_total]) from the last LU-SGS step. */
int cfd_case_features(cfd_case_t c, float* d_x);
/* Attach (m != NULL) or detach the learned relaxation; apply_cfl also applies
 * the CFL output.  spread >= 0 bounds each cell's factor to the mesh mean of
 * the predicted factors +- spread (spread < 0: each cell uses its own;
 * measured: unbounded per-cell factors can stall the iteration, spread 0 is
 * the robust choice).
 * Detaching restores the constant CFL and the unit update. */
int cfd_case_set_mlp(cfd_case_t c, cfd_mlp_t m, int apply_cfl, double spread);

/* Residual norm of a caller-owned device array that allocates nothing (no
 * counterpart in the reference, which has no device code).  For callers that
 * may not allocate device memory while they run: solvers that reserve all of
 * it at start-up, or hosts whose own memory pool owns the device.
 * d_records: n records of 4 doubles ([4*cell + eq], component 0 is reduced);
 * which: CFD_NORM_DW_RHO2 (sum x^2) or CFD_NORM_L2_R_RHO (sqrt(sum x^2 / n));
 * the result is written to d_out[0] on the device, asynchronously on `stream`.
 * The scratch is a static 32 KiB device array shared by all calls: n is
 * limited to 33,554,432 records (CFD_ERR_ARG beyond), overlapping calls race,
 * and the first call on each device looks up the array's address (make it
 * before any stream capture); that address is kept for the life of the
 * process, so a device reset (cudaDeviceReset) while the library is loaded is
 * not supported.  A NaN record gives a NaN result with CFD_OK: unlike
 * cfd_residual_norm there is no device error word to raise
 * CFD_ERR_NONPHYSICAL. */
int cfd_residual_norm_noalloc(const double* d_records, int n, int which, double* d_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* CFDGB_H */
