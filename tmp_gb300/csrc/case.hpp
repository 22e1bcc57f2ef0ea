// Device-resident state of one case (one or more meshes packed together) and
// the host-side launchers of the kernels that operate on it.
#pragma once
#include <cuda_runtime.h>
#include <string>
#include <vector>

#include "fv_device.cuh"
#include "mesh.hpp"

namespace cfdgb {

struct DevArrays {
    int nc = 0, nf = 0, nn = 0, nmesh = 0;
    int resid32 = 0;             // 1 while the residual runs in binary32 (the FP32 form)
    int turb = 0;                // 1 when the SST k-omega model is coupled into every step (CFD_FLOW_SST)
    int residq = 0;              // 1 while the residual runs in float-float (the MIXFF form)
    // topology
    int2* lr = nullptr;          // [nf]
    int2* enodes = nullptr;      // [nf] global node ids
    int* fmesh = nullptr;        // [nf]
    int* cmesh = nullptr;        // [nc]
    int4* cface = nullptr;       // [nc] signed face codes
    int4* cverts = nullptr;      // [nc] global node ids, -1 padded
    int* cnvert = nullptr;       // [nc]
    d2* xy = nullptr;            // [nn]
    MeshPrm* prm = nullptr;      // [nmesh]
    // binary64 geometry
    d4* fgeo = nullptr;          // [nf] (nx, ny, length, 0)
    d2* fcen = nullptr;          // [nf] face centre
    d4* cgeo = nullptr;          // [nc] (vol, xc, yc, 0)
    d4* fg0 = nullptr;           // [nf] (nx, ny, length, 125*vol_left)
    d4* fg1 = nullptr;           // [nf] (xf-xl, yf-yl, xf-xr, yf-yr)
    d4* fvis = nullptr;          // [nf] (dx, dy, dx^2+dy^2, 0)
    double* walld = nullptr;     // [nc] projected wall distance
    int* wall_ptr = nullptr;     // [nmesh+1] per-mesh ranges of wall_faces
    int* wall_faces = nullptr;   // global ids of wall faces, ascending within each mesh
    int4* wblocks = nullptr;     // (mesh, begin, end) chunks of wall_faces for the force sum
    int nwblk = 0;
    double* wpartial = nullptr;  // [2*nwblk]
    double* wforce = nullptr;    // [2*nmesh] (Fx, Fy)
    // binary32 copies (fast form)
    float4* fg0f = nullptr;
    float4* fg1f = nullptr;
    float4* fvisf = nullptr;
    float4* cgeof = nullptr;
    // state (binary64)
    d4* U = nullptr;
    d4* W = nullptr;
    d4* W0 = nullptr;
    d4* R = nullptr;
    double* dt = nullptr;
    double* diag = nullptr;
    float* cflmul = nullptr;     // [nc] optional per-cell CFL multiplier (null = 1)
    d4* dW1 = nullptr;
    d4* dW = nullptr;
    d4* dWprev = nullptr;        // [nc] previous LU-SGS increment (kept while tracking / learned)
    // SST k-omega (k_sst.cu), allocated by cfd_sst_enable
    double* sstT = nullptr;      // [2*nc] k, omega
    double* sstTf = nullptr;     // [2*nf] face k, omega
    double* sstG = nullptr;      // [4*nc] grad k, grad omega
    double* sstF1 = nullptr;     // [nc]
    double* sstF2 = nullptr;     // [nc]
    double* sstMut = nullptr;    // [nc] eddy viscosity
    double* sstMutf = nullptr;   // [nf]
    double* sstFc = nullptr;     // [2*nf] convective face flux
    double* sstFv = nullptr;     // [2*nf] viscous face flux
    double* sstR = nullptr;      // [2*nc] residual
    double* sstD = nullptr;      // [2*nc] LU-SGS diagonal
    // coupled SST LU-SGS (CFD_FLOW_SST; k_sst.cu)
    double* sstW = nullptr;      // [2*nc] rho k, rho omega: the turbulence equations' conservative state
    double* sstDW1 = nullptr;    // [2*nc] forward-sweep increment
    double* sstDW = nullptr;     // [2*nc] backward-sweep increment
    double* sstFcs = nullptr;    // [8*nc] per (cell, slot): the neighbour's convective flux W_t,j Vn(W_j), 2 values
    double* sstRA = nullptr;     // [4*nc] per (cell, slot): r_A of SolveViscousFlux
    double* sstVnp = nullptr;    // [4*nc] per (cell, slot): Vn(W_j + dW_j) with the flow's increment of that sweep
    double* sstDinv = nullptr;   // [2*nc] 1 / diagonal (the binary32 sweep)
    float2* sstDW1f = nullptr;   // [nc] binary32 copies published by the binary32 sweep
    float2* sstDWf = nullptr;    // [nc]
    float4* sstSlotf = nullptr;  // [4*nc] binary32 sweep: per (cell, slot) (0, 0, r_A, face length)
    float2* sstVnpf = nullptr;   // [4*nc] binary32 sweep: per (cell, slot) Vn(W_j + dW_j) and its change dVn
    float2* sstWf = nullptr;     // [nc] binary32 copy of sstW for that sweep
    ff* sstTq = nullptr;         // [2*nc] MIXFF: float-float copies of k, omega, mu_t and the wall distance
    ff* sstMutq = nullptr;       // [nc]   that the model's float-float passes read
    ff* walldq = nullptr;        // [nc]
    int ffsst = 0;               // 1: the model's residual passes run in float-float (MIXFF)
    int sst_grid = 0;            // co-resident blocks of the turbulence sweeps
    int cpl_grid = 0;            // co-resident blocks of the flow + turbulence sweep launch
    int cpl_nflow = 0;           // of which the flow's sweep takes [0, cpl_nflow)
    float* omega = nullptr;      // [nc] relaxation of the last learned update
    float* omega_mean = nullptr; // [nmesh] its mean per mesh
    int* mlp_samples = nullptr;  // cells the network is evaluated on, mesh by mesh
    int* mlp_samp_off = nullptr; // [nmesh+1] each mesh's range in mlp_samples
    int mlp_nsamp = 0;
    // residual intermediates, binary64 form
    d4* grad = nullptr;          // [2*nc]
    d4* phi = nullptr;
    double* specc = nullptr;
    double* specv = nullptr;
    d2* gradT = nullptr;
    double* mu = nullptr;
    d4* Ue = nullptr;            // [nf]
    d2* fspec = nullptr;         // [nf]
    double* mue = nullptr;       // [nf]
    d4* Fc = nullptr;            // [nf]
    d4* Fv = nullptr;            // [nf]
    // residual intermediates, binary32 form
    float4* Uf = nullptr;
    float4* gradf = nullptr;
    float4* phif = nullptr;
    float* speccf = nullptr;
    float* specvf = nullptr;
    float2* gradTf = nullptr;
    float* muf = nullptr;
    float4* Uef = nullptr;
    float2* fspecf = nullptr;
    float* muef = nullptr;
    float4* Fcf = nullptr;
    float4* Fvf = nullptr;
    // residual intermediates, float-float form (hi, lo pairs; same record sizes as binary64)
    q4* Uq = nullptr;            // [nc] float-float copy of U, made at the start of each residual
    q4* gradq = nullptr;         // [2*nc]
    q4* phiq = nullptr;
    ff* speccq = nullptr;
    ff* specvq = nullptr;
    q2* gradTq = nullptr;
    ff* muq = nullptr;
    q4* Ueq = nullptr;           // [nf]
    q2* fspecq = nullptr;
    ff* mueq = nullptr;
    q4* Fcq = nullptr;
    q4* Fvq = nullptr;
    q4* fg0q = nullptr;          // float-float geometry copies
    q4* fg1q = nullptr;
    q4* fvisq = nullptr;
    q4* cgeoq = nullptr;
    // LU-SGS per-step constants of SolveDF for every (cell, face slot)
    double* swfc = nullptr;      // [16*nc] F_c(W_j)[m] at (i*4+s)*4+m
    double* swra = nullptr;      // [4*nc]  r_A at i*4+s
    double* invD = nullptr;      // [nc] 1/D (fast form's sweep)
    // fast-form sweep: binary32 copies and level-paired order
    float* swraf = nullptr;      // [4*nc]
    float4* Wf = nullptr;        // [nc]
    float4* dW1f = nullptr;      // [nc]
    float4* dWf = nullptr;       // [nc]
    int* fwd_order2 = nullptr;   // [npos2_fwd] cells of each level in pairs, odd levels padded with -1
    int* bwd_order2 = nullptr;
    int npos2_fwd = 0, npos2_bwd = 0;
    int flow_grid = 0;           // co-resident blocks of the dataflow sweep
    int flow_threads = 256;      // threads per block of the round-robin dataflow sweeps
    int flow_pf = 1;             // round-robin sweeps load the next position's inputs while waiting
    // chain-scheduled fast-form sweep (sweep_mode 5), index 0 forward, 1 backward
    int chain_nh = 0;            // warps (lists) the schedule was built for (0: not built)
    int* chain_ptr[2] = {nullptr, nullptr};    // [chain_nh+1] each warp's range of positions
    int2* chain_cells[2] = {nullptr, nullptr}; // [nc] (cell, local-dependency bits) at each position
    int2* chain_rec[2] = {nullptr, nullptr};   // [4*nc] (lower/upper neighbour or -1, face code) per slot
    float4* chain_stage[2] = {nullptr, nullptr};  // [16*nc] per-position stage records (k_fp64.cu)
    int* chain_jenc[2] = {nullptr, nullptr};   // [4*nc] each slot's dependency as the sweep reads it
    int chain_tbl = 0;            // shared-memory hand-off entries per block (mode 6; 0 = none)
    int chain_local = 0;          // the schedule keeps a block's lists consecutive (mode 6)
    int* chain_posb = nullptr;    // [nc] position of each cell in the backward schedule
    float4* chain_dF = nullptr;   // [nc] binary32 slot sums of the last chain sweep
    int poll_ns = 0;             // back-off between a dataflow sweep's polls (ns, 0 = spin)
    // LU-SGS level schedule (all meshes merged level by level)
    int* fwd_order = nullptr;
    int* bwd_order = nullptr;
    std::vector<int> fwd_ptr, bwd_ptr;  // host copies, size nlev+1
    // reductions
    int nblk_norm = 0;
    int4* norm_blocks = nullptr;  // (mesh, begin, end, 0) per block
    double* norm_partial = nullptr;
    double* norm_out = nullptr;   // [nmesh]
    unsigned* err = nullptr;      // [2] device error word; err[1] stays 0 (a flag nothing sets)
    int* iblank_cell = nullptr;   // [nc] overset cell blanking (1 field, 0 hole, -1 receptor) or null: the
                                  // LU-SGS update leaves every cell that is not a field cell as it is
};

// Case-level overset exchange (k_fringe.cu): device arrays built by cfd_case_connect.
struct FringePlan {
    int nsrc = 0;                 // donor nodes whose cell means the lists read
    int* src_nodes = nullptr;     // [nsrc] global node ids
    int* src_ptr = nullptr;       // [nsrc+1] ranges of src_cells
    int* src_cells = nullptr;     // cells around each donor node, ascending
    int nrecv = 0;                // interpolation entries (receptor nodes)
    int* recv_node = nullptr;     // [nrecv] global receiving node
    int* nw = nullptr;            // [nrecv] 3 or 4
    int* inode = nullptr;         // [4*nrecv] global donor nodes
    double* w = nullptr;          // [4*nrecv] weights
    int ncells = 0;               // receptor cells
    int* recv_cells = nullptr;    // [ncells] global cell ids (iblank_cell -1)
    double* qn = nullptr;         // [4*nn] node values, ROW layout
    double* vals = nullptr;       // [4*nrecv] interpolated values before they are written
};

struct LaunchCfg {
    cudaStream_t stream;
    long long* counter;  // launches issued
};

// ---- k_fp64.cu (compiled with -fmad=false) ----
void launch_geometry(const DevArrays& d, const LaunchCfg& L);
// which: -1 = all three residual passes, 0 = face_state, 1 = cell_grad, 2 = face_flux
void launch_residual_fp64(const DevArrays& d, const LaunchCfg& L, bool viscous, int first_order, int which = -1);
// ---- k_fp64fma.cu (the same binary64 residual with multiply-add contraction: the mixed form) ----
void launch_residual_fp64_contracted(const DevArrays& d, const LaunchCfg& L, bool viscous, int first_order, int which = -1);
void launch_update_fp64(const DevArrays& d, const LaunchCfg& L, bool viscous, int mode, double cfl, int stage, double alpha);
void launch_sweep_level(const DevArrays& d, const LaunchCfg& L, bool viscous, bool forward, int begin, int end, bool fp32);
void launch_sweep_prep(const DevArrays& d, const LaunchCfg& L, bool viscous, bool fp32, bool reset);
void launch_sweep16_level(const DevArrays& d, const LaunchCfg& L, bool forward, int begin, int end);
cudaError_t launch_sweep_flow(const DevArrays& d, const LaunchCfg& L, bool forward, int grid);
cudaError_t launch_sweep_pair64(const DevArrays& d, const LaunchCfg& L, bool forward, int grid);
int sweep_flow_max_grid(bool low, int blocks_per_sm, int threads = 256, bool pf = true);
void launch_inv_diag(const DevArrays& d, const LaunchCfg& L);
// kind of the viscosity array the binary32 sweep staging reads: the residual's form
enum MuKind { MU_F32 = 0, MU_F64 = 1, MU_FF = 2 };
void launch_sweep_prep32(const DevArrays& d, const LaunchCfg& L, bool viscous, int mu_kind);
cudaError_t launch_sweep_flow32(const DevArrays& d, const LaunchCfg& L, bool forward, int grid, bool independent);
int sweep_chain_max_grid(int blocks_per_sm);
bool sweep_chain_fits(int grid, int tbl_bytes);
cudaError_t launch_sweep_chain32(const DevArrays& d, const LaunchCfg& L, bool forward, int grid, bool viscous, int mu_kind);
void launch_chain_static(const DevArrays& d, const LaunchCfg& L);
void launch_cp_ma(const DevArrays& d, const LaunchCfg& L, int begin, int end, double pinf, double uinf, double vinf,
                  double* out);
void launch_face_lr(const DevArrays& d, const LaunchCfg& L, int begin, int end, bool right, d4* out);
void launch_wait_selftest(const DevArrays& d, const LaunchCfg& L, long long limit);
void launch_lusgs_update(const DevArrays& d, const LaunchCfg& L, bool fp32_copy);
void launch_cons_from_prim(const DevArrays& d, const LaunchCfg& L, int begin, int end);
// ---- k_fringe.cu ----
void launch_fringe(const DevArrays& d, const FringePlan& f, const LaunchCfg& L);
// form: 0 binary64, 1 binary32, 2 float-float (the residual arrays read)
void launch_local_dt(const DevArrays& d, const LaunchCfg& L, double cfl, int form);
void launch_wall_distance(const DevArrays& d, const LaunchCfg& L);
void launch_wall_force(const DevArrays& d, const LaunchCfg& L, bool viscous, int form);
// ---- k_sst.cu (compiled with -fmad=false) ----
void launch_sst_residual(const DevArrays& d, const LaunchCfg& L);
void launch_sst_update_mut(const DevArrays& d, const LaunchCfg& L);
// one pass of the coupled model's residual: 0 face values, 1 gradients + F1/F2,
// 2 face fluxes, 3 residual (sum(Fc - Fv) - Q vol) and diagonal
void launch_sst_stage(const DevArrays& d, const LaunchCfg& L, int stage);
// the turbulence LU-SGS sweeps of a coupled step (after the flow's sweeps):
// per-slot constants, forward and backward dataflow sweeps, binary64 or binary32
cudaError_t launch_sst_sweeps(const DevArrays& d, const LaunchCfg& L, bool fp32);
// the same sweeps overlapped with the flow's round-robin sweeps: the per-slot
// constants before the flow's sweeps (coupled: Vn(W_j + dW_j) left to the
// flow's sweep), then one cooperative launch per direction holding both, the
// flow on blocks [0, nflow)
void launch_sst_sweep_prep(const DevArrays& d, const LaunchCfg& L, bool fp32, bool coupled);
cudaError_t launch_sweep_coupled(const DevArrays& d, const LaunchCfg& L, bool forward, bool fp32, int grid, int nflow);
int sweep_coupled_max_grid(bool fp32, int blocks_per_sm, int threads, bool pf);
// W_t += dW_t, k and omega from the updated rho (floored), mu_t (after the flow's update)
void launch_sst_update(const DevArrays& d, const LaunchCfg& L);
// W_t = rho (k, omega) from the current U and k, omega
void launch_sst_cons(const DevArrays& d, const LaunchCfg& L);
int sst_sweep_max_grid(int blocks_per_sm, int threads = 256, bool pf = true);
// ---- k_fp32.cu ----
void launch_residual_fp32(const DevArrays& d, const LaunchCfg& L, bool viscous, int first_order, int which = -1);
void launch_update_fp32(const DevArrays& d, const LaunchCfg& L, bool viscous, int mode, double cfl, int stage, double alpha);
// ---- k_ff.cu (float-float residual of the MIXFF form, compiled with -fmad=false) ----
void launch_residual_ff(const DevArrays& d, const LaunchCfg& L, bool viscous, int first_order, int which = -1);
void launch_update_ff(const DevArrays& d, const LaunchCfg& L, bool viscous, int mode, double cfl, int stage, double alpha);
void launch_to_ff(const DevArrays& d, const LaunchCfg& L, bool geometry);
// ---- k_misc.cu ----
void launch_to_fp32(const DevArrays& d, const LaunchCfg& L, bool geometry);
void launch_norm(const DevArrays& d, const LaunchCfg& L, int which);

}  // namespace cfdgb
