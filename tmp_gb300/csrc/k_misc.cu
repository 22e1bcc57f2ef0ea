// Precision conversions and the residual-norm reductions.
//
// Norms are reduced deterministically: a first pass over fixed per-mesh chunks
// (one block each, fixed tree order) writes one partial per chunk, a second pass
// adds each mesh's partials in chunk order.  The same inputs give the same bits
// on every run.
#include "case.hpp"
#include "fv_kernels.cuh"

namespace cfdgb {

static inline int nblk(int n, int bs) { return (n + bs - 1) / bs; }

__global__ void k_to_f4(int n, const d4* __restrict__ a, float4* __restrict__ b) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    d4 v = ld4(a + i);
    b[i] = make_float4((float)v.x, (float)v.y, (float)v.z, (float)v.w);
}

void launch_to_fp32(const DevArrays& d, const LaunchCfg& L, bool geometry) {
    if (geometry) {
        k_to_f4<<<nblk(d.nf, 256), 256, 0, L.stream>>>(d.nf, d.fg0, d.fg0f);
        k_to_f4<<<nblk(d.nf, 256), 256, 0, L.stream>>>(d.nf, d.fg1, d.fg1f);
        k_to_f4<<<nblk(d.nf, 256), 256, 0, L.stream>>>(d.nf, d.fvis, d.fvisf);
        k_to_f4<<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.cgeo, d.cgeof);
        *L.counter += 4;
    }
    k_to_f4<<<nblk(d.nc, 256), 256, 0, L.stream>>>(d.nc, d.U, d.Uf);
    *L.counter += 1;
}

// which: 0 = sum dW_rho^2, 1 = sum |rho - rho0|, 2 = sum R_rho^2 (sqrt(./n) on the host side of the final pass)
constexpr int kNormThreads = 256;

__global__ void __launch_bounds__(kNormThreads) k_norm_partial(const int4* __restrict__ blocks, int which,
                                                               const d4* __restrict__ dW, const d4* __restrict__ U,
                                                               const d4* __restrict__ W0, const d4* __restrict__ R,
                                                               double* __restrict__ partial,
                                                               unsigned* __restrict__ err) {
    __shared__ double sh[kNormThreads];
    int4 b = blocks[blockIdx.x];
    double acc = 0.0;
    bool bad = false;
    for (int c = b.y + threadIdx.x; c < b.z; c += kNormThreads) {
        double v;
        if (which == 0) {
            double x = dW[c].x;
            v = x * x;
        } else if (which == 1) {
            v = fabs(U[c].x - W0[c].x);
        } else {
            double x = R[c].x;
            v = x * x;
        }
        if (!(v == v)) bad = true;
        acc += v;
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kNormThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
    if (bad) atomicOr(err, ERR_NONPHYS);
}

__global__ void k_norm_final(int nblk_total, const int4* __restrict__ blocks, const double* __restrict__ partial,
                             int nmesh, double* __restrict__ out) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmesh) return;
    double s = 0.0;
    for (int i = 0; i < nblk_total; i++)
        if (blocks[i].x == m) s += partial[i];
    out[m] = s;
}

void launch_norm(const DevArrays& d, const LaunchCfg& L, int which) {
    k_norm_partial<<<d.nblk_norm, kNormThreads, 0, L.stream>>>(d.norm_blocks, which, d.dW, d.U, d.W0, d.R,
                                                               d.norm_partial, d.err);
    k_norm_final<<<nblk(d.nmesh, 128), 128, 0, L.stream>>>(d.nblk_norm, d.norm_blocks, d.norm_partial, d.nmesh,
                                                           d.norm_out);
    *L.counter += 2;
}

}  // namespace cfdgb
