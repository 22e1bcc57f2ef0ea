// Residual norm over a caller-owned device array, with no device allocation.
//
// Some callers cannot allocate device memory while they run: a host solver
// that reserves all of its device memory at start-up and forbids allocation
// inside the time loop (fixed footprint, no allocator stalls), or code that
// issues work while another framework's pool owns the device memory.  This
// entry point serves them: the only scratch it needs (one partial sum per
// 8192-record chunk) lives in a file-scope __device__ array.
//
// Limits and sharing rules:
//   * at most kNoAllocMaxChunks chunks, i.e. n <= 4096 * 8192 = 33,554,432
//     records; larger n is rejected with CFD_ERR_ARG;
//   * the array is global to the library: every call on a device shares it and
//     it keeps the last call's partial sums (each call writes every slot it
//     reads, so nothing needs clearing);  calls that overlap on the GPU (on
//     different streams, or from different threads) race on it and must be
//     serialised by the caller;
//   * every GPU that loads the library holds the 32 KiB array until exit;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (once per device, with that device current), so make
//     that first call before any stream capture begins; the address is cached
//     for the life of the process, so a device reset while the library is
//     loaded is not supported;
//   * a NaN record gives a NaN result and CFD_OK (no device error word here).
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/cfdgb.h"

namespace cfdgb {
int set_last_error(int code, const std::string& msg);
}

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocChunk = 8192;        // records per block (same chunking as the case norms)
constexpr int kNoAllocMaxChunks = 4096;    // 32 KiB of partial sums
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partial[kNoAllocMaxChunks];

std::mutex g_mu;
double* g_ptr[kMaxDevices] = {nullptr};

__global__ void __launch_bounds__(kNoAllocThreads) k_noalloc_partial(const double* __restrict__ rec, int n,
                                                                     double* __restrict__ partial) {
    __shared__ double sh[kNoAllocThreads];
    int b0 = blockIdx.x * kNoAllocChunk;
    int b1 = min(b0 + kNoAllocChunk, n);
    double acc = 0.0;
    for (int c = b0 + threadIdx.x; c < b1; c += kNoAllocThreads) {
        double x = rec[4 * (size_t)c];
        acc += x * x;
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kNoAllocThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void k_noalloc_final(const double* __restrict__ partial, int nchunk, int n, int rms,
                                double* __restrict__ out) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    double s = 0.0;
    for (int i = 0; i < nchunk; i++) s += partial[i];
    *out = rms ? sqrt(s / (double)n) : s;
}

// message goes to the same per-thread slot that cfd_last_error() reads
int set_error(int code, const std::string& m) { return cfdgb::set_last_error(code, m); }

}  // namespace

extern "C" int cfd_residual_norm_noalloc(const double* d_records, int n, int which, double* d_out, void* stream) {
    if (!d_records || !d_out) return set_error(CFD_ERR_ARG, "cfd_residual_norm_noalloc: null device pointer");
    if (n <= 0) return set_error(CFD_ERR_ARG, "cfd_residual_norm_noalloc: n must be positive");
    if (which != CFD_NORM_DW_RHO2 && which != CFD_NORM_L2_R_RHO)
        return set_error(CFD_ERR_ARG, "cfd_residual_norm_noalloc: only CFD_NORM_DW_RHO2 and CFD_NORM_L2_R_RHO");
    long long nchunk = ((long long)n + kNoAllocChunk - 1) / kNoAllocChunk;
    if (nchunk > kNoAllocMaxChunks)
        return set_error(CFD_ERR_ARG, "cfd_residual_norm_noalloc: n = " + std::to_string(n) + " exceeds the " +
                                          std::to_string((long long)kNoAllocMaxChunks * kNoAllocChunk) +
                                          "-record limit of the static scratch array");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(CFD_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return set_error(CFD_ERR_ARG, "cfd_residual_norm_noalloc: device index too large");
    double* scratch;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_ptr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_partial);
            if (e != cudaSuccess)
                return set_error(CFD_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_ptr[dev] = static_cast<double*>(p);
        }
        scratch = g_ptr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    k_noalloc_partial<<<(int)nchunk, kNoAllocThreads, 0, s>>>(d_records, n, scratch);
    k_noalloc_final<<<1, 32, 0, s>>>(scratch, (int)nchunk, n, which == CFD_NORM_L2_R_RHO, d_out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CFD_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    return CFD_OK;
}
