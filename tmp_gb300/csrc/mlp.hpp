// The learned relaxation network (k_mlp.cu): device buffers and launchers.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace cfdgb {

struct DevArrays;
struct LaunchCfg;

constexpr int kMlpIn = 12, kMlpHidden = 64, kMlpOut = 2;
constexpr int kMlpParams = kMlpHidden * kMlpIn + kMlpHidden + kMlpHidden * kMlpHidden + kMlpHidden +
                           kMlpOut * kMlpHidden + kMlpOut;  // 5122

// Layout of p: W1[64][12], b1[64], W2[64][64], b2[64], W3[2][64], b3[2];
// norm: mean[12], scale[12] of the input transform.
struct MlpNet {
    float* p = nullptr;           // fp32 master weights
    float* m1 = nullptr;          // Adam moments
    float* m2 = nullptr;
    float* G = nullptr;           // gradient of the last batch
    float* norm = nullptr;        // [24]
    __nv_bfloat16* wq = nullptr;  // bf16 weights used by every forward pass
    long long t = 0;              // Adam step count
    // training scratch for `cap` rows
    int cap = 0;
    float *XH = nullptr, *H1 = nullptr, *H2 = nullptr, *D1 = nullptr, *D2 = nullptr, *DO = nullptr, *L = nullptr;
    int* idx = nullptr;
    double* losses = nullptr;
    int losses_cap = 0;
    cudaError_t init();
    cudaError_t reserve(int B);
    void quantize(cudaStream_t s) const;
    ~MlpNet();
};

void launch_case_features(const DevArrays& d, const LaunchCfg& L, float* X);
// samples[nsamp]: the cells the network is evaluated on, mesh by mesh;
// samp_off[nmesh + 1]: each mesh's range in samples.
void launch_learned_update(const DevArrays& d, const LaunchCfg& L, const MlpNet& net, bool apply_cfl, float spread,
                           const int* samples, const int* samp_off, int nsamp, bool fp32_copy);
cudaError_t mlp_forward(const MlpNet& net, const float* X, long long n, float* Y, cudaStream_t s);
// Loss and gradient of B rows (idx[b], or rows 0..B-1 when idx is null); the
// loss (sum over rows of M-weighted squared errors times inv_msum) goes to d_loss.
cudaError_t mlp_batch_grad(MlpNet& net, const int* idx, int B, const float* X, const float* T, const float* M,
                           float inv_msum, double* d_loss, cudaStream_t s);
cudaError_t mlp_adam(MlpNet& net, float lr, cudaStream_t s);
cudaError_t mlp_batch_rows(MlpNet& net, int B, long long n, unsigned long long seed, cudaStream_t s);

}  // namespace cfdgb
