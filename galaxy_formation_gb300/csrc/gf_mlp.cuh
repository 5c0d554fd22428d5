// gf_mlp.cuh — the smoothing-length MLP (gf_mlp.cu).
#pragma once

#include <cuda_bf16.h>

#include "gf_common.cuh"

namespace gf {

constexpr int kMlpHidden = 64;
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kMlpHidden * 4;
constexpr int kOffW2 = kOffB1 + kMlpHidden;
constexpr int kOffB2 = kOffW2 + kMlpHidden * kMlpHidden;
constexpr int kOffW3 = kOffB2 + kMlpHidden;
constexpr int kOffB3 = kOffW3 + kMlpHidden;
constexpr int kMlpParams = kOffB3 + 1;  // 4545

// Standardisation of the 4 inputs and of the target (log distance of the 48th nearest).
struct MlpNorm {
    float mean[4] = {0.f, 0.f, 0.f, 0.f};
    float inv_std[4] = {1.f, 1.f, 1.f, 1.f};
    float t_mean = 0.f, t_std = 1.f;
};

struct Mlp {
    bool ready = false;
    int n_data = 0;
    long long step_count = 0;
    MlpNorm norm;
    DevBuf w, wb, m, v, grad, partial, loss_buf, idx, X, T, check_y;
    // tensor-core inference: -1 not checked yet, 1 in use (agrees with the CUDA-core kernel
    // on the first call), 0 not used
    int tensor_cores = -1;

    void init(unsigned seed, cudaStream_t s);
    void set_params(const float* host, cudaStream_t s);
    void get_params(float* host, cudaStream_t s);
    // predictions (log distance of the 48th nearest) of n samples (X: n x 4 float, device)
    void predict(int n, const float* X, float* Y, cudaStream_t s);
    // gradient of 0.5 mean (y - t)^2 (standardised) over samples idx[0..n) (or 0..n) into grad
    double gradient(int n, const int* idx, const float* X, const float* T, float* grad, cudaStream_t s);
    // Adam steps on random minibatches of the stored training set; returns the last loss
    double train(int steps, int batch, double lr, cudaStream_t s);
    double train_data(const float* X, const float* T, int steps, int batch, double lr, cudaStream_t s);
};

Mlp& mlp();
// The inference of Mlp::predict with layer 2 on the tensor cores (gf_mlp_tc.cu).
void mlp_forward_tc(int n, const float* X, const MlpNorm& nm, const __nv_bfloat16* P, float* Y, cudaStream_t s);
// Adam steps on random minibatches of the device training set (X n x 4, T n); returns the
// mean loss of the last minibatch (standardised units).
double train_on(Mlp& M, const float* X, const float* T, int steps, int batch, double lr, cudaStream_t s);

}  // namespace gf
