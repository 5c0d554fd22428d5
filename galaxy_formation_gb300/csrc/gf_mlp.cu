// gf_mlp.cu — the smoothing-length guess: a 4 -> 64 -> 64 -> 1 ReLU MLP predicting the log
// distance of a gas particle's 48th nearest neighbour (the radius a full search has to reach)
// from (log cell density, log previous h, leaf count, velocity divergence). Its output starts
// the neighbour-count iteration of the kNN search; the iteration stays the judge, so the
// converged h does not depend on the guess, only the iteration count.
//
// Weights live as float32 masters (for Adam) and bfloat16 copies; every forward and backward
// pass reads the bfloat16 weights and accumulates in float32. Layout of the flat parameter
// vector: W1 (64x4, row j = hidden unit), b1 (64), W2 (64x64), b2 (64), w3 (64), b3.
//   k_mlp_forward ... one thread per sample, weights staged in shared memory as float32;
//   k_mlp_grad ...... one block of 64 samples: per-sample forward/backward, then the block's
//                     outer products (dL/dW2 = D2^T A1 over its samples) in shared memory,
//                     written as a per-block partial; k_mlp_reduce sums the partials in a
//                     fixed order (deterministic gradients);
//   k_mlp_adam ...... Adam on the float32 masters, refreshes the bfloat16 copies.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "gf_mlp.cuh"

namespace gf {

namespace {

constexpr int H = kMlpHidden;
constexpr int kGradBlock = 64;  // samples per gradient block

struct MlpW {  // float32 view in shared memory
    float W1[H * 4], b1[H], W2[H * H], b2[H], w3[H], b3;
};

__device__ void load_weights(MlpW& s, const __nv_bfloat16* __restrict__ p) {
    float* dst = reinterpret_cast<float*>(&s);
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) dst[i] = __bfloat162float(p[i]);
    __syncthreads();
}

__device__ __forceinline__ void normalise(const float* x, const MlpNorm& nm, float* xn) {
#pragma unroll
    for (int i = 0; i < 4; ++i) xn[i] = (x[i] - nm.mean[i]) * nm.inv_std[i];
}

// one thread per sample, layer 2 accumulated column by column: for each hidden unit k of
// layer 1, a1_k is formed and multiplied into the 64 layer-2 sums z (registers) with column k
// of W2 read from shared memory as float4 (one address for the whole warp: a broadcast per 4
// multiply-adds).
constexpr int kFwdThreads = 128;
struct MlpFwdW {  // float32 in shared memory, W2 transposed (row k = column k of W2)
    float W1[H * 4], b1[H], W2T[H * H], b2[H], w3[H], b3;
};

__global__ void __launch_bounds__(kFwdThreads) k_mlp_forward(int n, const float* __restrict__ X, MlpNorm nm,
                                                             const __nv_bfloat16* __restrict__ P, float* __restrict__ Y) {
    __shared__ __align__(16) MlpFwdW w;
    {
        const int o2 = H * 4 + H;  // offset of W2 in the flat parameter vector
        for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) {
            const float v = __bfloat162float(P[i]);
            if (i >= o2 && i < o2 + H * H) {
                const int j = (i - o2) / H, k = (i - o2) % H;
                w.W2T[k * H + j] = v;
            } else {
                reinterpret_cast<float*>(&w)[i] = v;
            }
        }
        __syncthreads();
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float xn[4];
        normalise(X + 4 * size_t(i), nm, xn);
        float z[H];
#pragma unroll
        for (int j = 0; j < H; ++j) z[j] = w.b2[j];
#pragma unroll 1
        for (int k = 0; k < H; ++k) {
            const float4 r = *reinterpret_cast<const float4*>(&w.W1[k * 4]);
            float a = w.b1[k];
            a = fmaf(r.x, xn[0], a);
            a = fmaf(r.y, xn[1], a);
            a = fmaf(r.z, xn[2], a);
            a = fmaf(r.w, xn[3], a);
            a = __bfloat162float(__float2bfloat16(fmaxf(a, 0.f)));  // bfloat16 layer-2 input
            const float4* col = reinterpret_cast<const float4*>(&w.W2T[k * H]);
#pragma unroll
            for (int j4 = 0; j4 < H / 4; ++j4) {
                const float4 c = col[j4];
                z[4 * j4] = fmaf(c.x, a, z[4 * j4]);
                z[4 * j4 + 1] = fmaf(c.y, a, z[4 * j4 + 1]);
                z[4 * j4 + 2] = fmaf(c.z, a, z[4 * j4 + 2]);
                z[4 * j4 + 3] = fmaf(c.w, a, z[4 * j4 + 3]);
            }
        }
        float y = w.b3;
#pragma unroll
        for (int j = 0; j < H; ++j) y = fmaf(w.w3[j], fmaxf(z[j], 0.f), y);
        Y[i] = y * nm.t_std + nm.t_mean;  // log d48
    }
}

// one block = kGradBlock samples (indices idx[b0 .. b0+64), or b0.. when idx is null).
// Per-sample vectors are staged in shared memory (dynamic, ~70 KB): x, a1, z2, d (d2 then
// d1). Thread t owns sample t in the per-sample phases and hidden unit t in the reductions.
constexpr int kLd = H + 1;  // padded row stride
constexpr size_t kGradSmem = sizeof(MlpW) + sizeof(float) * (3 * kGradBlock * kLd + kGradBlock * 4 + kGradBlock);

__global__ void __launch_bounds__(kGradBlock) k_mlp_grad(int n, const int* __restrict__ idx, const float* __restrict__ X,
                                                         const float* __restrict__ T, MlpNorm nm,
                                                         const __nv_bfloat16* __restrict__ P, float inv_batch,
                                                         float* __restrict__ partial, float* __restrict__ loss_part) {
    extern __shared__ float smem[];
    MlpW& w = *reinterpret_cast<MlpW*>(smem);
    float* sA1 = smem + sizeof(MlpW) / sizeof(float);
    float* sZ2 = sA1 + kGradBlock * kLd;
    float* sD = sZ2 + kGradBlock * kLd;
    float* sX = sD + kGradBlock * kLd;
    float* sR = sX + kGradBlock * 4;
    load_weights(w, P);
    const int t = threadIdx.x;
    const int s = blockIdx.x * kGradBlock + t;
    const bool ok = s < n;
    const int i = ok ? (idx ? idx[s] : s) : 0;
    float xn[4] = {0.f, 0.f, 0.f, 0.f};
    if (ok) normalise(X + 4 * size_t(i), nm, xn);
#pragma unroll
    for (int q = 0; q < 4; ++q) sX[t * 4 + q] = xn[q];
    // forward, staged in shared memory
    for (int j = 0; j < H; ++j) {
        float z = w.b1[j];
#pragma unroll
        for (int q = 0; q < 4; ++q) z = fmaf(w.W1[j * 4 + q], xn[q], z);
        sA1[t * kLd + j] = ok ? fmaxf(z, 0.f) : 0.f;
    }
    float y = w.b3;
    for (int j = 0; j < H; ++j) {
        float z = w.b2[j];
        for (int k = 0; k < H; ++k) z = fmaf(w.W2[j * H + k], sA1[t * kLd + k], z);
        sZ2[t * kLd + j] = ok ? z : 0.f;
        y = fmaf(w.w3[j], fmaxf(z, 0.f), y);
    }
    float r = 0.f;
    if (ok) {
        const float tn = (T[i] - nm.t_mean) / nm.t_std;
        r = (y - tn) * inv_batch;  // d(0.5 mean (y - t)^2)/dy
        loss_part[s] = 0.5f * (y - tn) * (y - tn) * inv_batch;
    }
    sR[t] = r;
    for (int j = 0; j < H; ++j) sD[t * kLd + j] = sZ2[t * kLd + j] > 0.f ? r * w.w3[j] : 0.f;  // d2
    __syncthreads();
    float* out = partial + size_t(blockIdx.x) * kMlpParams;
    const int j = t;  // hidden unit owned in the reductions (kGradBlock == H)
    {   // dL/dW2 row j = sum_q d2[q][j] a1[q][:], dL/db2[j]
        float g[H];
#pragma unroll
        for (int k = 0; k < H; ++k) g[k] = 0.f;
        float gb = 0.f;
        for (int q = 0; q < kGradBlock; ++q) {
            const float dq = sD[q * kLd + j];
            gb += dq;
#pragma unroll
            for (int k = 0; k < H; ++k) g[k] = fmaf(dq, sA1[q * kLd + k], g[k]);
        }
#pragma unroll
        for (int k = 0; k < H; ++k) out[kOffW2 + j * H + k] = g[k];
        out[kOffB2 + j] = gb;
        // dL/dw3[j] = sum_q r[q] a2[q][j], dL/db3 = sum_q r[q]
        float gw = 0.f;
        for (int q = 0; q < kGradBlock; ++q) gw = fmaf(sR[q], fmaxf(sZ2[q * kLd + j], 0.f), gw);
        out[kOffW3 + j] = gw;
        if (t == 0) {
            float g3 = 0.f;
            for (int q = 0; q < kGradBlock; ++q) g3 += sR[q];
            out[kOffB3] = g3;
        }
    }
    __syncthreads();
    // d1[t][k] = sum_j d2[t][j] W2[j][k] [a1[t][k] > 0], into sZ2 (no longer needed)
    for (int k = 0; k < H; ++k) {
        float d = 0.f;
        for (int jj = 0; jj < H; ++jj) d = fmaf(sD[t * kLd + jj], w.W2[jj * H + k], d);
        sZ2[t * kLd + k] = sA1[t * kLd + k] > 0.f ? d : 0.f;
    }
    __syncthreads();
    {   // dL/dW1 row j, dL/db1[j]
        float g0 = 0.f, g1 = 0.f, g2 = 0.f, g3 = 0.f, gb = 0.f;
        for (int q = 0; q < kGradBlock; ++q) {
            const float dq = sZ2[q * kLd + j];
            g0 = fmaf(dq, sX[q * 4 + 0], g0);
            g1 = fmaf(dq, sX[q * 4 + 1], g1);
            g2 = fmaf(dq, sX[q * 4 + 2], g2);
            g3 = fmaf(dq, sX[q * 4 + 3], g3);
            gb += dq;
        }
        out[kOffW1 + j * 4 + 0] = g0;
        out[kOffW1 + j * 4 + 1] = g1;
        out[kOffW1 + j * 4 + 2] = g2;
        out[kOffW1 + j * 4 + 3] = g3;
        out[kOffB1 + j] = gb;
    }
}

// fixed-order sum of the per-block partials
__global__ void k_mlp_reduce(int nblocks, const float* __restrict__ partial, float* __restrict__ grad) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kMlpParams) return;
    float s = 0.f;
    for (int b = 0; b < nblocks; ++b) s += partial[size_t(b) * kMlpParams + p];
    grad[p] = s;
}

__global__ void k_mlp_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                           float* __restrict__ v, __nv_bfloat16* __restrict__ wb, float lr, float b1, float b2,
                           float eps, float c1, float c2) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kMlpParams) return;
    const float gg = g[p];
    const float mm = b1 * m[p] + (1.f - b1) * gg;
    const float vv = b2 * v[p] + (1.f - b2) * gg * gg;
    m[p] = mm;
    v[p] = vv;
    const float nw = w[p] - lr * (mm * c1) / (sqrtf(vv * c2) + eps);
    w[p] = nw;
    wb[p] = __float2bfloat16(nw);
}

__global__ void k_to_bf16(int n, const float* __restrict__ a, __nv_bfloat16* __restrict__ b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = __float2bfloat16(a[i]);
}

__global__ void k_sample_idx(int batch, int n, unsigned long long seed, int* __restrict__ idx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= batch) return;
    unsigned long long x = seed ^ (0x9E3779B97F4A7C15ull * (i + 1));
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    idx[i] = int(x % (unsigned long long)n);
}

}  // namespace

static Mlp g_mlp;
Mlp& mlp() { return g_mlp; }

void Mlp::init(unsigned seed, cudaStream_t s) {
    std::mt19937 rng(seed);
    std::vector<float> p(kMlpParams, 0.f);
    std::normal_distribution<float> n1(0.f, std::sqrt(2.f / 4.f)), n2(0.f, std::sqrt(2.f / H)),
        n3(0.f, std::sqrt(1.f / H));
    for (int i = 0; i < H * 4; ++i) p[kOffW1 + i] = n1(rng);
    for (int i = 0; i < H * H; ++i) p[kOffW2 + i] = n2(rng);
    for (int i = 0; i < H; ++i) p[kOffW3 + i] = n3(rng);
    set_params(p.data(), s);
    step_count = 0;
    GF_CUDA(cudaMemsetAsync(m.get<float>(kMlpParams), 0, sizeof(float) * kMlpParams, s));
    GF_CUDA(cudaMemsetAsync(v.get<float>(kMlpParams), 0, sizeof(float) * kMlpParams, s));
    ready = true;
}

void Mlp::set_params(const float* host, cudaStream_t s) {
    tensor_cores = tensor_cores == 0 ? 0 : -1;  // re-check with the new weights
    float* d = w.get<float>(kMlpParams);
    GF_CUDA(cudaMemcpyAsync(d, host, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, s));
    k_to_bf16<<<div_up(kMlpParams, 256), 256, 0, s>>>(kMlpParams, d, wb.get<__nv_bfloat16>(kMlpParams));
    GF_CHECK_LAUNCH();
    ready = true;
}

void Mlp::get_params(float* host, cudaStream_t s) {
    GF_CUDA(cudaMemcpyAsync(host, w.p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, s));
    GF_CUDA(cudaStreamSynchronize(s));
}

static void forward_cuda_cores(int n, const float* X, const MlpNorm& nm, const __nv_bfloat16* P, float* Y,
                               cudaStream_t s) {
    const int blocks = std::min(div_up(n, kFwdThreads), 8 * ctx().sms);
    k_mlp_forward<<<blocks, kFwdThreads, 0, s>>>(n, X, nm, P, Y);
    GF_CHECK_LAUNCH();
}

// Inference: layer 2 on the tensor cores once the first call has shown that they agree with
// the CUDA-core kernel (both use bfloat16 layer-2 inputs and float32 accumulation; only the
// summation order differs); otherwise on the CUDA cores.
void Mlp::predict(int n, const float* X, float* Y, cudaStream_t s) {
    if (n <= 0) return;
    const __nv_bfloat16* P = wb.as<__nv_bfloat16>();
    if (tensor_cores < 0) {
        const int m = std::min(n, 8192);
        float* y2 = check_y.get<float>(m);
        forward_cuda_cores(m, X, norm, P, y2, s);
        mlp_forward_tc(m, X, norm, P, Y, s);
        std::vector<float> a(m), b(m);
        GF_CUDA(cudaMemcpyAsync(a.data(), y2, sizeof(float) * m, cudaMemcpyDeviceToHost, s));
        GF_CUDA(cudaMemcpyAsync(b.data(), Y, sizeof(float) * m, cudaMemcpyDeviceToHost, s));
        GF_CUDA(cudaStreamSynchronize(s));
        float worst = 0.f;
        for (int i = 0; i < m; ++i) worst = std::max(worst, std::fabs(a[i] - b[i]) / (1.f + std::fabs(a[i])));
        tensor_cores = worst <= 1e-4f ? 1 : 0;
    }
    if (tensor_cores == 1)
        mlp_forward_tc(n, X, norm, P, Y, s);
    else
        forward_cuda_cores(n, X, norm, P, Y, s);
}

double Mlp::gradient(int n, const int* idx, const float* X, const float* T, float* grad, cudaStream_t s) {
    const int nb = div_up(n, kGradBlock);
    float* part = partial.get<float>(size_t(nb) * kMlpParams);
    float* lp = loss_buf.get<float>(size_t(nb) * kGradBlock);
    GF_CUDA(cudaMemsetAsync(lp, 0, sizeof(float) * size_t(nb) * kGradBlock, s));
    static bool attr = false;
    if (!attr) {
        GF_CUDA(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kGradSmem)));
        attr = true;
    }
    k_mlp_grad<<<nb, kGradBlock, kGradSmem, s>>>(n, idx, X, T, norm, wb.as<__nv_bfloat16>(), 1.f / float(n), part,
                                                 lp);
    GF_CHECK_LAUNCH();
    k_mlp_reduce<<<div_up(kMlpParams, 256), 256, 0, s>>>(nb, part, grad);
    GF_CHECK_LAUNCH();
    return 0.0;
}

double train_on(Mlp& M, const float* X, const float* T, int steps, int batch, double lr, cudaStream_t s) {
    return M.train_data(X, T, steps, batch, lr, s);
}

double Mlp::train(int steps, int batch, double lr, cudaStream_t s) {
    return train_data(X.as<float>(), T.as<float>(), steps, batch, lr, s);
}

double Mlp::train_data(const float* dX, const float* dT, int steps, int batch, double lr, cudaStream_t s) {
    float* g = grad.get<float>(kMlpParams);
    int* ix = idx.get<int>(batch);
    double last = 0;
    for (int it = 0; it < steps; ++it) {
        k_sample_idx<<<div_up(batch, 256), 256, 0, s>>>(batch, n_data, 0x5eedull + 7919ull * step_count, ix);
        GF_CHECK_LAUNCH();
        gradient(batch, ix, dX, dT, g, s);
        ++step_count;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f / (1.f - std::pow(b1, float(step_count)));
        const float c2 = 1.f / (1.f - std::pow(b2, float(step_count)));
        k_mlp_adam<<<div_up(kMlpParams, 256), 256, 0, s>>>(w.as<float>(), g, m.as<float>(), v.as<float>(),
                                                          wb.as<__nv_bfloat16>(), float(lr), b1, b2, 1e-8f, c1, c2);
        GF_CHECK_LAUNCH();
    }
    // mean loss of the last batch
    const int nb = div_up(batch, kGradBlock);
    std::vector<float> lp(size_t(nb) * kGradBlock);
    GF_CUDA(cudaMemcpyAsync(lp.data(), loss_buf.p, sizeof(float) * lp.size(), cudaMemcpyDeviceToHost, s));
    GF_CUDA(cudaStreamSynchronize(s));
    for (float x : lp) last += x;
    return last;
}

}  // namespace gf
