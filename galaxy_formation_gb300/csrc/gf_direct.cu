// gf_direct.cu — exact float64 direct sum (cpp/nbody.cpp:428-441): the oracle of every
// Barnes-Hut error report. One thread per target, sources staged through shared memory in
// tiles of 256 (x, y, z, m). Same pair formula as the reference:
//   a_i += m_j d / (r2 sqrt(r2)),  r2 = |d|^2 + eps^2,  d = x_j - x_i.
#include "gf_common.cuh"

namespace gf {

namespace {

constexpr int kDirThreads = 256;

__global__ void __launch_bounds__(kDirThreads) k_direct(int n, const double* __restrict__ pos,
                                                        const double* __restrict__ mass, int nt,
                                                        const int64_t* __restrict__ targets,
                                                        double* __restrict__ acc, double eps2) {
    __shared__ double4 src[kDirThreads];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool ok = t < nt;
    const int64_t i = ok ? (targets ? targets[t] : t) : 0;
    const double xi = ok ? pos[3 * i] : 0, yi = ok ? pos[3 * i + 1] : 0, zi = ok ? pos[3 * i + 2] : 0;
    double ax = 0, ay = 0, az = 0;
    for (int base = 0; base < n; base += kDirThreads) {
        const int j = base + threadIdx.x;
        __syncthreads();
        src[threadIdx.x] = j < n ? make_double4(pos[3 * size_t(j)], pos[3 * size_t(j) + 1],
                                                pos[3 * size_t(j) + 2], mass[j])
                                 : make_double4(0, 0, 0, 0);
        __syncthreads();
        const int cnt = min(kDirThreads, n - base);
        for (int q = 0; q < cnt; ++q) {
            const double4 s = src[q];
            const double dx = s.x - xi, dy = s.y - yi, dz = s.z - zi;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            const double f = s.w / (r2 * sqrt(r2));
            ax += f * dx;
            ay += f * dy;
            az += f * dz;
        }
    }
    if (ok) {
        acc[3 * size_t(t)] = ax;
        acc[3 * size_t(t) + 1] = ay;
        acc[3 * size_t(t) + 2] = az;
    }
}

}  // namespace

void direct_sum(int n, const double* pos, const double* mass, int nt, const int64_t* targets,
                double* acc, double eps, cudaStream_t s) {
    if (nt <= 0) return;
    k_direct<<<div_up(nt, kDirThreads), kDirThreads, 0, s>>>(n, pos, mass, nt, targets, acc, eps * eps);
    GF_CHECK_LAUNCH();
}

}  // namespace gf
