// gf_sph32.cu — the mixed-precision form of sph_forces (galaxy_formation/sph.py:57-106):
// the same density / pressure / viscosity / du/dt / Courant formulas in float32, with
//   * positions split hi + lo (x = float(x) + float(x - float(x))), so a pair separation
//     (hi_i - hi_j) + (lo_i - lo_j) keeps ~1e-7 relative accuracy however far the pair
//     sits from the origin;
//   * Kahan-compensated accumulation of every neighbour sum (density, the three
//     acceleration components and du/dt);
//   * packed float4 records, so one neighbour costs two 32-byte sectors in the force pass:
//       A = (x_hi, y_hi, z_hi, h), B = (x_lo, y_lo, z_lo, m), C = (vx, vy, vz, 0),
//       D = (rho, (gamma-1) u / rho = P / rho^2, sound speed, 1/h)  [written by the density
//       pass, which also evaluates the equation of state].
// Inputs and outputs stay float64 (gas-local order, neighbour rows of stride ld); only the
// arithmetic is float32. Threads visit particles in `order` (e.g. Morton order of the
// neighbour-search tree) when given, so neighbouring threads share cache lines.
#include "gf_sph.cuh"

namespace gf {

namespace {

constexpr int kThreads = 256;
constexpr float kInvPi = 0.318309886183790671538f;

struct Kahan {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float v) {
        const float y = v - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

__global__ void k_sph32_pack(int n, const double* __restrict__ pos, const double* __restrict__ vel,
                             const double* __restrict__ mass, const double* __restrict__ h,
                             float4* __restrict__ A, float4* __restrict__ B, float4* __restrict__ C) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = pos[3 * size_t(i)], y = pos[3 * size_t(i) + 1], z = pos[3 * size_t(i) + 2];
    const float fx = float(x), fy = float(y), fz = float(z);
    A[i] = make_float4(fx, fy, fz, float(h[i]));
    B[i] = make_float4(float(x - double(fx)), float(y - double(fy)), float(z - double(fz)), float(mass[i]));
    C[i] = make_float4(float(vel[3 * size_t(i)]), float(vel[3 * size_t(i) + 1]), float(vel[3 * size_t(i) + 2]), 0.f);
}

// M4 kernel without its 1/(pi h^3) factor (sph.py:31-40)
__device__ __forceinline__ float w_shape(float q) {
    if (q < 1.f) return 1.f - 1.5f * q * q + 0.75f * q * q * q;
    if (q < 2.f) {
        const float t = 2.f - q;
        return 0.25f * t * t * t;
    }
    return 0.f;
}

// dW/dr without its 1/(pi h^4) factor (sph.py:43-54, before the division by r)
__device__ __forceinline__ float dw_shape(float q) {
    if (q < 1.f) return -3.f * q + 2.25f * q * q;
    if (q < 2.f) {
        const float t = 2.f - q;
        return -0.75f * t * t;
    }
    return 0.f;
}

template <class Idx>
__global__ void k_sph32_density(int n, int k, int ld, const Idx* __restrict__ nb, const int* __restrict__ order,
                                const float4* __restrict__ A, const float4* __restrict__ B,
                                const double* __restrict__ u, float gamma, float4* __restrict__ D,
                                double* __restrict__ rho_out, Subset sub) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    int i;
    if (!subset_item(sub, t, n, order, i)) return;  // others keep their last density record
    const float4 ai = A[i], bi = B[i];
    const float inv_h = 1.f / ai.w;
    Kahan s;
    // unrolled: the neighbours' loads of several iterations are in flight together (the sums
    // keep their order)
#pragma unroll 8
    for (int jj = 0; jj < k; ++jj) {
        const int j = int(nb[size_t(i) * ld + jj]);
        const float4 aj = A[j], bj = B[j];
        const float dx = (ai.x - aj.x) + (bi.x - bj.x);
        const float dy = (ai.y - aj.y) + (bi.y - bj.y);
        const float dz = (ai.z - aj.z) + (bi.z - bj.z);
        const float r = sqrtf(dx * dx + dy * dy + dz * dz);
        s.add(bj.w * w_shape(r * inv_h));
    }
    const float rho = s.s * (inv_h * inv_h * inv_h * kInvPi);
    const float ui = float(u[i]);
    D[i] = make_float4(rho, (gamma - 1.f) * ui / rho, sqrtf(gamma * (gamma - 1.f) * ui), inv_h);
    rho_out[i] = rho;
}

template <class Idx>
__global__ void k_sph32_force(int n, int k, int ld, const Idx* __restrict__ nb, const int* __restrict__ order,
                              const float4* __restrict__ A, const float4* __restrict__ B,
                              const float4* __restrict__ C, const float4* __restrict__ D, float alpha,
                              float beta, double* __restrict__ acc, double* __restrict__ dudt,
                              double* __restrict__ dt_i, float* __restrict__ divv, Subset sub) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    int i;
    if (!subset_item(sub, t, n, order, i)) return;
    const float4 ai = A[i], bi = B[i], ci = C[i], di = D[i];
    const float hi = ai.w, inv_hi = di.w, rhoi = di.x, pri = di.y, csi = di.z;
    const float ih2 = inv_hi * inv_hi;
    const float s4i = ih2 * ih2 * kInvPi;
    Kahan ax, ay, az, du, dv;
    float mu_max = 0.f;
#pragma unroll 4
    for (int jj = 0; jj < k; ++jj) {
        const int j = int(nb[size_t(i) * ld + jj]);
        if (j == i) continue;
        const float4 aj = A[j], bj = B[j], cj = C[j], dj = D[j];
        const float dx = (ai.x - aj.x) + (bi.x - bj.x);
        const float dy = (ai.y - aj.y) + (bi.y - bj.y);
        const float dz = (ai.z - aj.z) + (bi.z - bj.z);
        const float r2 = dx * dx + dy * dy + dz * dz;
        const float r = sqrtf(r2);
        const float inv_r = 1.f / fmaxf(r, 1e-30f);
        const float ihj2 = dj.w * dj.w;
        const float gi = s4i * dw_shape(r * inv_hi) * inv_r;
        const float gj = ihj2 * ihj2 * kInvPi * dw_shape(r * dj.w) * inv_r;
        const float vr = (ci.x - cj.x) * dx + (ci.y - cj.y) * dy + (ci.z - cj.z) * dz;
        float visc = 0.f;
        if (vr < 0.f) {
            const float hb = 0.5f * (hi + aj.w);
            const float mu = hb * vr / (r2 + 0.01f * hb * hb);
            mu_max = fmaxf(mu_max, -mu);
            visc = (-alpha * 0.5f * (csi + dj.z) * mu + beta * mu * mu) / (0.5f * (rhoi + dj.x));
        }
        const float gb = 0.5f * (gi + gj);
        const float f = pri * gi + dj.y * gj + visc * gb;
        const float mf = bj.w * f;
        ax.add(-mf * dx);
        ay.add(-mf * dy);
        az.add(-mf * dz);
        du.add(bj.w * (pri * gi + 0.5f * visc * gb) * vr);
        dv.add(bj.w * vr * gi);
    }
    if (divv) divv[i] = -dv.s / rhoi;
    acc[3 * size_t(i)] = ax.s;
    acc[3 * size_t(i) + 1] = ay.s;
    acc[3 * size_t(i) + 2] = az.s;
    dudt[i] = du.s;
    dt_i[i] = 0.3 * double(hi) / (double(csi) + 1.2 * (double(alpha) * csi + double(beta) * mu_max) + 1e-30);
}

}  // namespace

template <class Idx>
void sph_forces32(Sph32Scratch& S, int n, int k, int ld, const int* order, const double* pos, const double* vel,
                  const double* mass, const Idx* nb, const double* h, const double* u, double gamma, double alpha,
                  double beta, double* rho, double* acc, double* dudt, double* dt_i, cudaStream_t s, float* divv,
                  Subset sub) {
    if (n <= 0) return;
    const int grid = div_up(n, kThreads);
    float4* A = S.A.get<float4>(n);
    float4* B = S.B.get<float4>(n);
    float4* C = S.C.get<float4>(n);
    float4* D = S.D.get<float4>(n);
    k_sph32_pack<<<grid, kThreads, 0, s>>>(n, pos, vel, mass, h, A, B, C);
    GF_CHECK_LAUNCH();
    {
        ProfScope ps(kStSphDensity, s);
        k_sph32_density<Idx><<<grid, kThreads, 0, s>>>(n, k, ld, nb, order, A, B, u, float(gamma), D, rho, sub);
        GF_CHECK_LAUNCH();
    }
    ProfScope ps(kStSphForce, s);
    k_sph32_force<Idx><<<grid, kThreads, 0, s>>>(n, k, ld, nb, order, A, B, C, D, float(alpha), float(beta), acc,
                                                 dudt, dt_i, divv, sub);
    GF_CHECK_LAUNCH();
}

template void sph_forces32<int64_t>(Sph32Scratch&, int, int, int, const int*, const double*, const double*,
                                    const double*, const int64_t*, const double*, const double*, double, double,
                                    double, double*, double*, double*, double*, cudaStream_t, float*,
                                    Subset);
template void sph_forces32<int>(Sph32Scratch&, int, int, int, const int*, const double*, const double*,
                                const double*, const int*, const double*, const double*, double, double, double,
                                double*, double*, double*, double*, cudaStream_t, float*, Subset);

}  // namespace gf
