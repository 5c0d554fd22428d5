// gf_stars.cu — star formation and supernova feedback (galaxy_formation/star_formation.py:35-65)
// on the device, for the step loop.
//
//   form_stars: the gas of the last SPH evaluation that is dense (rho > rho_sf) and cold
//     (T < 3e4 K) turns into a star with probability p = 1 - exp(-sf_eff dt / t_ff),
//     t_ff = sqrt(3 pi / (32 rho)) (G = 1). The reference draws rng.uniform(size=#dense) from
//     NumPy's PCG64 in the order of the dense particles; here the dense particle of rank r takes
//     draw r + 1 of the same stream, computed independently by jumping the 128-bit LCG ahead
//     (O(log r) affine compositions), and the stream then advances by #dense: the same uniforms
//     as the reference's, so the same particles become stars.
//   supernova_feedback: each new star heats its fb_ngb nearest gas particles (float64
//     distances, brute force over the current gas: new stars are few) with
//     du = E / k / (m_target MSUN MSUN_G) / U_CGS, E = fb_eff E_SN / MSUN_G * m_star MSUN MSUN_G,
//     and switches their cooling off until t + fb_myr / MYR.
// Float64 with the reference's order of operations; the heating sums of a particle heated by
// several stars are atomic (their order, hence the last bit, differs from np.add.at's).
#include <algorithm>

#include "gf_stars.cuh"

namespace gf {

namespace {

constexpr int kThreads = 256;
constexpr double kPi = 3.14159265358979323846;
constexpr double kTSfMax = 3e4;  // star_formation.py:29
constexpr int kGas = 0, kStar = 1;
constexpr int kFbThreads = 128;
constexpr int kFbMaxK = 64;  // largest fb_ngb handled

using u128 = unsigned __int128;

__device__ __forceinline__ u128 pcg_mult() {
    return ((u128)0x2360ED051FC65DA4ull << 64) | 0x4385DF649FCCF645ull;
}
__device__ __forceinline__ u128 make128(unsigned long long hi, unsigned long long lo) { return ((u128)hi << 64) | lo; }

// state after `delta` steps of state -> state * mult + inc (mod 2^128): binary powering of
// the affine map (the LCG jump-ahead of Brown 1994)
__device__ u128 pcg_advance(u128 state, u128 inc, unsigned long long delta) {
    u128 acc_mult = 1, acc_plus = 0, cur_mult = pcg_mult(), cur_plus = inc;
    while (delta) {
        if (delta & 1) {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1) * cur_plus;
        cur_mult *= cur_mult;
        delta >>= 1;
    }
    return acc_mult * state + acc_plus;
}

// XSL-RR output of a state, as a double in [0, 1) (53 bits)
__device__ __forceinline__ double pcg_uniform(u128 state) {
    const unsigned long long hi = (unsigned long long)(state >> 64), lo = (unsigned long long)state;
    const unsigned long long x = hi ^ lo;
    const unsigned r = unsigned(hi >> 58);
    const unsigned long long out = (x >> r) | (x << ((64 - r) & 63));
    return double(out >> 11) * (1.0 / 9007199254740992.0);
}

__global__ void k_sf_flag(int ng, const int* __restrict__ gidx, const double* __restrict__ rho,
                          const double* __restrict__ u, double u_per_k, double rho_sf, int* __restrict__ flag) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const int i = gidx[g];
    flag[g] = (rho[g] > rho_sf && __ddiv_rn(u[i], u_per_k) < kTSfMax) ? 1 : 0;
}

__global__ void k_sf_decide(int ng, const int* __restrict__ gidx, const double* __restrict__ rho,
                            const int* __restrict__ flag, const int* __restrict__ rank, const Pcg64* __restrict__ rng,
                            double sf_eff, double dt, double t, int8_t* __restrict__ kind,
                            double* __restrict__ birth, int* __restrict__ fresh) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    fresh[g] = 0;
    if (!flag[g]) return;
    const Pcg64 R = *rng;
    const u128 st = pcg_advance(make128(R.w[0], R.w[1]), make128(R.w[2], R.w[3]),
                                (unsigned long long)rank[g] + 1);
    const double x = pcg_uniform(st);
    const double t_ff = sqrt(__ddiv_rn(3.0 * kPi, __dmul_rn(32.0, rho[g])));
    const double p = __dadd_rn(1.0, -exp(__ddiv_rn(__dmul_rn(-sf_eff, dt), t_ff)));
    if (x < p) {
        const int i = gidx[g];
        kind[i] = int8_t(kStar);
        birth[i] = t;
        fresh[g] = 1;
    }
}

__global__ void k_sf_advance(Pcg64* rng, const int* __restrict__ ndense) {
    Pcg64 R = *rng;
    const u128 st = pcg_advance(make128(R.w[0], R.w[1]), make128(R.w[2], R.w[3]), (unsigned long long)*ndense);
    R.w[0] = (unsigned long long)(st >> 64);
    R.w[1] = (unsigned long long)st;
    *rng = R;
}

__global__ void k_sf_list(int ng, const int* __restrict__ gidx, const int* __restrict__ fresh,
                          const int* __restrict__ pos_in_list, int* __restrict__ list) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < ng && fresh[g]) list[pos_in_list[g]] = gidx[g];
}

// (squared distance, index) pairs ordered lexicographically
__device__ __forceinline__ bool closer(double da, int ia, double db, int ib) {
    return da < db || (da == db && ia < ib);
}

// One block per new star: the K nearest current gas particles (float64 squared distances;
// ties by index), then their heating and bubble times. Each thread keeps its own sorted K best
// over a strided share of the particles; K rounds of a block-wide minimum over the threads'
// heads then give the K nearest in order.
template <int K>
__global__ void __launch_bounds__(kFbThreads) k_feedback(int n, int k, const int* __restrict__ stars,
                                                         const double* __restrict__ pos,
                                                         const double* __restrict__ mass,
                                                         const int8_t* __restrict__ kind, double* __restrict__ u,
                                                         double* __restrict__ no_cool, double t, StarParams P) {
    __shared__ double s_d[kFbThreads / 32];
    __shared__ int s_i[kFbThreads / 32];
    __shared__ int s_win[kFbMaxK];
    const int star = stars[blockIdx.x];
    const double sx = pos[3 * size_t(star)], sy = pos[3 * size_t(star) + 1], sz = pos[3 * size_t(star) + 2];
    double bd[K];
    int bi[K];
#pragma unroll
    for (int q = 0; q < K; ++q) {
        bd[q] = INFINITY;
        bi[q] = 0x7fffffff;
    }
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        if (kind[j] != kGas) continue;
        const double dx = pos[3 * size_t(j)] - sx, dy = pos[3 * size_t(j) + 1] - sy, dz = pos[3 * size_t(j) + 2] - sz;
        const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
        if (!closer(d2, j, bd[k - 1], bi[k - 1])) continue;
        // insertion into the sorted list (the last entry falls out)
        double cd = d2;
        int ci = j;
#pragma unroll
        for (int q = 0; q < K; ++q) {
            if (q < k && closer(cd, ci, bd[q], bi[q])) {
                const double td = bd[q];
                const int ti = bi[q];
                bd[q] = cd;
                bi[q] = ci;
                cd = td;
                ci = ti;
            }
        }
    }
    // K rounds: block-wide minimum of the threads' heads; the winner pops its head
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int r = 0; r < k; ++r) {
        double d = bd[0];
        int idx = bi[0];
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            const double od = __shfl_xor_sync(0xffffffffu, d, o);
            const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
            if (closer(od, oi, d, idx)) {
                d = od;
                idx = oi;
            }
        }
        if (lane == 0) {
            s_d[w] = d;
            s_i[w] = idx;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double bdm = s_d[0];
            int bim = s_i[0];
            for (int q = 1; q < kFbThreads / 32; ++q)
                if (closer(s_d[q], s_i[q], bdm, bim)) {
                    bdm = s_d[q];
                    bim = s_i[q];
                }
            s_win[r] = bim;
        }
        __syncthreads();
        if (bi[0] == s_win[r]) {  // pop (indices are unique)
#pragma unroll
            for (int q = 0; q < K - 1; ++q) {
                bd[q] = bd[q + 1];
                bi[q] = bi[q + 1];
            }
            bd[K - 1] = INFINITY;
            bi[K - 1] = 0x7fffffff;
        }
    }
    __syncthreads();
    // star_formation.py:60-65
    const double e_per_g = __ddiv_rn(__dmul_rn(P.fb_eff, P.e_sn_per_msun), P.msun_g);
    const double E = __dmul_rn(__dmul_rn(__dmul_rn(e_per_g, mass[star]), P.msun), P.msun_g);
    for (int r = threadIdx.x; r < k; r += blockDim.x) {
        const int tgt = s_win[r];
        if (tgt < 0 || tgt >= n) continue;  // fewer gas particles than k: cannot happen (k <= #gas)
        const double mg = __dmul_rn(__dmul_rn(mass[tgt], P.msun), P.msun_g);
        const double du = __ddiv_rn(__ddiv_rn(__ddiv_rn(E, double(k)), mg), P.u_cgs);
        atomicAdd(&u[tgt], du);
        no_cool[tgt] = __dadd_rn(t, P.fb_time);
    }
}

}  // namespace

int form_stars_and_feedback(int n, int ng, const int* gidx, const double* rho, const double* pos,
                            const double* mass, int8_t* kind, double* u, double* birth, double* no_cool,
                            double dt, double t, const StarParams& P, Pcg64* rng_dev, cudaStream_t s) {
    if (ng <= 0) return 0;
    static DevBuf flag, rank, fresh, fscan, list, counts;
    static int* h_counts = nullptr;
    if (!h_counts) GF_CUDA(cudaMallocHost(&h_counts, 2 * sizeof(int)));
    int* fl = flag.get<int>(ng);
    int* rk = rank.get<int>(ng);
    int* fr = fresh.get<int>(ng);
    int* fs = fscan.get<int>(ng);
    int* ls = list.get<int>(ng);
    int* cnt = counts.get<int>(2);
    const int grid = div_up(ng, kThreads);
    k_sf_flag<<<grid, kThreads, 0, s>>>(ng, gidx, rho, u, P.u_per_k, P.rho_sf, fl);
    GF_CHECK_LAUNCH();
    exclusive_scan(fl, rk, ng, &cnt[0], s);
    k_sf_decide<<<grid, kThreads, 0, s>>>(ng, gidx, rho, fl, rk, rng_dev, P.sf_eff, dt, t, kind, birth, fr);
    GF_CHECK_LAUNCH();
    k_sf_advance<<<1, 1, 0, s>>>(rng_dev, &cnt[0]);
    GF_CHECK_LAUNCH();
    exclusive_scan(fr, fs, ng, &cnt[1], s);
    k_sf_list<<<grid, kThreads, 0, s>>>(ng, gidx, fr, fs, ls);
    GF_CHECK_LAUNCH();
    GF_CUDA(cudaMemcpyAsync(h_counts, cnt, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    GF_CUDA(cudaStreamSynchronize(s));
    const int nnew = h_counts[1];
    // supernova_feedback (star_formation.py:50-65)
    const int ngas = ng - nnew;  // the gas of the last SPH evaluation that stayed gas
    if (nnew == 0 || P.fb_eff <= 0 || ngas < 10) return nnew;
    const int k = std::min(int(P.fb_ngb), ngas);
    if (k > kFbMaxK) throw Error(GF_ERR_ARG, "fb_ngb above 64 is not supported");
    if (k <= 16)
        k_feedback<16><<<nnew, kFbThreads, 0, s>>>(n, k, ls, pos, mass, kind, u, no_cool, t, P);
    else if (k <= 32)
        k_feedback<32><<<nnew, kFbThreads, 0, s>>>(n, k, ls, pos, mass, kind, u, no_cool, t, P);
    else
        k_feedback<64><<<nnew, kFbThreads, 0, s>>>(n, k, ls, pos, mass, kind, u, no_cool, t, P);
    GF_CHECK_LAUNCH();
    return nnew;
}

}  // namespace gf
