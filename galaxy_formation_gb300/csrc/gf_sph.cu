// gf_sph.cu — SPH on the GPU (galaxy_formation/sph.py).
//
//   kernel / kernel_grad ..... sph.py:31-54, float64
//   sph_forces ............... sph.py:57-106: density pass, then an equation-of-state pass
//                              (P/rho^2 and sound speed per particle), then the force pass
//                              (pressure, Monaghan-Gingold viscosity on approaching pairs,
//                              du/dt, Courant step); one thread per particle, float64.
//   knn_from_candidates ...... sph.py:109-135: one warp per particle, float64 distances,
//                              bitonic sort of the (<= 64) candidates in shared memory.
//   exact k nearest .......... replaces cKDTree(p).query(p, k) (sph.py:165-166):
//                              octree of the points (same builder as gravity); one warp per
//                              two consecutive queries walks it with a radius per query,
//                              collecting the points within each radius (float32 distances
//                              from hi/lo split coordinates) until the count lies in
//                              [k, 128] — the radius iteration, Newton steps on
//                              count ~ R^3 from a guess (2.5 x the previous h, 1.06 x the
//                              learned guess of the k-th-neighbour distance, or the leaf's
//                              cell density). The collected points are sorted,
//                              the k nearest plus near-ties at the boundary are re-measured
//                              in float64 and sorted again, so the result is the exact
//                              float64 kNN.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <string>

#include "gf_mlp.cuh"
#include "gf_sph.cuh"
#include "gf_tree.cuh"

namespace gf {

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr int kThreads = 256;

// sph.py:31-40
__device__ __forceinline__ double w_m4(double r, double h) {
    const double q = r / h;
    const double s = 1.0 / (kPi * h * h * h);
    if (q < 1.0) return s * (1 - 1.5 * q * q + 0.75 * q * q * q);
    if (q < 2.0) {
        const double t = 2 - q;
        return s * 0.25 * t * t * t;
    }
    return 0.0;
}

// sph.py:43-54
__device__ __forceinline__ double dw_m4(double r, double h) {
    const double q = r / h;
    const double s = 1.0 / (kPi * h * h * h * h);
    double g;
    if (q < 1.0) {
        g = s * (-3 * q + 2.25 * q * q);
    } else if (q < 2.0) {
        const double t = 2 - q;
        g = -s * 0.75 * t * t;
    } else {
        return 0.0;
    }
    return g / fmax(r, 1e-30);
}

__global__ void k_sph_kernel(int n, const double* __restrict__ r, const double* __restrict__ h,
                             double* __restrict__ w, double* __restrict__ dw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (w) w[i] = w_m4(r[i], h[i]);
    if (dw) dw[i] = dw_m4(r[i], h[i]);
}

// A neighbour row from the caller may hold an index outside [0, n): such a particle gets NaN
// outputs and GF_ERR_ARG is raised (status may be null), instead of a read out of bounds.
template <class Idx>
__device__ __forceinline__ bool row_in_range(const Idx* __restrict__ row, int k, int n, uint32_t* status) {
    bool ok = true;
    for (int jj = 0; jj < k; ++jj) {
        const int64_t j = row[jj];
        ok &= j >= 0 && j < n;
    }
    if (!ok) raise_status(status, GF_ERR_ARG);
    return ok;
}

// pass 1 (sph.py:63-71): rho_i = sum_j m_j W(r_ij, h_i), the particle itself included
template <class Idx>
__global__ void k_sph_density(int n, int k, int ld, const double* __restrict__ pos, const double* __restrict__ mass,
                              const Idx* __restrict__ nb, const double* __restrict__ h,
                              double* __restrict__ rho, Subset sub, uint32_t* status) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (!subset_item(sub, i, n, nullptr, i)) return;
    if (!row_in_range(nb + size_t(i) * ld, k, n, status)) {
        rho[i] = __longlong_as_double(0x7ff8000000000000ll);
        return;
    }
    const double xi = pos[3 * size_t(i)], yi = pos[3 * size_t(i) + 1], zi = pos[3 * size_t(i) + 2];
    const double hi = h[i];
    double s = 0.0;
    for (int jj = 0; jj < k; ++jj) {
        const int64_t j = nb[size_t(i) * ld + jj];
        const double dx = xi - pos[3 * j], dy = yi - pos[3 * j + 1], dz = zi - pos[3 * j + 2];
        s += mass[j] * w_m4(sqrt(dx * dx + dy * dy + dz * dz), hi);
    }
    rho[i] = s;
}

// P / rho^2 and the sound speed of every particle (the per-j factors of sph.py:88-89)
__global__ void k_sph_eos(int n, const double* __restrict__ rho, const double* __restrict__ u,
                          double gamma, double* __restrict__ pr2, double* __restrict__ cs, Subset sub) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (!subset_item(sub, i, n, nullptr, i)) return;
    const double P = (gamma - 1) * rho[i] * u[i];
    pr2[i] = P / (rho[i] * rho[i]);
    cs[i] = sqrt(gamma * (gamma - 1) * u[i]);
}

// (1/r) dW/dr of sph.py:43-54 with the per-particle factors 1/h and 1/(pi h^4) precomputed
// and 1/r shared by both smoothing lengths of a pair (one float64 division per pair).
__device__ __forceinline__ double dw_m4_pre(double r, double inv_r, double inv_h, double s4) {
    const double q = r * inv_h;
    double g;
    if (q < 1.0) {
        g = s4 * (-3 * q + 2.25 * q * q);
    } else if (q < 2.0) {
        const double t = 2 - q;
        g = -s4 * 0.75 * t * t;
    } else {
        return 0.0;
    }
    return g * inv_r;
}

// pass 2 (sph.py:72-106)
template <class Idx>
__global__ void k_sph_force(int n, int k, int ld, const double* __restrict__ pos, const double* __restrict__ vel,
                            const double* __restrict__ mass, const Idx* __restrict__ nb,
                            const double* __restrict__ h, const double* __restrict__ rho,
                            const double* __restrict__ pr2, const double* __restrict__ cs, double alpha,
                            double beta, double* __restrict__ acc, double* __restrict__ dudt,
                            double* __restrict__ dt_i, float* __restrict__ divv, Subset sub, uint32_t* status) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (!subset_item(sub, i, n, nullptr, i)) return;
    if (!row_in_range(nb + size_t(i) * ld, k, n, status)) {
        const double nan = __longlong_as_double(0x7ff8000000000000ll);
        acc[3 * size_t(i)] = acc[3 * size_t(i) + 1] = acc[3 * size_t(i) + 2] = nan;
        dudt[i] = dt_i[i] = nan;
        if (divv) divv[i] = __int_as_float(0x7fc00000);
        return;
    }
    const double xi = pos[3 * size_t(i)], yi = pos[3 * size_t(i) + 1], zi = pos[3 * size_t(i) + 2];
    const double vxi = vel[3 * size_t(i)], vyi = vel[3 * size_t(i) + 1], vzi = vel[3 * size_t(i) + 2];
    const double hi = h[i], rhoi = rho[i], pri = pr2[i], ci = cs[i];
    const double inv_hi = 1.0 / hi, s4i = 1.0 / (kPi * hi * hi * hi * hi);
    double ax = 0, ay = 0, az = 0, du = 0, mu_max = 0, dv = 0;
    for (int jj = 0; jj < k; ++jj) {
        const int64_t j = nb[size_t(i) * ld + jj];
        if (j == i) continue;
        const double dx = xi - pos[3 * j], dy = yi - pos[3 * j + 1], dz = zi - pos[3 * j + 2];
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        const double hj = h[j];
        const double inv_r = 1.0 / fmax(r, 1e-30);
        const double gi = dw_m4_pre(r, inv_r, inv_hi, s4i);
        const double inv_hj = 1.0 / hj, ih2 = inv_hj * inv_hj;
        const double gj = dw_m4_pre(r, inv_r, inv_hj, ih2 * ih2 * (1.0 / kPi));
        const double vr = (vxi - vel[3 * j]) * dx + (vyi - vel[3 * j + 1]) * dy + (vzi - vel[3 * j + 2]) * dz;
        double visc = 0.0;
        if (vr < 0) {
            const double hb = 0.5 * (hi + hj);
            const double mu = hb * vr / (r * r + 0.01 * hb * hb);
            mu_max = fmax(mu_max, -mu);
            visc = (-alpha * 0.5 * (ci + cs[j]) * mu + beta * mu * mu) / (0.5 * (rhoi + rho[j]));
        }
        const double gb = 0.5 * (gi + gj);
        const double f = pri * gi + pr2[j] * gj + visc * gb;
        const double mj = mass[j];
        ax -= mj * f * dx;
        ay -= mj * f * dy;
        az -= mj * f * dz;
        du += mj * (pri * gi + 0.5 * visc * gb) * vr;
        dv += mj * vr * gi;
    }
    acc[3 * size_t(i)] = ax;
    acc[3 * size_t(i) + 1] = ay;
    acc[3 * size_t(i) + 2] = az;
    dudt[i] = du;
    dt_i[i] = 0.3 * hi / (ci + 1.2 * (alpha * ci + beta * mu_max) + 1e-30);
    if (divv) divv[i] = float(-dv / rhoi);  // SPH velocity divergence (a feature of the h guess)
}

// ------------------------------------------------------------------- warp bitonic sorts

// --------------------------------------------------------------- knn_from_candidates

constexpr int kCandWarps = 8;

__global__ void __launch_bounds__(kCandWarps * 32) k_knn_cand(
    int n, int m, const double* __restrict__ pos, const int64_t* __restrict__ cand, int k,
    int64_t* __restrict__ nb, double* __restrict__ dist, int* __restrict__ all_ok) {
    __shared__ unsigned long long s_key[kCandWarps][64];
    __shared__ int s_tag[kCandWarps][64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned long long* key = s_key[w];
    int* tag = s_tag[w];
    const int nwarps = gridDim.x * kCandWarps;
    for (int i = blockIdx.x * kCandWarps + w; i < n; i += nwarps) {
        const double xi = pos[3 * size_t(i)], yi = pos[3 * size_t(i) + 1], zi = pos[3 * size_t(i) + 2];
        int valid = 0;
        for (int jj = lane; jj < 64; jj += 32) {
            double d2 = INFINITY;
            if (jj < m) {
                const int64_t j = cand[size_t(i) * m + jj];
                if (j >= 0) {
                    const double dx = xi - pos[3 * j], dy = yi - pos[3 * j + 1], dz = zi - pos[3 * j + 2];
                    d2 = dx * dx + dy * dy + dz * dz;
                    ++valid;
                }
            }
            key[jj] = (unsigned long long)__double_as_longlong(d2);
            tag[jj] = jj;
        }
        valid = warp_sum(valid);
        __syncwarp();
        if (valid < k) {  // sph.py:128-130: not enough candidates, row untouched
            if (lane == 0) *all_ok = 0;
            continue;
        }
        warp_bitonic(key, tag, 64);
        for (int t = lane; t < k; t += 32) {
            nb[size_t(i) * k + t] = cand[size_t(i) * m + tag[t]];
            dist[size_t(i) * k + t] = sqrt(__longlong_as_double((long long)key[t]));
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------------ exact kNN

constexpr int kKnnWarps = 8;
// Leaf capacity of the neighbour-search tree. The search is exact for any tree; 16 walks
// fewer levels per query (7 % faster on the 1M disk) but its coarser leaf counts make the
// learned guess's features less informative, so the reference's 8 is kept.
constexpr int kKnnLeaf = kLeafMax;
constexpr int kKnnStack = 512;
constexpr int kKnnCap = 128;

// A collected point: (float32 squared distance bits << 32) | tree position. The bits of a
// non-negative float order like the float, so sorting the keys orders by distance, then index.
__device__ __forceinline__ unsigned long long knn_key(float d2, int j) {
    return ((unsigned long long)__float_as_uint(d2) << 32) | unsigned(j);
}
__device__ __forceinline__ float key_d2(unsigned long long k) { return __uint_as_float(unsigned(k >> 32)); }
__device__ __forceinline__ int key_idx(unsigned long long k) { return int(unsigned(k)); }

struct KnnSmem {
    int stack[kKnnStack];
    unsigned long long key[2][kKnnCap];  // the collected points of the warp's two queries
    unsigned long long dd[64];  // float64 squared distances as bit patterns
    int di[64];
};

// A query of a neighbour walk: position (hi/lo), radius; `on` (warp-uniform) false for a slot
// without a query or one already settled.
struct KnnQuery {
    float4 xh, xl;
    float R, R2;
    bool on;
};

struct KnnArgs {
    int n, k, nn;
    const float4* wb;
    const float4* wgeo;
    const float4* p4;
    const float4* plo;
    const int* perm;
    const int* leaf_of;
    const double* pos;      // caller order
    const float* r_guess;   // caller order, optional
    int64_t* nb;            // (n, k) caller order, or null
    double* dist;           // (n, k), or null
    int* nb32;              // (n, ld32) caller order, or null
    int ld32;
    double* dsel;           // distance of neighbour `dsel_col` (n,), or null
    int dsel_col;
    int* dsel_idx;          // instead of dsel (float32 order): that neighbour's caller index, whose
                            // float64 distance the caller measures a thread per query (-1: failed)
    float* dfar;            // distance of the k-th nearest in float32 (n,), or null
    uint32_t* status;
    unsigned long long* iters;
    const int* wparent;     // breadth-first parent of each node (-1 for the root)
    int exact_order;        // 1: float64 re-sort of the k nearest; 0: float32 order, float64
                            //    only to settle the neighbour at dsel_col (the h boundary)
};

// Collects, for each of the warp's (up to) two queries that is on, the points within its radius
// into S.key[i] (the first kKnnCap of them) and their number into cnt[i]; one walk serves both:
// a node is opened when it meets either sphere, and each point of an opened leaf is tested
// against both. Returns false on stack overflow. The two queries of a warp are neighbours in
// the tree's order (usually in one leaf), so their walks share most nodes.
__device__ bool knn_collect(const KnnArgs& A, KnnSmem& S, const KnnQuery (&Q)[2], int leaf, int (&cnt)[2]) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = lanemask_lt();
    // start at the smallest ancestor of the leaf whose cube contains every sphere that is on
    // (every point within a radius then lies in that subtree)
    int start = leaf;
    for (int up = 0; start > 0 && up < 64; ++up) {
        const float4 g = A.wgeo[start];
        const float pad = 2e-6f * (fabsf(g.x) + fabsf(g.y) + fabsf(g.z) + g.w) + 1e-30f;
        bool inside = true;
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            if (!Q[i].on) continue;
            const float lim = g.w - Q[i].R - pad;
            inside = inside && fabsf((Q[i].xh.x - g.x) + Q[i].xl.x) <= lim &&
                     fabsf((Q[i].xh.y - g.y) + Q[i].xl.y) <= lim && fabsf((Q[i].xh.z - g.z) + Q[i].xl.z) <= lim;
        }
        if (inside) break;
        start = A.wparent[start];
    }
    if (start < 0) start = 0;
    cnt[0] = cnt[1] = 0;
    int sp = 1;
    if (lane == 0) S.stack[0] = (start << 4) | 1;
    __syncwarp();
    for (int rounds = 0; sp > 0; ++rounds) {
        if (rounds > A.nn) return false;  // each node is popped at most once
        // pop up to 64 nodes (two per lane: their loads overlap)
        int node[2];
        const int nnodes = pop_round<2>(S.stack, sp, node);
        float4 G[2], B[2];
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            if (node[j] >= 0) {
                G[j] = A.wgeo[node[j]];
                B[j] = A.wb[node[j]];
            }
        }
        int first[2] = {0, 0}, lcs[2] = {0, 0};
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            if (32 * j >= nnodes) break;  // warp-uniform
            bool open = false;
            int code = 0;
            if (node[j] >= 0) {
                const float4 g = G[j];
                first[j] = __float_as_int(B[j].y);
                code = __float_as_int(B[j].z);
                // distance from each query to the cell cube, padded for float32 rounding
                const float lim = g.w + 2e-6f * (fabsf(g.x) + fabsf(g.y) + fabsf(g.z) + g.w) + 1e-30f;
#pragma unroll
                for (int i = 0; i < 2; ++i) {
                    if (!Q[i].on) continue;
                    const float ex = fmaxf(fabsf((g.x - Q[i].xh.x) - Q[i].xl.x) - lim, 0.f);
                    const float ey = fmaxf(fabsf((g.y - Q[i].xh.y) - Q[i].xl.y) - lim, 0.f);
                    const float ez = fmaxf(fabsf((g.z - Q[i].xh.z) - Q[i].xl.z) - lim, 0.f);
                    open = open || ex * ex + ey * ey + ez * ez <= Q[i].R2;
                }
            }
            const bool inner = open && code > 0;
            const unsigned om = __ballot_sync(0xffffffffu, inner);
            const int npush = __popc(om);
            if (sp + npush > kKnnStack) return false;
            if (inner) S.stack[sp + __popc(om & lt)] = (first[j] << 4) | code;
            sp += npush;
            lcs[j] = open && code < 0 ? -code : 0;
        }
        // particles of the opened leaves, concatenated in lane order (a lane's two leaves in
        // turn) and tested 32 at a time: lane l takes offset o = base + l
        const int lc = lcs[0] + lcs[1];
        if (__any_sync(0xffffffffu, lc > 0)) {  // some leaf opened in this round
        const int lincl = warp_incl_scan(lc);
        const int lexcl = lincl - lc;
        const int ltot = __shfl_sync(0xffffffffu, lincl, 31);
        for (int base = 0; base < ltot; base += 32) {
            const int o = base + lane;
            int src = 0;  // lanes whose inclusive end is <= o (branch-free lower bound)
#pragma unroll
            for (int step = 16; step; step >>= 1) {
                const int v = __shfl_sync(0xffffffffu, lincl, src + step - 1);
                if (v <= o) src += step;
            }
            src = min(src, 31);
            const int f0 = __shfl_sync(0xffffffffu, first[0], src);
            const int f1 = __shfl_sync(0xffffffffu, first[1], src);
            const int l0 = __shfl_sync(0xffffffffu, lcs[0], src);
            const int e_src = __shfl_sync(0xffffffffu, lexcl, src);
            float4 ph = make_float4(0.f, 0.f, 0.f, 0.f), pl = ph;
            int j = 0;
            if (o < ltot) {
                const int off = o - e_src;
                j = off < l0 ? f0 + off : f1 + (off - l0);
                ph = A.p4[j];
                pl = A.plo[j];
            }
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                if (!Q[i].on) continue;
                const float dx = (ph.x - Q[i].xh.x) + (pl.x - Q[i].xl.x);
                const float dy = (ph.y - Q[i].xh.y) + (pl.y - Q[i].xl.y);
                const float dz = (ph.z - Q[i].xh.z) + (pl.z - Q[i].xl.z);
                const float d2 = dx * dx + dy * dy + dz * dz;
                const bool hit = o < ltot && d2 <= Q[i].R2;
                const unsigned hm = __ballot_sync(0xffffffffu, hit);
                if (hit) {
                    const int slot = cnt[i] + __popc(hm & lt);
                    if (slot < kKnnCap) S.key[i][slot] = knn_key(d2, j);
                }
                cnt[i] += __popc(hm);
            }
        }
        }  // any leaf
        __syncwarp();
    }
    return true;
}

// Sorts the cnt (<= kKnnCap) collected points of query q (tree position), re-measures the
// k nearest and the float32 near-ties in float64 and writes the k nearest (ascending, ties by
// index) in the caller's order.
__device__ __forceinline__ double d2_f64(const KnnArgs& A, int pi, int pj) {
    const double dx = A.pos[3 * size_t(pi)] - A.pos[3 * size_t(pj)];
    const double dy = A.pos[3 * size_t(pi) + 1] - A.pos[3 * size_t(pj) + 1];
    const double dz = A.pos[3 * size_t(pi) + 2] - A.pos[3 * size_t(pj) + 2];
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

__device__ void knn_finish(const KnnArgs& A, unsigned long long* key, unsigned long long* dd, int* di, int cnt,
                           int q) {
    const int lane = threadIdx.x & 31;
    const int k = A.k;
    const int oq = A.perm[q];
    int P = 64;
    while (P < cnt) P <<= 1;
    for (int t = cnt + lane; t < P; t += 32) key[t] = ~0ull;
    __syncwarp();
    warp_sort_u64(key, P);
    const int pi = oq;
    if (!A.exact_order) {
        // Float32 order: the k nearest as a set (only pairs tied to float32 rounding can
        // swap). The neighbour at dsel_col fixes h: the entries within float32 rounding of
        // it are re-measured in float64 and the dsel_col-th smallest is taken.
        const int c = A.dsel_col;
        const float dc = key_d2(key[c]);
        const float lo = dc * (1.0f - 2e-5f), hi = dc * (1.0f + 2e-5f);
        int below = 0, inband = 0;
        for (int t = lane; t < cnt; t += 32) {
            const float v = key_d2(key[t]);
            below += v < lo;
            inband += v >= lo && v <= hi;
        }
        below = warp_sum(below);
        inband = warp_sum(inband);
        double best = 0.0;
        int selc = -1;  // caller index of the entry that fixes h
        if (inband == 1) {  // no float32 near-tie: entry c itself, measured in float64
            selc = A.perm[key_idx(key[c])];
            if (!A.dsel_idx) best = d2_f64(A, pi, selc);
        } else {
            const int rank_need = c - below;  // rank of the wanted entry among the ambiguous ones
            for (int t = lane; t < 64; t += 32) {
                double v = INFINITY;
                int tag = 0x7fffffff;
                const float vf = t < cnt ? key_d2(key[t]) : INFINITY;
                if (t < cnt && vf >= lo && vf <= hi) {
                    const int j = key_idx(key[t]);
                    v = d2_f64(A, pi, A.perm[j]);
                    tag = j;
                }
                dd[t] = (unsigned long long)__double_as_longlong(v);
                di[t] = tag;
            }
            __syncwarp();
            warp_bitonic(dd, di, 64);
            best = __longlong_as_double((long long)dd[max(0, rank_need)]);
            selc = A.perm[di[max(0, rank_need)]];
            // the tied entries [below, below + inband) take the float64 order (ties by tree
            // position), so the first c + 1 entries are the exact set the smoothing length is
            // measured on; their float32 distance bits stay (all within the band)
            if (below + inband <= 64)
                for (int t = lane; t < inband; t += 32)
                    key[below + t] = (key[below + t] & 0xffffffff00000000ull) | unsigned(di[t]);
            __syncwarp();
        }
        for (int t = lane; t < k; t += 32) {
            const int pj = A.perm[key_idx(key[t])];
            if (A.nb32) A.nb32[size_t(oq) * A.ld32 + t] = pj;
            if (A.nb) A.nb[size_t(oq) * k + t] = pj;
        }
        if (A.dsel_idx) {
            if (lane == 0) A.dsel_idx[oq] = selc;
        } else if (A.dsel && lane == 0) {
            A.dsel[oq] = __dsqrt_rn(best);
        }
        if (A.dfar && lane == 0) A.dfar[oq] = sqrtf(key_d2(key[k - 1]));
        __syncwarp();
        return;
    }
    // the k nearest and everything within float32 rounding of the k-th distance
    const float thr = key_d2(key[k - 1]) * (1.0f + 2e-5f);
    int m = 0;
    for (int t = lane; t < cnt; t += 32) m += key_d2(key[t]) <= thr;
    m = min(64, warp_sum(m));
    for (int t = lane; t < 64; t += 32) {
        double v = INFINITY;
        int tag = 0x7fffffff;
        if (t < m) {
            const int pj = A.perm[key_idx(key[t])];
            v = d2_f64(A, pi, pj);
            tag = pj;
        }
        dd[t] = (unsigned long long)__double_as_longlong(v);
        di[t] = tag;
    }
    __syncwarp();
    warp_bitonic(dd, di, 64);
    for (int t = lane; t < k; t += 32) {
        const double dt = __longlong_as_double((long long)dd[t]);
        if (A.nb) A.nb[size_t(oq) * k + t] = di[t];
        if (A.dist) A.dist[size_t(oq) * k + t] = __dsqrt_rn(dt);
        if (A.nb32) A.nb32[size_t(oq) * A.ld32 + t] = di[t];
        if (A.dsel && t == A.dsel_col) A.dsel[oq] = __dsqrt_rn(dt);
        if (A.dfar && t == k - 1) A.dfar[oq] = sqrtf(float(dt));
    }
    __syncwarp();
}

__device__ void knn_fail_output(const KnnArgs& A, int q, bool stack) {
    const int lane = threadIdx.x & 31;
    const int oq = A.perm[q];
    if (lane == 0) raise_status(A.status, stack ? GF_ERR_WALK_STACK : GF_ERR_KNN);
    for (int t = lane; t < A.k; t += 32) {
        if (A.nb) A.nb[size_t(oq) * A.k + t] = -1;
        if (A.dist) A.dist[size_t(oq) * A.k + t] = INFINITY;
        if (A.nb32) A.nb32[size_t(oq) * A.ld32 + t] = -1;
    }
    if (A.dsel && lane == 0) A.dsel[oq] = INFINITY;
    if (A.dsel_idx && lane == 0) A.dsel_idx[oq] = -1;
}

// Radius step of the count-to-k iteration: Newton on count ~ R^3 until the count is
// bracketed by [lo, hi], bisection afterwards.
__device__ __forceinline__ float knn_next_radius(float R, int cnt, int k, int cap, float& lo, float& hi) {
    float next;
    if (cnt < k) {
        lo = R;
        next = R * (cnt >= 4 ? cbrtf(1.3f * float(k) / float(cnt)) : 2.0f);
    } else {
        hi = R;
        next = R * cbrtf(0.75f * float(cap) / float(cnt));
    }
    if (lo > 0.f && hi < INFINITY) next = 0.5f * (lo + hi);
    return next;
}

// One warp per pair of consecutive queries (tree order): walk from the smallest ancestor cell
// containing both search spheres, collecting for both at once; each query iterates its radius
// on its own, and a query still searching after the other has settled walks alone. Four blocks
// of 8 warps per SM (64 registers): 15 % faster than with the 80 registers the compiler takes
// unbounded (3 blocks), and 15 % faster than one query per warp.
__global__ void __launch_bounds__(kKnnWarps * 32, 4) k_knn(KnnArgs A) {
    __shared__ KnnSmem smem_all[kKnnWarps];
    KnnSmem& S = smem_all[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int k = A.k;
    const int cap = kKnnCap;  // count window [k, cap]
    const int nwarps = gridDim.x * kKnnWarps;
    for (int q0 = 2 * (blockIdx.x * kKnnWarps + (threadIdx.x >> 5)); q0 < A.n; q0 += 2 * nwarps) {
        KnnQuery Q[2];
        float lo[2], hi[2];
        int it[2] = {0, 0};
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int q = q0 + i;
            Q[i].on = q < A.n;
            lo[i] = 0.f;
            hi[i] = INFINITY;
            if (!Q[i].on) continue;
            Q[i].xh = A.p4[q];
            Q[i].xl = A.plo[q];
            float R;
            if (A.r_guess) {
                R = A.r_guess[A.perm[q]];
            } else {  // from the density of the particle's leaf cell
                const int lf = A.leaf_of[q];
                const float half = A.wgeo[lf].w;
                const int c = max(1, -__float_as_int(A.wb[lf].z));
                R = 2.0f * half * cbrtf(float(k) / float(c));
            }
            if (!(R > 0.f) || !isfinite(R)) R = 1e-3f;
            Q[i].R = R;
            Q[i].R2 = R * R;
        }
        while (Q[0].on || Q[1].on) {
            int cnt[2];
            const int leaf = A.leaf_of[Q[0].on ? q0 : q0 + 1];
            const bool ok_walk = knn_collect(A, S, Q, leaf, cnt);
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                if (!Q[i].on) continue;
                ++it[i];
                if (!ok_walk) {
                    knn_fail_output(A, q0 + i, true);
                    Q[i].on = false;
                } else if (cnt[i] >= k && cnt[i] <= cap) {
                    knn_finish(A, S.key[i], S.dd, S.di, cnt[i], q0 + i);
                    Q[i].on = false;
                } else if (it[i] >= 48) {
                    knn_fail_output(A, q0 + i, false);
                    Q[i].on = false;
                } else {
                    Q[i].R = knn_next_radius(Q[i].R, cnt[i], k, cap, lo[i], hi[i]);
                    Q[i].R2 = Q[i].R * Q[i].R;
                }
            }
        }
        if (lane == 0 && A.iters) atomicAdd(A.iters, (unsigned long long)(it[0] + it[1]));
    }
}

}  // namespace

// ------------------------------------------------------------------------------- host

void sph_kernel_values(int n, const double* r, const double* h, double* w, double* dw, cudaStream_t s) {
    if (n <= 0) return;
    k_sph_kernel<<<div_up(n, kThreads), kThreads, 0, s>>>(n, r, h, w, dw);
    GF_CHECK_LAUNCH();
}

template <class Idx>
void sph_forces(SphScratch& S, int n, int k, int ld, const double* pos, const double* vel, const double* mass,
                const Idx* nb, const double* h, const double* u, double gamma, double alpha,
                double beta, double* rho, double* acc, double* dudt, double* dt_i, cudaStream_t s, float* divv,
                Subset sub) {
    if (n <= 0) return;
    const int grid = div_up(n, kThreads);
    {
        ProfScope ps(kStSphDensity, s);
        k_sph_density<Idx><<<grid, kThreads, 0, s>>>(n, k, ld, pos, mass, nb, h, rho, sub, ctx().d_status);
        GF_CHECK_LAUNCH();
    }
    double* pr2 = S.pr2.get<double>(n);
    double* cs = S.cs.get<double>(n);
    k_sph_eos<<<grid, kThreads, 0, s>>>(n, rho, u, gamma, pr2, cs, sub);
    GF_CHECK_LAUNCH();
    ProfScope ps(kStSphForce, s);
    k_sph_force<Idx><<<grid, kThreads, 0, s>>>(n, k, ld, pos, vel, mass, nb, h, rho, pr2, cs, alpha, beta,
                                               acc, dudt, dt_i, divv, sub, ctx().d_status);
    GF_CHECK_LAUNCH();
}
template void sph_forces<int64_t>(SphScratch&, int, int, int, const double*, const double*, const double*,
                                  const int64_t*, const double*, const double*, double, double, double,
                                  double*, double*, double*, double*, cudaStream_t, float*, Subset);
template void sph_forces<int>(SphScratch&, int, int, int, const double*, const double*, const double*,
                              const int*, const double*, const double*, double, double, double,
                              double*, double*, double*, double*, cudaStream_t, float*, Subset);

void knn_from_candidates(int n, int m, const double* pos, const int64_t* cand, int k, int64_t* nb,
                         double* dist, int* d_ok, cudaStream_t s) {
    if (n <= 0) return;
    const int blocks = std::min(div_up(n, kCandWarps), 8 * ctx().sms);
    k_knn_cand<<<blocks, kCandWarps * 32, 0, s>>>(n, m, pos, cand, k, nb, dist, d_ok);
    GF_CHECK_LAUNCH();
}

// Features of the smoothing-length guess, per gas particle (caller order):
// (log cell density of its leaf, log previous h, leaf count, previous velocity divergence).
// Features of the learned guess: log cell density, log previous h, leaf count, velocity
// divergence. A particle without a previous h (the first search of a particle set) gets, in
// its place, the h that its cell density implies (the search radius of the cell-density start
// over 2.5: a function of the first feature, cold_log_h) and a divergence of 0.
__global__ void k_hfeatures(int n, int k, const int* __restrict__ perm, const int* __restrict__ leaf_of,
                            const float4* __restrict__ wb, const float4* __restrict__ wgeo, const int* __restrict__ gidx,
                            const double* __restrict__ hprev, const float* __restrict__ divv, float* __restrict__ X) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int i = perm[q];
    const int lf = leaf_of[q];
    const float c = float(max(1, -__float_as_int(wb[lf].z)));
    const float side = 2.f * wgeo[lf].w;
    const int g = gidx ? gidx[i] : i;
    const double hp = hprev ? hprev[g] : 0.0;
    const float f0 = logf(c / fmaxf(side * side * side, 1e-30f));
    X[4 * size_t(i) + 0] = f0;
    X[4 * size_t(i) + 1] = hp > 0 ? float(log(hp)) : cold_log_h(f0, k);
    X[4 * size_t(i) + 2] = c;
    X[4 * size_t(i) + 3] = hp > 0 && divv ? divv[g] : 0.f;
}

// The learned guess predicts the log distance of the k-th nearest; the search starts a little
// outside it, so that nearly every first sphere holds the k nearest and rarely more than 64
// points (one sort of 64 keys instead of 128).
constexpr float kFarMargin = 1.06f;

__global__ void k_guess_from_logdk(int n, const float* __restrict__ Y, float* __restrict__ rg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) rg[i] = kFarMargin * expf(Y[i]);
}

void knn_exact(Octree& T, int n, const double* pos, int k, const float* r_guess, int64_t* nb,
               double* dist, unsigned long long* d_iters, cudaStream_t s, int* nb32, int ld32,
               double* dsel, int dsel_col, const HGuess* hg, bool same_set, int* dsel_idx) {
    if (n <= 0) return;
    // same_set (the caller's point set drifted since the last search): the synchronisation-free
    // rebuild inside the node buffers of the last regular build (no host round trip in the middle
    // of the hydro chain), unless the last tree came close to filling them
    const bool same = same_set && T.valid && T.n == n && T.want_knn && T.leaf_max == kKnnLeaf && !T.outgrowing();
    T.want_knn = true;
    T.leaf_max = kKnnLeaf;
    if (same) {
        T.reserve_graph_build();
        T.build(n, pos, nullptr, 0.7, s, true);
    } else {
        T.build(n, pos, nullptr, 0.7, s);
    }
    if (hg && hg->X) {  // features for the learned guess (and for training pairs)
        k_hfeatures<<<div_up(n, kThreads), kThreads, 0, s>>>(n, k, T.perm.as<int>(), T.leaf_of.as<int>(),
                                                             T.w_b.as<float4>(), T.w_geo.as<float4>(), hg->gidx,
                                                             hg->hprev, hg->divv, hg->X);
        GF_CHECK_LAUNCH();
        if (hg->use_mlp) {
            mlp().predict(n, hg->X, hg->Y, s);
            k_guess_from_logdk<<<div_up(n, kThreads), kThreads, 0, s>>>(n, hg->Y, hg->rg);
            GF_CHECK_LAUNCH();
            r_guess = hg->rg;
        }
    }
    KnnArgs A{};
    A.n = n;
    A.k = k;
    A.nn = std::max(T.nn, T.node_cap);  // bounds the walk rounds (the live count is on the device)
    A.wb = T.w_b.as<float4>();
    A.wgeo = T.w_geo.as<float4>();
    A.p4 = T.p4.as<float4>();
    A.plo = T.plo.as<float4>();
    A.perm = T.perm.as<int>();
    A.leaf_of = T.leaf_of.as<int>();
    A.pos = pos;
    A.r_guess = r_guess;
    A.nb = nb;
    A.dist = dist;
    A.nb32 = nb32;
    A.ld32 = ld32;
    A.dsel = dsel;
    A.dsel_col = dsel_col;
    A.dsel_idx = dsel_col >= 0 ? dsel_idx : nullptr;
    A.dfar = hg ? hg->dk : nullptr;
    A.exact_order = (nb != nullptr || dist != nullptr || dsel_col < 0) ? 1 : 0;
    A.status = ctx().d_status;
    A.iters = d_iters;
    A.wparent = T.w_parent.as<int>();
    ProfScope ps(kStKnn, s);
    const int blocks = std::min(div_up(n, 2 * kKnnWarps), 16 * ctx().sms);  // two queries per warp
    k_knn<<<blocks, kKnnWarps * 32, 0, s>>>(A);
    GF_CHECK_LAUNCH();
}

}  // namespace gf

// ---------------------------------------------------------------------------------------
// sph_forces without any device allocation.
//
// Some callers cannot call cudaMalloc: hosts whose own memory pool owns the whole GPU (an
// extra allocation fails or fragments their pool), and step loops that must not allocate
// because cudaMalloc / cudaFree synchronise the device. gf_sph_forces_noalloc_dev serves
// them: the caller passes inputs and outputs in device memory as for gf_sph_forces_dev, and
// the per-particle scratch (P / rho^2 and the sound speed, 16 bytes per particle) lives in
// the fixed array below instead of a growing allocation. The array holds
// GF_SPH_NOALLOC_MAX_N particles (4 MiB); every GPU that loads the library keeps it until
// the process exits.
//
// In host code `g_sph_noalloc_scratch` names a host-side stand-in, not device memory: the
// device address is fetched with cudaGetSymbolAddress once per device (with that device
// current) by the first call on that device, and passed to the kernels. The cached address
// belongs to the device's context of that moment: after cudaDeviceReset (or a reset of the
// primary context) the array is loaded anew elsewhere and the cache is stale, so a process
// that resets a device must not call this entry point on it afterwards.

namespace gf {
namespace {

constexpr int kNoallocMaxN = GF_SPH_NOALLOC_MAX_N;
constexpr int kNoallocMaxDevices = 64;

static __device__ __align__(256) double g_sph_noalloc_scratch[2 * size_t(kNoallocMaxN)];

std::mutex g_noalloc_mu;
double* g_noalloc_ptr[kNoallocMaxDevices] = {};

// Device address of g_sph_noalloc_scratch on the current device (set up on first use).
cudaError_t noalloc_scratch(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kNoallocMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_sph_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return cudaSuccess;
}

int noalloc_fail(int code, const std::string& msg) {
    Context& c = ctx();
    c.last_status = code;
    c.last_error = msg;
    return code;
}

}  // namespace

}  // namespace gf

extern "C" int gf_sph_forces_noalloc_dev(int n, int k, const double* pos, const double* vel,
                                         const double* mass, const int64_t* nb, const double* h,
                                         const double* u, double gamma, double alpha, double beta,
                                         double* rho, double* acc, double* dudt, double* dt_i,
                                         void* stream) {
    using namespace gf;
    Context& c = ctx();
    c.last_status = 0;
    c.last_error.clear();
    if (n < 0 || k < 0) return noalloc_fail(GF_ERR_ARG, "gf_sph_forces_noalloc_dev: negative size");
    if (n > kNoallocMaxN) {
        char buf[160];
        snprintf(buf, sizeof buf, "gf_sph_forces_noalloc_dev: n = %d exceeds the fixed scratch of %d particles",
                 n, kNoallocMaxN);
        return noalloc_fail(GF_ERR_CAPACITY, buf);
    }
    if (n == 0) return GF_OK;
    if (!(pos && vel && mass && nb && h && u && rho && acc && dudt && dt_i))
        return noalloc_fail(GF_ERR_ARG, "gf_sph_forces_noalloc_dev: null array");
    double* scratch = nullptr;
    cudaError_t e = noalloc_scratch(&scratch);
    if (e != cudaSuccess)
        return noalloc_fail(GF_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    // P / rho^2 and the sound speed are written for every particle before they are read,
    // so nothing left by an earlier call needs clearing.
    double* pr2 = scratch;
    double* cs = scratch + kNoallocMaxN;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int grid = div_up(n, kThreads);
    k_sph_density<int64_t><<<grid, kThreads, 0, s>>>(n, k, k, pos, mass, nb, h, rho, Subset(), nullptr);
    k_sph_eos<<<grid, kThreads, 0, s>>>(n, rho, u, gamma, pr2, cs, Subset());
    k_sph_force<int64_t><<<grid, kThreads, 0, s>>>(n, k, k, pos, vel, mass, nb, h, rho, pr2, cs, alpha,
                                                   beta, acc, dudt, dt_i, nullptr, Subset(), nullptr);
    e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(GF_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    c.launches += 3;
    return GF_OK;
}
