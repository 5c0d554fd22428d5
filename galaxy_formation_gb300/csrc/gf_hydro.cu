// gf_hydro.cu — one device-resident force evaluation: GalaxyFormation.accelerations() and
// _hydro() of galaxy_formation/simulation.py:61-95, with the SPH neighbour cache of
// NeighbourFinder (galaxy_formation/sph.py:138-170), all on the GPU.
//
//   gravity ........ Barnes-Hut of the active particles into the persistent acc_grav
//                    (inactive rows keep their previous value, as self.acc_grav does);
//   _hydro ......... (when sph) gas = flatnonzero(kind == GAS); returns early at <= 40 gas;
//                    neighbours: on a sub-step (fresh_nb = 0) the 32 nearest are re-selected
//                    among the 48 cached candidates that are still gas; a full search runs
//                    when fresh_nb, when some gas particle is not in the cache, or when a
//                    particle has fewer than 32 candidates left; h = max(d_32 / 2, eps / 2);
//                    sph_forces; acc_sph and dt_courant scattered to global rows (zero / inf
//                    elsewhere); dt_gas = min dt_i;
//   combination .... acc = acc_grav + acc_sph, dt_ind = min(0.3 sqrt(eps / |a|), dt_courant),
//                    dt_grav = 0.3 sqrt(eps / max |a|)  (|a| floored at 1e-30).
// When sph = 0, acc_sph and dt_courant keep the values of the last hydro call, as in the
// reference.
#include <algorithm>
#include <cfloat>

#include "gf_hydro.cuh"
#include "gf_mlp.cuh"

namespace gf {

namespace {

constexpr int kThreads = 256;
constexpr int kCand = 48;   // sph.py:27 N_CANDIDATES
constexpr int kNgb = 32;    // sph.py:26 N_NEIGHBOURS

__global__ void k_gas_flag(int n, const int8_t* __restrict__ kind, int* __restrict__ flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flag[i] = kind[i] == 0 ? 1 : 0;
}

// The gas in gas-local order; with ghi/glo also its positions as float32 hi + lo pairs
// (x = float(x) + float(x - float(x))), for the float32 neighbour reselection.
__global__ void k_gas_gather(int n, const int* __restrict__ flag, const int* __restrict__ scan,
                             const double* __restrict__ pos, const double* __restrict__ vel,
                             const double* __restrict__ mass, const double* __restrict__ u,
                             int* __restrict__ gidx, double* __restrict__ gpos, double* __restrict__ gvel,
                             double* __restrict__ gmass, double* __restrict__ gu, float4* __restrict__ ghi,
                             float4* __restrict__ glo) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !flag[i]) return;
    const int g = scan[i];
    gidx[g] = i;
    double x[3];
    for (int a = 0; a < 3; ++a) {
        x[a] = pos[3 * size_t(i) + a];
        gpos[3 * size_t(g) + a] = x[a];
        gvel[3 * size_t(g) + a] = vel[3 * size_t(i) + a];
    }
    gmass[g] = mass[i];
    gu[g] = u[i];
    if (ghi) {
        const float fx = float(x[0]), fy = float(x[1]), fz = float(x[2]);
        ghi[g] = make_float4(fx, fy, fz, 0.f);
        glo[g] = make_float4(float(x[0] - double(fx)), float(x[1] - double(fy)), float(x[2] - double(fz)), 0.f);
    }
}

// loc[global] = local gas index (loc preset to -1); fails when a gas particle has no cache row
__global__ void k_verlet_prep(int ng, const int* __restrict__ gidx, const int* __restrict__ row,
                              int* __restrict__ loc, int* __restrict__ fail) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng) return;
    const int g = gidx[i];
    loc[g] = i;
    if (row[g] < 0) *fail = 1;
}

// sph.py:155-164 + knn_from_candidates (sph.py:109-135): one warp per gas particle.
constexpr int kSelWarps = 8;
__global__ void __launch_bounds__(kSelWarps * 32) k_verlet_select(
    int ng, const int* __restrict__ gidx, const int* __restrict__ row, const int* __restrict__ cache,
    const int* __restrict__ cgidx, const int* __restrict__ loc, const double* __restrict__ gpos,
    int* __restrict__ nb, double* __restrict__ d31, int* __restrict__ fail, Subset sub) {
    __shared__ unsigned long long s_key[kSelWarps][64];  // float64 d^2 bit patterns (see below)
    __shared__ int s_tag[kSelWarps][64];
    __shared__ int s_loc[kSelWarps][64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int q = blockIdx.x * kSelWarps + w;; q += gridDim.x * kSelWarps) {
        int i;
        if (!subset_item(sub, q, ng, nullptr, i)) break;
        const int r = row[gidx[i]];
        if (r < 0) continue;  // handled by k_verlet_prep's flag
        const double xi = gpos[3 * size_t(i)], yi = gpos[3 * size_t(i) + 1], zi = gpos[3 * size_t(i) + 2];
        int valid = 0;
        for (int jj = lane; jj < 64; jj += 32) {
            double d2 = INFINITY;
            int j = -1;
            if (jj < kCand) {
                // cached candidate: its local index at caching time; now (loc: null when the gas
                // set is the cached one)
                const int c = cache[size_t(r) * kCand + jj];
                j = c < 0 ? -1 : loc ? loc[cgidx[c]] : c;
                if (j >= 0) {
                    const double dx = xi - gpos[3 * size_t(j)], dy = yi - gpos[3 * size_t(j) + 1],
                                 dz = zi - gpos[3 * size_t(j) + 2];
                    d2 = dx * dx + dy * dy + dz * dz;
                    ++valid;
                }
            }
            s_key[w][jj] = (unsigned long long)__double_as_longlong(d2);
            s_tag[w][jj] = jj;
            s_loc[w][jj] = j;
        }
        valid = warp_sum(valid);
        __syncwarp();
        if (valid < kNgb) {
            if (lane == 0) *fail = 1;
            continue;
        }
        // bitonic sort of 64 (key, slot) pairs; non-negative float64 keys compare as their bit
        // patterns (integer compares: the float64 pipe is narrow on this GPU)
        for (int size = 2; size <= 64; size <<= 1) {
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                const int t = lane;
                const int a = 2 * stride * (t / stride) + (t % stride);
                const int b = a + stride;
                const bool up = (a & size) == 0;
                const unsigned long long ka = s_key[w][a], kb = s_key[w][b];
                const int ta = s_tag[w][a], tb = s_tag[w][b];
                const bool gt = ka > kb || (ka == kb && ta > tb);
                if (gt == up) {
                    s_key[w][a] = kb;
                    s_key[w][b] = ka;
                    s_tag[w][a] = tb;
                    s_tag[w][b] = ta;
                }
                __syncwarp();
            }
        }
        nb[size_t(i) * kCand + lane] = s_loc[w][s_tag[w][lane]];
        if (lane == kNgb - 1) d31[i] = sqrt(__longlong_as_double((long long)s_key[w][lane]));
        __syncwarp();
    }
}

// Float64 squared distance of gas particles i and j (gas-local), rounded as NumPy sums the three
// squares: (dx^2 + dy^2) + dz^2.
__device__ __forceinline__ double gas_d2(const double* __restrict__ gpos, int i, int j) {
    const double dx = __dsub_rn(gpos[3 * size_t(i)], gpos[3 * size_t(j)]);
    const double dy = __dsub_rn(gpos[3 * size_t(i) + 1], gpos[3 * size_t(j) + 1]);
    const double dz = __dsub_rn(gpos[3 * size_t(i) + 2], gpos[3 * size_t(j) + 2]);
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// The same reselection for the float32 SPH of the mixed form, in float32: the candidates'
// squared distances from hi + lo positions (~1e-7 relative error), sorted as (float32 d^2,
// slot) keys. Only the candidates within float32 rounding of the 32nd are measured in float64,
// so the set of the 32 nearest is the float64 one; the neighbour that fixes h is returned in
// sel (its float64 distance is taken by k_smoothing, a thread per particle, instead of
// warp-uniformly here: the float64 pipe is narrow on this GPU). The 32 come out in float32
// order (only float32 near-ties can swap with respect to the float64 order).
__global__ void __launch_bounds__(kSelWarps * 32) k_verlet_select32(
    int ng, const int* __restrict__ gidx, const int* __restrict__ row, const int* __restrict__ cache,
    const int* __restrict__ cgidx, const int* __restrict__ loc, const float4* __restrict__ ghi,
    const float4* __restrict__ glo, const double* __restrict__ gpos, int* __restrict__ nb, int* __restrict__ sel,
    int* __restrict__ fail, Subset sub) {
    __shared__ unsigned long long s_key[kSelWarps][64];  // (float32 d^2 bits << 32) | slot
    __shared__ unsigned long long s_dd[kSelWarps][64];   // float64 d^2 bits of the boundary band
    __shared__ int s_di[kSelWarps][64];
    __shared__ int s_loc[kSelWarps][64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int q = blockIdx.x * kSelWarps + w;; q += gridDim.x * kSelWarps) {
        int i;
        if (!subset_item(sub, q, ng, nullptr, i)) break;
        const int r = row[gidx[i]];
        if (r < 0) continue;  // handled by k_verlet_prep's flag
        const float4 hi_i = ghi[i], lo_i = glo[i];
        int valid = 0;
        for (int jj = lane; jj < 64; jj += 32) {
            unsigned long long key = ~0ull;
            int j = -1;
            if (jj < kCand) {
                const int c = cache[size_t(r) * kCand + jj];
                j = c < 0 ? -1 : loc ? loc[cgidx[c]] : c;
                if (j >= 0) {
                    const float4 hj = ghi[j], lj = glo[j];
                    const float dx = (hi_i.x - hj.x) + (lo_i.x - lj.x);
                    const float dy = (hi_i.y - hj.y) + (lo_i.y - lj.y);
                    const float dz = (hi_i.z - hj.z) + (lo_i.z - lj.z);
                    key = ((unsigned long long)__float_as_uint(dx * dx + dy * dy + dz * dz) << 32) | unsigned(jj);
                    ++valid;
                }
            }
            s_key[w][jj] = key;
            s_loc[w][jj] = j;
        }
        valid = warp_sum(valid);
        __syncwarp();
        if (valid < kNgb) {
            if (lane == 0) *fail = 1;
            continue;
        }
        warp_sort_u64(s_key[w], 64);
        // the boundary: entries within float32 rounding of the 32nd (the unused slots' keys
        // read as NaN and fall in neither count)
        constexpr int c = kNgb - 1;
        const float dc = __uint_as_float(unsigned(s_key[w][c] >> 32));
        const float blo = dc * (1.0f - 2e-5f), bhi = dc * (1.0f + 2e-5f);
        int below = 0, inband = 0;
        for (int t = lane; t < 64; t += 32) {
            const float v = __uint_as_float(unsigned(s_key[w][t] >> 32));
            below += v < blo;
            inband += v >= blo && v <= bhi;
        }
        below = warp_sum(below);
        inband = warp_sum(inband);
        int selj;
        if (inband == 1) {
            selj = s_loc[w][unsigned(s_key[w][c]) & 63u];
        } else {  // re-measure the band in float64; its entries take the float64 order
            for (int t = lane; t < 64; t += 32) {
                double v = INFINITY;
                int tag = 0x7fffffff;
                const float vf = __uint_as_float(unsigned(s_key[w][t] >> 32));
                if (vf >= blo && vf <= bhi) {
                    tag = int(unsigned(s_key[w][t]) & 63u);
                    v = gas_d2(gpos, i, s_loc[w][tag]);
                }
                s_dd[w][t] = (unsigned long long)__double_as_longlong(v);
                s_di[w][t] = tag;
            }
            __syncwarp();
            warp_bitonic(s_dd[w], s_di[w], 64);
            selj = s_loc[w][s_di[w][max(0, c - below)]];
            if (below + inband <= 64)
                for (int t = lane; t < inband; t += 32)
                    s_key[w][below + t] = (s_key[w][below + t] & 0xffffffff00000000ull) | unsigned(s_di[w][t]);
            __syncwarp();
        }
        nb[size_t(i) * kCand + lane] = s_loc[w][unsigned(s_key[w][lane]) & 63u];
        if (lane == 0) sel[i] = selj;
        __syncwarp();
    }
}

// one thread per cache entry (coalesced rows of 48 local indices; cgidx keeps the local ->
// global map of the caching call)
// The full search wrote its candidates straight into the cache (kq columns of kCand); this
// records whose rows they are and marks the columns a search of fewer than kCand left empty.
__global__ void k_cache_rows(int ng, int kq, const int* __restrict__ gidx, int* __restrict__ row,
                             int* __restrict__ cache, int* __restrict__ cgidx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng) return;
    const int g = gidx[i];
    row[g] = i;
    cgidx[i] = g;
    for (int jj = kq; jj < kCand; ++jj) cache[size_t(i) * kCand + jj] = -1;
}

__global__ void k_guess(int ng, const int* __restrict__ gidx, const double* __restrict__ hprev, float* __restrict__ rg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng) return;
    // the 48th neighbour lies near 2 h (48/32)^(1/3) = 2.29 h; start outside it (2.5 h: 1 %
    // faster than 2.4 h, whose radius fell short for 15 % of the particles; 2.6 h is slower)
    rg[i] = float(2.5 * hprev[gidx[i]]);
}

// h from the distance of the 32nd neighbour: d31, or (sel) measured here in float64 to the
// neighbour sel[i] and stored into d31.
__global__ void k_smoothing(int ng, double* __restrict__ d31, double eps, const int* __restrict__ gidx,
                            double* __restrict__ h, double* __restrict__ hprev, Subset sub,
                            const int* __restrict__ sel = nullptr, const double* __restrict__ gpos = nullptr) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (!subset_item(sub, i, ng, nullptr, i)) return;
    double d;
    if (sel) {
        const int j = sel[i];
        d = j >= 0 ? __dsqrt_rn(gas_d2(gpos, i, j)) : INFINITY;
        d31[i] = d;
    } else {
        d = d31[i];
    }
    const double v = fmax(0.5 * d, 0.5 * eps);  // simulation.py:84
    h[i] = v;
    hprev[gidx[i]] = 0.5 * d > 0 ? 0.5 * d : v;
}

// Training pairs: the features and the log distance of the 48th nearest (the radius the
// search has to reach), twice per particle: with its previous h and divergence, and as a
// particle without them would see it (the cold_log_h stand-in, divergence 0), so that the one
// network serves searches with and without a previous h.
__global__ void k_collect(int ng, long long base, int k, const float* __restrict__ X, const float* __restrict__ dk,
                          float* __restrict__ colX, float* __restrict__ colT) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng) return;
    const size_t r = size_t(base) + 2 * size_t(i);
    const float t = logf(fmaxf(dk[i], 1e-30f));
    for (int c = 0; c < 4; ++c) colX[4 * r + c] = X[4 * size_t(i) + c];
    colT[r] = t;
    const float f0 = X[4 * size_t(i)];
    colX[4 * (r + 1) + 0] = f0;
    colX[4 * (r + 1) + 1] = cold_log_h(f0, k);
    colX[4 * (r + 1) + 2] = X[4 * size_t(i) + 2];
    colX[4 * (r + 1) + 3] = 0.f;
    colT[r + 1] = t;
}

__global__ void k_scatter_f(int ng, const int* __restrict__ gidx, const float* __restrict__ v, float* __restrict__ out,
                            Subset sub) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (subset_item(sub, i, ng, nullptr, i)) out[gidx[i]] = v[i];
}

// gas-local flags of the particles due (active: per particle), in the visiting order (order:
// position -> gas-local index)
__global__ void k_flag_in_order(int ng, const int* __restrict__ order, const int* __restrict__ gidx,
                                const uint8_t* __restrict__ active, int* __restrict__ flag) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < ng) flag[t] = active[gidx[order ? order[t] : t]] ? 1 : 0;
}

__global__ void k_compact(int ng, const int* __restrict__ order, const int* __restrict__ flag,
                          const int* __restrict__ scan, int* __restrict__ list) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < ng && flag[t]) list[scan[t]] = order ? order[t] : t;
}

__global__ void k_fill(int n, double* __restrict__ a, double v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

// dtmin_bits (may be null): block minimum of the Courant steps, one atomic per block
__global__ void k_scatter_sph(int ng, const int* __restrict__ gidx, const double* __restrict__ a,
                              const double* __restrict__ dti, double* __restrict__ acc_sph,
                              double* __restrict__ dt_courant, unsigned long long* __restrict__ dtmin_bits,
                              Subset sub) {
    __shared__ double s_min[kThreads / 32];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = INFINITY;
    if (subset_item(sub, i, ng, nullptr, i)) {
        const int g = gidx[i];
        for (int c = 0; c < 3; ++c) acc_sph[3 * size_t(g) + c] = a[3 * size_t(i) + c];
        dt_courant[g] = dti[i];
        v = dti[i];
    }
    if (!dtmin_bits) return;
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) s_min[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kThreads / 32; ++w) v = fmin(v, s_min[w]);
        if (v >= 0) atomicMin(dtmin_bits, __double_as_longlong(v));
    }
}

// f32 (mixed form): |a| and the gravitational step criterion in float32 (two float64
// square roots and a division per particle are the float64 pipe's bottleneck here)
// only: when set, the particles whose terms changed (inactive rows would be recomputed to
// the values they hold); amax_bits (block maximum, one atomic per block) may then be null.
__global__ void k_combine(int n, const double* __restrict__ ag, const double* __restrict__ as,
                          const double* __restrict__ dtc, double eps, double* __restrict__ acc,
                          double* __restrict__ dt_ind, unsigned long long* __restrict__ amax_bits, int f32,
                          const uint8_t* __restrict__ only) {
    __shared__ double s_max[kThreads / 32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double m = 0;
    if (i < n && !(only && !only[i])) {
        double a2 = 0;
        for (int c = 0; c < 3; ++c) {
            const double v = ag[3 * size_t(i) + c] + as[3 * size_t(i) + c];
            acc[3 * size_t(i) + c] = v;
            a2 += v * v;
        }
        if (f32) {
            const float mf = sqrtf(float(a2));
            m = mf;
            dt_ind[i] = fmin(double(0.3f * sqrtf(float(eps) / fmaxf(mf, 1e-30f))), dtc[i]);
        } else {
            m = sqrt(a2);
            dt_ind[i] = fmin(0.3 * sqrt(eps / fmax(m, 1e-30)), dtc[i]);
        }
    }
    if (!amax_bits) return;
#pragma unroll
    for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kThreads / 32; ++w) m = fmax(m, s_max[w]);
        atomicMax(amax_bits, __double_as_longlong(m));  // |a| >= 0: bit order = numeric order
    }
}

__global__ void k_finish(HydroScalars* sc, double eps) {
    const double amax = __longlong_as_double(sc->amax_bits);
    sc->dt_grav = 0.3 * sqrt(eps / fmax(amax, 1e-30));
    sc->dt_gas = sc->ng > 40 ? __longlong_as_double(sc->dtmin_bits) : INFINITY;
}

}  // namespace

static ForceEngine g_force;
ForceEngine& force_engine() { return g_force; }

void ForceEngine::evaluate(const ForceArgs& a, cudaStream_t s) {
    Context& C = ctx();
    ProfScope ps(kStForce, s);
    const int n = a.n;
    if (n_total != n) {  // new particle set: reset persistent state (np.zeros / np.full)
        n_total = n;
        double* ag = acc_grav.get<double>(3 * size_t(n));
        GF_CUDA(cudaMemsetAsync(ag, 0, sizeof(double) * 3 * size_t(n), s));
        GF_CUDA(cudaMemsetAsync(acc_sph.get<double>(3 * size_t(n)), 0, sizeof(double) * 3 * size_t(n), s));
        k_fill<<<div_up(n, kThreads), kThreads, 0, s>>>(n, dt_courant.get<double>(n), INFINITY);
        GF_CHECK_LAUNCH();
        GF_CUDA(cudaMemsetAsync(h_prev.get<double>(n), 0, sizeof(double) * size_t(n), s));
        cache_valid = false;
        have_hprev = false;
        have_divv = false;
        have_aold = false;
        GF_CUDA(cudaMemsetAsync(divv_prev.get<float>(n), 0, sizeof(float) * size_t(n), s));
        row.get<int>(n);
        loc.get<int>(n);
    }
    if (!scalars_h) GF_CUDA(cudaMallocHost(&scalars_h, sizeof(HydroScalars)));
    HydroScalars* sc = scalars.get<HydroScalars>(1);

    // Gravity on s, hydro on a second stream: the two are independent until the combination.
    // The gravity chain is queued first and without host synchronisation (a tree of this
    // particle set was built before: its node buffers bound the new one), so the GPU runs it
    // while the host drives the hydro chain, whose own synchronisations wait on its stream only.
    if (!s3) {
        int lowest = 0, greatest = 0;
        GF_CUDA(cudaDeviceGetStreamPriorityRange(&lowest, &greatest));
        GF_CUDA(cudaStreamCreateWithPriority(&s3, cudaStreamNonBlocking, greatest));
        GF_CUDA(cudaEventCreateWithFlags(&ev_gathered, cudaEventDisableTiming));
        GF_CUDA(cudaEventCreateWithFlags(&ev_moments, cudaEventDisableTiming));
    }
    const bool fork = a.sph != 0;
    if (fork) {
        if (!s2) {
            // the hydro chain at the highest priority: its small kernels (neighbour-tree build,
            // SPH passes) then get SMs ahead of the walk's blocks (measured 0.8 % faster; the
            // reverse order is 3 % slower)
            int lowest = 0, greatest = 0;
            GF_CUDA(cudaDeviceGetStreamPriorityRange(&lowest, &greatest));
            GF_CUDA(cudaStreamCreateWithPriority(&s2, cudaStreamNonBlocking, greatest));
            GF_CUDA(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
            GF_CUDA(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
        }
        GF_CUDA(cudaEventRecord(ev_fork, s));
        GF_CUDA(cudaStreamWaitEvent(s2, ev_fork, 0));
    }

    // gravity (simulation.py:64)
    Octree& T = grav;
    const int gmax = gravity_quad ? walk_group : kGroupMax;  // the mixed form's groups are tunable
    const bool rel = gravity_quad && grav_rel > 0 && have_aold;
    const double theta = rel ? kRelFloorTheta : a.theta;
    // a refit's moments run beside the preparation of the walk items (joined before the walk)
    bool split_refit = false;
    if (a.nosync) {  // inside a captured graph: the tree of the last regular build, rebuilt or refitted
        if (!T.valid || T.n != n) throw Error(GF_ERR_ARG, "a synchronisation-free evaluation needs a built tree");
        if (a.rebuild) {
            T.build(n, a.pos, a.mass, theta, s, true);
        } else {
            T.refit(a.pos, a.mass, s, s3, ev_gathered);
            split_refit = true;
        }
    } else if (a.rebuild || !T.valid || T.n != n || T.quad != (gravity_quad != 0) || T.group_max != gmax) {
        const bool same_set = T.valid && T.n == n && T.quad == (gravity_quad != 0) && T.group_max == gmax &&
                              !T.outgrowing();
        T.quad = gravity_quad != 0;
        T.group_max = gmax;
        if (same_set) {
            T.reserve_graph_build();
            T.build(n, a.pos, a.mass, theta, s, true);
        } else {
            T.build(n, a.pos, a.mass, theta, s);
        }
    } else {
        T.refit(a.pos, a.mass, s, s3, ev_gathered);
        split_refit = true;
    }
    T.merge_cap = gravity_quad ? walk_merge : 0;
    T.prepare_walk(a.active, s, a.walk_chunk ? a.walk_chunk : walk_chunk, rel ? acc_grav.as<double>() : nullptr,
                   rel ? float(grav_rel) : 0.f, rel ? float(grav_rel_mono) : 0.f);
    if (split_refit) {
        GF_CUDA(cudaEventRecord(ev_moments, s3));
        GF_CUDA(cudaStreamWaitEvent(s, ev_moments, 0));
    }
    T.walk(a.eps, acc_grav.as<double>(), s, nullptr, a.walk_npl, a.walk_shape >= 0 ? a.walk_shape : walk_shape);
    if (!a.active) have_aold = true;  // every particle has a previous gravity now

    if (fork) {
        hydro(a, s2);
        GF_CUDA(cudaEventRecord(ev_join, s2));
        GF_CUDA(cudaStreamWaitEvent(s, ev_join, 0));
    }

    // combination (simulation.py:68-71)
    if (!a.nosync) GF_CUDA(cudaMemsetAsync(&sc->amax_bits, 0, sizeof(unsigned long long), s));
    // inside a captured block only the active rows change, and nothing reads dt_grav
    const bool only_active = a.nosync && a.active;
    k_combine<<<div_up(n, kThreads), kThreads, 0, s>>>(n, acc_grav.as<double>(), acc_sph.as<double>(),
                                                       dt_courant.as<double>(), a.eps, a.acc, a.dt_ind,
                                                       only_active ? nullptr : &sc->amax_bits,
                                                       gravity_quad ? 1 : 0, only_active ? a.active : nullptr);
    GF_CHECK_LAUNCH();
    if (a.nosync) return;  // the host reads no scalars inside a captured block
    k_finish<<<1, 1, 0, s>>>(sc, a.eps);
    GF_CHECK_LAUNCH();
    GF_CUDA(cudaMemcpyAsync(scalars_h, sc, sizeof(HydroScalars), cudaMemcpyDeviceToHost, s));
    (void)C;
}

void ForceEngine::autotune_walk(double eps, cudaStream_t s, int* merge_out, int* shape_out, double* ms_out) {
    Octree& T = grav;
    if (!T.valid || !T.quad || !gravity_quad)
        throw Error(GF_ERR_ARG, "the walk autotuner needs a mixed-form (quadrupole) evaluation first");
    const bool rel = grav_rel > 0 && have_aold;
    double* ta = tune_acc.get<double>(3 * size_t(T.n));
    static const int merges[] = {0, 24, 32, 40, 48, 64};
    Event e0, e1;
    double best = INFINITY;
    int best_m = walk_merge, best_s = walk_shape;
    for (int m : merges) {
        for (int shape = 0; shape < kNumWalkShapes; ++shape) {
            double ms[3];
            for (int r = 0; r < 3; ++r) {
                T.merge_cap = m;
                T.prepare_walk(nullptr, s, 0, rel ? acc_grav.as<double>() : nullptr, rel ? float(grav_rel) : 0.f,
                               rel ? float(grav_rel_mono) : 0.f);
                e0.record(s);
                T.walk(eps, ta, s, nullptr, 2, shape);
                e1.record(s);
                GF_CUDA(cudaStreamSynchronize(s));
                ms[r] = e1.since(e0);
            }
            std::sort(ms, ms + 3);
            if (ms[1] < best) {
                best = ms[1];
                best_m = m;
                best_s = shape;
            }
        }
    }
    walk_merge = best_m;
    walk_shape = best_s;
    T.merge_cap = best_m;
    if (merge_out) *merge_out = best_m;
    if (shape_out) *shape_out = best_s;
    if (ms_out) *ms_out = best;
}

void ForceEngine::hydro(const ForceArgs& a, cudaStream_t s) {
    const int n = a.n;
    const int grid = div_up(n, kThreads);
    HydroScalars* sc = scalars.as<HydroScalars>();
    double* as = acc_sph.as<double>();
    double* dtc = dt_courant.as<double>();
    const bool partial = a.sph_active != nullptr;
    if (!partial) {
        GF_CUDA(cudaMemsetAsync(as, 0, sizeof(double) * 3 * size_t(n), s));  // simulation.py:75-76
        k_fill<<<grid, kThreads, 0, s>>>(n, dtc, INFINITY);
        GF_CHECK_LAUNCH();
    }

    int* fl = flag.get<int>(n);
    int* sc_ = scan.get<int>(n);
    if (!a.nosync) {
        k_gas_flag<<<grid, kThreads, 0, s>>>(n, a.kind, fl);
        GF_CHECK_LAUNCH();
        GF_CUDA(cudaMemsetAsync(sc, 0, sizeof(HydroScalars), s));
        GF_CUDA(cudaMemsetAsync(&sc->dtmin_bits, 0x7f, sizeof(unsigned long long), s));
        exclusive_scan(fl, sc_, n, &sc->ng, s, &hscratch);
        GF_CUDA(cudaMemcpyAsync(&scalars_h->ng, &sc->ng, sizeof(int), cudaMemcpyDeviceToHost, s));
        GF_CUDA(cudaStreamSynchronize(s));
        ng = scalars_h->ng;
        if (ng <= 40) {  // simulation.py:80
            ng_valid = 0;
            return;
        }
        ng_valid = ng;
    } else {
        if (ng_valid == 0) return;  // gas set of the last regular call
        GF_CUDA(cudaMemsetAsync(&sc->dtmin_bits, 0x7f, sizeof(unsigned long long), s));
    }
    int* gi = gidx.get<int>(ng);
    double* gp = gpos.get<double>(3 * size_t(ng));
    double* gv = gvel.get<double>(3 * size_t(ng));
    double* gm = gmass.get<double>(ng);
    double* gu = gu_.get<double>(ng);
    if (a.late_inputs) GF_CUDA(cudaStreamWaitEvent(s, a.late_inputs, 0));
    // the mixed form reselects neighbours from float32 hi + lo positions
    const bool sel32 = sph_float32 && !a.fresh_nb && cache_valid;
    float4* ghi_ = sel32 ? ghi.get<float4>(ng) : nullptr;
    float4* glo_ = sel32 ? glo.get<float4>(ng) : nullptr;
    k_gas_gather<<<grid, kThreads, 0, s>>>(n, fl, sc_, a.pos, a.vel, a.mass, a.u, gi, gp, gv, gm, gu, ghi_, glo_);
    GF_CHECK_LAUNCH();

    const int ggrid = div_up(ng, kThreads);
    int* nb = nb48.get<int>(size_t(ng) * kCand);
    double* d31 = dsel.get<double>(ng);
    // partial: the gas due, compacted in the visiting order of the last neighbour-search tree
    Subset sub;
    if (partial) {
        const int* vorder = order_ng == ng ? knn_tree.perm.as<int>() : nullptr;
        int* fl2 = aflag.get<int>(ng);
        int* sc2 = ascan.get<int>(ng);
        int* lst = alist.get<int>(ng);
        k_flag_in_order<<<ggrid, kThreads, 0, s>>>(ng, vorder, gi, a.sph_active, fl2);
        GF_CHECK_LAUNCH();
        exclusive_scan(fl2, sc2, ng, &sc->nact, s, &hscratch);
        k_compact<<<ggrid, kThreads, 0, s>>>(ng, vorder, fl2, sc2, lst);
        GF_CHECK_LAUNCH();
        sub = Subset{lst, &sc->nact};
    }
    bool have_nb = false;
    int* vsel_ = nullptr;  // float32 reselection: the neighbour that fixes each h
    if (!a.fresh_nb && cache_valid) {
        // inside a captured block the gas set is the cached one: local index == cache row
        int* lc = a.nosync ? row.as<int>() : loc.as<int>();
        if (!a.nosync) {
            GF_CUDA(cudaMemsetAsync(lc, 0xff, sizeof(int) * size_t(n), s));
            GF_CUDA(cudaMemsetAsync(&sc->fail, 0, sizeof(int), s));
            k_verlet_prep<<<ggrid, kThreads, 0, s>>>(ng, gi, row.as<int>(), lc, &sc->fail);
            GF_CHECK_LAUNCH();
        }
        const int blocks = std::min(div_up(ng, kSelWarps), 16 * ctx().sms);
        ProfScope pv(kStVerlet, s);
        if (sel32) {
            vsel_ = vsel.get<int>(ng);
            k_verlet_select32<<<blocks, kSelWarps * 32, 0, s>>>(ng, gi, row.as<int>(), cache.as<int>(),
                                                                cgidx.as<int>(), a.nosync ? nullptr : lc, ghi_,
                                                                glo_, gp, nb, vsel_, &sc->fail, sub);
        } else {
            k_verlet_select<<<blocks, kSelWarps * 32, 0, s>>>(ng, gi, row.as<int>(), cache.as<int>(),
                                                              cgidx.as<int>(), a.nosync ? nullptr : lc, gp, nb, d31,
                                                              &sc->fail, sub);
        }
        GF_CHECK_LAUNCH();
        if (a.nosync) {  // the gas set is the cached one: every particle keeps its candidates
            have_nb = true;
        } else {
            GF_CUDA(cudaMemcpyAsync(&scalars_h->fail, &sc->fail, sizeof(int), cudaMemcpyDeviceToHost, s));
            GF_CUDA(cudaStreamSynchronize(s));
            have_nb = scalars_h->fail == 0;
        }
        verlet_hits += have_nb ? 1 : 0;
    }
    if (!have_nb && a.nosync) throw Error(GF_ERR_ARG, "a synchronisation-free evaluation needs a neighbour cache");
    if (!have_nb) {  // full search, 48 candidates (sph.py:165-169), written into the cache
        vsel_ = vsel.get<int>(ng);  // the neighbour that fixes each h (k_smoothing measures it)
        const int kq = std::min(kCand, ng);
        nb = cache.get<int>(size_t(ng) * kCand);
        float* rg = nullptr;
        if (have_hprev && (hguess == 0 || hguess == 2)) {  // previous h
            rg = rguess.get<float>(ng);
            k_guess<<<ggrid, kThreads, 0, s>>>(ng, gi, h_prev.as<double>(), rg);
            GF_CHECK_LAUNCH();
        }
        const bool collect = collect_cap > collect_n && have_hprev;
        // the learned guess starts the searches that have no previous h (the first of a particle
        // set); where a previous h exists, 2.5 h is the better start (fewer radius iterations)
        HGuess hg{gi, have_hprev ? h_prev.as<double>() : nullptr, have_divv ? divv_prev.as<float>() : nullptr,
                  hX.get<float>(4 * size_t(ng)), hY.get<float>(ng), hrg.get<float>(ng),
                  hguess == 2 && !have_hprev && mlp().ready, collect ? hdk.get<float>(ng) : nullptr};
        const bool features = collect || hg.use_mlp;
        GF_CUDA(cudaMemsetAsync(&sc->knn_iters, 0, sizeof(unsigned long long), s));
        // the gas of the last full search, moved (same count): rebuild without a host round trip
        knn_exact(knn_tree, ng, gp, kq, rg, nullptr, nullptr, &sc->knn_iters, s, nb, kCand, d31, kNgb - 1,
                  features ? &hg : nullptr, order_ng == ng, vsel_);
        if (collect) {
            const long long take = std::min<long long>(ng, (collect_cap - collect_n) / 2);  // two rows each
            if (take > 0) {
                k_collect<<<div_up(take, kThreads), kThreads, 0, s>>>(int(take), collect_n, kq, hg.X, hg.dk,
                                                                      colX.as<float>(), colT.as<float>());
                GF_CHECK_LAUNCH();
                collect_n += 2 * take;
            }
        }
        int* rw = row.as<int>();
        GF_CUDA(cudaMemsetAsync(rw, 0xff, sizeof(int) * size_t(n), s));
        k_cache_rows<<<ggrid, kThreads, 0, s>>>(ng, kq, gi, rw, nb, cgidx.get<int>(ng));
        GF_CHECK_LAUNCH();
        cache_valid = true;
        full_searches += 1;
        order_ng = ng;
    }
    last_nb = nb;
    double* hh = h.get<double>(ng);
    k_smoothing<<<ggrid, kThreads, 0, s>>>(ng, d31, a.eps, gi, hh, h_prev.as<double>(), sub, vsel_, gp);
    GF_CHECK_LAUNCH();
    have_hprev = true;

    double* r = rho.get<double>(ng);
    double* gacc_ = gacc.get<double>(3 * size_t(ng));
    double* du = dudt.get<double>(ng);
    double* dti = dt_i.get<double>(ng);
    float* dv = gdivv.get<float>(ng);
    if (sph_float32) {
        // visit the gas in the Morton order of the last neighbour-search tree (same gas set)
        const int* order = order_ng == ng ? knn_tree.perm.as<int>() : nullptr;
        sph_forces32<int>(sph32, ng, kNgb, kCand, order, gp, gv, gm, nb, hh, gu, a.gamma, a.alpha, a.beta, r,
                          gacc_, du, dti, s, dv, sub);
    } else {
        sph_forces<int>(sph, ng, kNgb, kCand, gp, gv, gm, nb, hh, gu, a.gamma, a.alpha, a.beta, r, gacc_, du, dti,
                        s, dv, sub);
    }
    k_scatter_f<<<ggrid, kThreads, 0, s>>>(ng, gi, dv, divv_prev.as<float>(), sub);
    GF_CHECK_LAUNCH();
    have_divv = true;
    k_scatter_sph<<<ggrid, kThreads, 0, s>>>(ng, gi, gacc_, dti, as, dtc, a.nosync ? nullptr : &sc->dtmin_bits, sub);
    GF_CHECK_LAUNCH();
}

}  // namespace gf
