// gf_tree.cu — GPU octree that reproduces the reference's Barnes-Hut tree
// (cpp/nbody.cpp:76-256) and its refit (cpp/nbody.cpp:262-305).
//
// The reference partitions index ranges recursively: a particle goes to octant bit k of a
// cell when coordinate k is strictly greater than the cell centre, centres being computed
// in float64 by repeated halving (child = parent +- half/2). Partitions are stable, so
// inside every cell particles keep increasing index order; a cell is a leaf when it holds
// at most 8 particles or sits at depth 48; nodes are stored depth-first with `next` links.
//
// Here the same tree comes out of a sort:
//   1. float64 bbox -> root cube, same formula as cpp/nbody.cpp:218-219.
//   2. 63-bit Morton key per particle holding its octant at levels 1..21. Fast path: a
//      fixed-point grid position; when a coordinate lies within a rounding margin of a
//      cell wall the key is recomputed with the exact float64 centre chain, so every
//      octant decision equals the reference's `pos > c` test.
//   3. stable radix sort of (key, index): tree order = (octant path, index).
//   4. cells: 9 consecutive sorted keys sharing a level-d prefix <=> that cell holds > 8
//      particles, so each particle's leaf depth and the nodes that start at it follow from
//      common-prefix lengths of neighbouring keys; an exclusive scan numbers the nodes in
//      depth-first order, and `next` is the id of the first node starting after the cell.
//      Cells that still hold > 8 particles at level 21 get extension keys (levels 22..48,
//      exact chain) and are re-sorted in shared memory.
//   5. leaves re-sorted by index (the reference never partitions a leaf).
//   6. moments bottom-up in one launch (the last child to arrive computes its parent,
//      children summed in octant order), float64 sums of the same terms as the reference,
//      rounded to the same float32 node record.
#include <algorithm>
#include <cfloat>
#include <climits>

#include "gf_tree.cuh"

namespace gf {

namespace {

constexpr int kThreads = 256;

// ---------------------------------------------------------------------------- bbox

// Order-preserving map of float64 values to int64 (and back): min / max of the images is the
// image of the min / max, so the reduction runs on the integer pipes instead of the narrow
// float64 one. Non-finite values are flagged separately.
__device__ __forceinline__ long long fkey(double v) {
    const long long b = __double_as_longlong(v);
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double fkey_inv(long long k) { return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffLL)); }
__device__ __forceinline__ bool finite_bits(double v) {
    return ((__double_as_longlong(v) >> 52) & 0x7ff) != 0x7ff;
}

// float64 bounding box -> root cube (cpp/nbody.cpp:210-219) in one launch: every block reduces
// its share of the positions and writes a partial; the last block to finish (arrival counter)
// reduces the partials and writes the root cube. min / max are exact, so the result does not
// depend on the order of the reductions.
__global__ void k_bbox(const double* __restrict__ pos, int n, double* __restrict__ part, RootBox* __restrict__ root,
                       uint32_t* status, int* __restrict__ done) {
    long long lo[3] = {LLONG_MAX, LLONG_MAX, LLONG_MAX}, hi[3] = {LLONG_MIN, LLONG_MIN, LLONG_MIN};
    int bad = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const double v = pos[3 * size_t(i) + a];
            bad |= finite_bits(v) ? 0 : 1;
            const long long k = fkey(v);
            lo[a] = min(lo[a], k);
            hi[a] = max(hi[a], k);
        }
    }
    __shared__ long long s[6][kThreads / 32];
    __shared__ int s_bad[kThreads / 32];
    __shared__ bool s_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    auto block_reduce = [&](long long* out, int* out_bad) {
#pragma unroll
        for (int o = 16; o; o >>= 1) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                lo[a] = min(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
                hi[a] = max(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
            }
            bad |= __shfl_xor_sync(0xffffffffu, bad, o);
        }
        if (lane == 0) {
            for (int a = 0; a < 3; ++a) {
                s[a][warp] = lo[a];
                s[3 + a][warp] = hi[a];
            }
            s_bad[warp] = bad;
        }
        __syncthreads();
        if (threadIdx.x < 6) {
            long long v = s[threadIdx.x][0];
            for (int w = 1; w < kThreads / 32; ++w)
                v = threadIdx.x < 3 ? min(v, s[threadIdx.x][w]) : max(v, s[threadIdx.x][w]);
            out[threadIdx.x] = v;
        }
        if (threadIdx.x == 6) {
            int v = 0;
            for (int w = 0; w < kThreads / 32; ++w) v |= s_bad[w];
            *out_bad = v;
        }
    };
    long long* ipart = reinterpret_cast<long long*>(part);
    int dummy;
    block_reduce(ipart + 7 * size_t(blockIdx.x), &dummy);
    if (threadIdx.x == 6) ipart[7 * size_t(blockIdx.x) + 6] = dummy;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(done, 1) == int(gridDim.x) - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    for (int a = 0; a < 3; ++a) {
        lo[a] = LLONG_MAX;
        hi[a] = LLONG_MIN;
    }
    bad = 0;
    for (int b = threadIdx.x; b < int(gridDim.x); b += blockDim.x) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = min(lo[a], __ldcg(&ipart[7 * size_t(b) + a]));
            hi[a] = max(hi[a], __ldcg(&ipart[7 * size_t(b) + 3 + a]));
        }
        bad |= int(__ldcg(&ipart[7 * size_t(b) + 6]));
    }
    __shared__ long long itot[6];
    __shared__ int tot_bad;
    __syncthreads();
    block_reduce(itot, &tot_bad);
    __syncthreads();
    if (threadIdx.x != 0) return;
    double tot[6];
    for (int a = 0; a < 6; ++a) tot[a] = fkey_inv(itot[a]);
    if (tot_bad) raise_status(status, GF_ERR_NONFINITE);
    RootBox R;
    double ext = 0;
    for (int a = 0; a < 3; ++a) {
        R.c[a] = __dmul_rn(0.5, __dadd_rn(tot[a], tot[3 + a]));
        ext = fmax(ext, __dsub_rn(tot[3 + a], tot[a]));
    }
    // 0.5 * max extent * 1.0001 + 1e-12 (cpp/nbody.cpp:219), unfused
    R.half = __dadd_rn(__dmul_rn(__dmul_rn(0.5, ext), 1.0001), 1e-12);
    double cmax = 0;
    for (int a = 0; a < 3; ++a) {
        R.lo[a] = __dsub_rn(R.c[a], R.half);
        cmax = fmax(cmax, fabs(R.c[a]));
    }
    R.inv_w = __ddiv_rn(2097152.0, __dmul_rn(2.0, R.half));
    // Rounding of the float64 centre chain (<= 21 roundings of <= 1/2 ulp(|c| + half)) plus
    // that of the fixed-point position stays below 2^-27 (|c|/half + 2) grid units; the
    // margin keeps a factor 8 on top.
    R.margin = ldexp(1.0, -24) * (cmax / R.half + 2.0);
    // the same test in 32.32 fixed point (scaling by 2^32 is exact): the fraction window
    // [m_lo, m_hi] of the truncated fixed-point position lies inside [margin, 1 - margin]
    R.inv_w32 = R.inv_w * 4294967296.0;
    const double ml = fmin(ceil(R.margin * 4294967296.0), 2147483648.0);
    R.m_lo = uint32_t(ml);
    R.m_hi = uint32_t(4294967295.0 - ml);
    *root = R;
}

// ---------------------------------------------------------------------------- keys

__device__ __forceinline__ uint64_t part1by2(uint32_t v) {
    uint64_t x = v & 0x1fffffu;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

// Exact octant digits from the float64 centre chain (cpp/nbody.cpp:80, :92-96, :135-139).
// Levels 1..21 -> k0, 22..42 -> k1, 43..48 -> k2 (each left-aligned in its word).
__device__ void exact_keys(double x, double y, double z, const RootBox& R, int levels,
                           uint64_t& k0, uint64_t& k1, uint64_t& k2) {
    double cx = R.c[0], cy = R.c[1], cz = R.c[2], h = R.half;
    k0 = k1 = k2 = 0;
    for (int l = 1; l <= levels; ++l) {
        h = 0.5 * h;
        const unsigned o = unsigned(x > cx) | (unsigned(y > cy) << 1) | (unsigned(z > cz) << 2);
        cx = __dadd_rn(cx, (o & 1) ? h : -h);
        cy = __dadd_rn(cy, (o & 2) ? h : -h);
        cz = __dadd_rn(cz, (o & 4) ? h : -h);
        if (l <= 21)
            k0 = (k0 << 3) | o;
        else if (l <= 42)
            k1 = (k1 << 3) | o;
        else
            k2 = (k2 << 3) | o;
    }
    if (levels < 21) k0 <<= 3 * (21 - levels);
}

// Grid cell of coordinate a on the 2^21 grid, when the position lies at least `margin` grid
// units from every cell wall (else the exact path decides). 32.32 fixed point: u = (x - lo) *
// inv_w * 2^32 (the same rounding as without the 2^32), truncated; the integer part is the
// cell, the fraction is tested against a window no wider than [margin, 1 - margin]. One float64
// subtract, multiply and conversion per coordinate; the tests are integer.
__device__ __forceinline__ bool grid_coord(double x, int a, const RootBox& R, uint32_t& ic) {
    const double u = __dmul_rn(__dsub_rn(x, R.lo[a]), R.inv_w32);
    const long long ub = __double_as_longlong(u);
    if (ub < 0 || ub >= 0x4340000000000000LL) return false;  // outside [0, 2^53) (or NaN)
    const unsigned long long q = __double2ull_rz(u);
    ic = uint32_t(q >> 32);
    const uint32_t fr = uint32_t(q);
    return ic < 2097152u && fr >= R.m_lo && fr <= R.m_hi;
}

__global__ void k_keys(const double* __restrict__ pos, int n, const RootBox* __restrict__ rootp,
                       uint64_t* __restrict__ key, int* __restrict__ perm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const RootBox R = *rootp;
    const double x = pos[3 * size_t(i)], y = pos[3 * size_t(i) + 1], z = pos[3 * size_t(i) + 2];
    uint32_t ix, iy, iz;
    uint64_t k;
    if (grid_coord(x, 0, R, ix) && grid_coord(y, 1, R, iy) && grid_coord(z, 2, R, iz)) {
        k = part1by2(ix) | (part1by2(iy) << 1) | (part1by2(iz) << 2);
    } else {
        uint64_t k1, k2;
        exact_keys(x, y, z, R, 21, k, k1, k2);
    }
    key[i] = k;
    perm[i] = i;
}

// ---------------------------------------------------------------------------- prefixes

struct KeyView {
    const uint64_t* k0;
    const uint64_t* k1;  // null unless some level-21 cell holds > 8 particles
    const uint64_t* k2;
};

// Number of leading octree levels shared by sorted positions i and j (0..48).
__device__ __forceinline__ int cpl(const KeyView& K, int i, int j) {
    uint64_t a = K.k0[i], b = K.k0[j];
    if (a != b) return (__clzll(a ^ b) - 1) / 3;
    if (!K.k1) return 21;
    a = K.k1[i];
    b = K.k1[j];
    if (a != b) return 21 + (__clzll(a ^ b) - 1) / 3;
    a = K.k2[i];
    b = K.k2[j];
    if (a != b) return 42 + (__clzll(a ^ b) - 46) / 3;
    return 48;
}

__device__ __forceinline__ int digit(const KeyView& K, int i, int l) {
    if (l <= 21) return int((K.k0[i] >> (3 * (21 - l))) & 7);
    if (l <= 42) return int((K.k1[i] >> (3 * (42 - l))) & 7);
    return int((K.k2[i] >> (3 * (48 - l))) & 7);
}

// cpl9[i] = common prefix of positions i and i + L (L = leaf capacity): a cell holding both
// holds L + 1 particles and must split
__global__ void k_cpl9(KeyView K, int n, int8_t* __restrict__ cpl9, TreeCounts* cnt, int L) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = -1;
    if (i + L < n) c = cpl(K, i, i + L);
    if (c == 21 && !K.k1) cnt->deep = 1;
    cpl9[i] = int8_t(c);
}

__global__ void k_nstart(KeyView K, int n, const int8_t* __restrict__ cpl9, int8_t* __restrict__ ldepth,
                         int8_t* __restrict__ dsplit, int* __restrict__ nstart, int L) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int m = -1;
    for (int j = max(0, i - L); j <= i; ++j) m = max(m, int(cpl9[j]));
    const int ld = min(kDepthMax, m + 1);
    const int ds = i == 0 ? 0 : cpl(K, i - 1, i) + 1;
    ldepth[i] = int8_t(ld);
    dsplit[i] = int8_t(min(ds, 127));
    nstart[i] = max(0, ld - ds + 1);
}

// first j > i with j == n or cpl(i, j) < d
__device__ int run_end(const KeyView& K, int n, int i, int d) {
    if (d == 0) return n;
    int j = i + 1;
    for (int t = 0; t < 9 && j < n; ++t, ++j)
        if (cpl(K, i, j) < d) return j;
    if (j >= n) return n;
    int lo = j, step = 16, hi;
    for (;;) {
        hi = lo + step;
        if (hi >= n) {
            hi = n;
            break;
        }
        if (cpl(K, i, hi) < d) break;
        lo = hi + 1;
        step *= 2;
    }
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (cpl(K, i, mid) < d)
            hi = mid;
        else
            lo = mid + 1;
    }
    return lo;
}

// first j <= i with cpl(j, i) >= lev
__device__ int run_begin(const KeyView& K, int i, int lev) {
    int hi = i, step = 1, lo;
    for (;;) {
        lo = hi - step;
        if (lo < 0) {
            lo = -1;
            break;
        }
        if (cpl(K, lo, i) < lev) break;
        hi = lo;
        step *= 2;
    }
    int a = lo + 1, b = hi;
    while (a < b) {
        const int mid = (a + b) >> 1;
        if (cpl(K, mid, i) >= lev)
            b = mid;
        else
            a = mid + 1;
    }
    return b;
}

// ---------------------------------------------------------------------------- emit

// Node emission, one thread per node. Position i starts the nodes of depths ds[i] .. ld[i]
// (ids nbase[i] ..); k_node_owner writes, for every node id, the position that starts it, and
// k_emit fills the node: the cube centre by the float64 halving chain from the root along
// i's octant digits (cpp/nbody.cpp:92-96), the particle range [i, end) with end the first
// position whose prefix leaves the node's, `next` = the first node starting at end, the leaf
// flag and the parent (the previous node of the chain, or the deepest node at depth d - 1 of
// the run containing i). Threads of consecutive ids take chains of similar depth, so a warp
// keeps most lanes busy (one thread per starting position left 5 of 32 busy).
__global__ void k_node_owner(int n, const int* __restrict__ nstart, const int* __restrict__ nbase,
                             int* __restrict__ owner, int cap) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = nstart[i], b = nbase[i];
    for (int t = 0; t < c && b + t < cap; ++t) owner[b + t] = i;
}

__global__ void k_emit(KeyView K, int n, int span, const RootBox* __restrict__ rootp,
                       const int8_t* __restrict__ ldepth, const int8_t* __restrict__ dsplit,
                       const int* __restrict__ nbase, const int* __restrict__ owner,
                       const TreeCounts* __restrict__ cnt, int4* __restrict__ n_i4,
                       double4* __restrict__ n_cd, float4* __restrict__ n_geo,
                       int* __restrict__ n_parent, int cap) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    const int total = cnt->total_nodes;
    if (id >= span || id >= total || id >= cap) return;  // past cap: reported by k_node_cap_check
    const int i = owner[id];
    const int ds = dsplit[i], ld = ldepth[i];
    const int d = ds + (id - nbase[i]);
    const RootBox R = *rootp;
    double c[3] = {R.c[0], R.c[1], R.c[2]};
    double h = R.half;
    for (int l = 1; l <= d; ++l) {
        h = 0.5 * h;
        const int o = digit(K, i, l);
        c[0] = __dadd_rn(c[0], (o & 1) ? h : -h);
        c[1] = __dadd_rn(c[1], (o & 2) ? h : -h);
        c[2] = __dadd_rn(c[2], (o & 4) ? h : -h);
    }
    const int end = run_end(K, n, i, d);
    const int next = end < n ? nbase[end] : total;
    int parent;
    if (d == 0) {
        parent = -1;
    } else if (d > ds) {
        parent = id - 1;
    } else {
        const int s = run_begin(K, i, d - 1);
        parent = nbase[s] + (d - 1 - dsplit[s]);
    }
    n_i4[id] = make_int4(i, end - i, next, (d == ld ? 1 : 0) | (d << 8));
    n_cd[id] = make_double4(c[0], c[1], c[2], h);
    n_geo[id] = make_float4(float(c[0]), float(c[1]), float(c[2]), float(h));
    n_parent[id] = parent;
}

__global__ void k_node_cap_check(TreeCounts* cnt, int cap, uint32_t* status) {
    if (cnt->total_nodes > cap) {
        raise_status(status, GF_ERR_CAPACITY);
        cnt->total_nodes = 0;
    }
}

// Node kernels: launched over [0, span); the live node count is *nn_dev.
__device__ __forceinline__ int live_nodes(int span, const int* nn_dev) {
    return nn_dev ? min(span, *nn_dev) : span;
}

// Child count of every node and its children's ids in octant order (kids[8k .. 8k + nchild)),
// so that the bottom-up passes load a node's children together.
__global__ void k_nchild(int span, const int* __restrict__ nn_dev, const int4* __restrict__ n_i4,
                         int* __restrict__ nchild, int* __restrict__ counter, int* __restrict__ kids) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= live_nodes(span, nn_dev)) return;
    const int4 q = n_i4[k];
    int c = 0;
    if (!(q.w & 1)) {
        for (int ch = k + 1; ch < q.z && c < 8; ch = n_i4[ch].z) kids[8 * size_t(k) + c++] = ch;  // <= 8 children
    }
    nchild[k] = c;
    counter[k] = 0;
}

// Inside a leaf the reference keeps increasing particle index (stable partitions).
__global__ void k_leaf_sort(int span, const int* __restrict__ nn_dev, const int4* __restrict__ n_i4,
                            int* __restrict__ perm) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= live_nodes(span, nn_dev)) return;
    const int4 q = n_i4[k];
    if (!(q.w & 1) || q.y > 64) return;  // larger leaves hold identical keys: already sorted
    int* p = perm + q.x;
    for (int a = 1; a < q.y; ++a) {
        const int v = p[a];
        int b = a - 1;
        while (b >= 0 && p[b] > v) {
            p[b + 1] = p[b];
            --b;
        }
        p[b + 1] = v;
    }
}

// Positions (and masses) in tree order: p4 = float32 position and mass, plo = the float32
// remainders. The build saves the float64 positions in tree order (xsave); a refit measures each
// particle's displacement since the build against them (xbuild, tree order: coalesced reads).
__global__ void k_gather(int n, const int* __restrict__ perm, const double* __restrict__ pos,
                         const double* __restrict__ mass, const double* __restrict__ xbuild,
                         float4* __restrict__ p4, float* __restrict__ pdisp, float4* __restrict__ plo,
                         int disp32 = 0, double* __restrict__ xsave = nullptr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int j = perm[i];
    const double x = pos[3 * size_t(j)], y = pos[3 * size_t(j) + 1], z = pos[3 * size_t(j) + 2];
    const double m = mass ? mass[j] : 1.0;
    const float fx = float(x), fy = float(y), fz = float(z);
    p4[i] = make_float4(fx, fy, fz, float(m));
    if (plo) plo[i] = make_float4(float(x - double(fx)), float(y - double(fy)), float(z - double(fz)), 0.f);
    if (xsave) {
        xsave[3 * size_t(i)] = x;
        xsave[3 * size_t(i) + 1] = y;
        xsave[3 * size_t(i) + 2] = z;
    }
    if (pdisp && disp32) {  // mixed form: float64 differences, float32 length
        const float dx = float(x - xbuild[3 * size_t(i)]), dy = float(y - xbuild[3 * size_t(i) + 1]),
                    dz = float(z - xbuild[3 * size_t(i) + 2]);
        pdisp[i] = m > 0 ? sqrtf(dx * dx + dy * dy + dz * dz) : 0.0f;
    } else if (pdisp) {  // refit: displacement since the build (cpp/nbody.cpp:273-275)
        const double dx = __dsub_rn(x, xbuild[3 * size_t(i)]);
        const double dy = __dsub_rn(y, xbuild[3 * size_t(i) + 1]);
        const double dz = __dsub_rn(z, xbuild[3 * size_t(i) + 2]);
        pdisp[i] = m > 0 ? float(__dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)),
                                                      __dmul_rn(dz, dz))))
                         : 0.0f;
    }
}

// ---------------------------------------------------------------------------- moments

struct MomentArgs {
    int nn;
    const int* nn_dev;  // when set: node count read on the device
    bool refit;
    float theta;
    const int4* n_i4;
    const int* parent;
    const int* nchild;
    const int* kids;    // children in octant order, 8 slots per node
    int* counter;
    const double4* n_cd;  // build: float64 centre + half
    const float4* n_geo;  // refit: float32 centre + half
    float4* mom;
    float* open_r;
    float* ndisp;
    // leaf inputs
    const int* perm;
    const double* pos;
    const double* mass;
    const float4* p4;
    const float* pdisp;
};

__device__ __forceinline__ void finalize(const MomentArgs& A, int k, double M, double sx, double sy,
                                         double sz, float dm) {
    const double inv = M > 0 ? __ddiv_rn(1.0, M) : 0.0;
    const double mx = __dmul_rn(sx, inv), my = __dmul_rn(sy, inv), mz = __dmul_rn(sz, inv);
    A.mom[k] = make_float4(float(mx), float(my), float(mz), float(M));
    double ox, oy, oz, first;
    if (!A.refit) {  // cpp/nbody.cpp:104-106
        const double4 c = A.n_cd[k];
        ox = __dsub_rn(mx, c.x);
        oy = __dsub_rn(my, c.y);
        oz = __dsub_rn(mz, c.z);
        first = __ddiv_rn(__dmul_rn(2.0, c.w), double(A.theta));
    } else {  // cpp/nbody.cpp:301-303: the first term is evaluated in float32
        const float4 g = A.n_geo[k];
        ox = __dsub_rn(mx, double(g.x));
        oy = __dsub_rn(my, double(g.y));
        oz = __dsub_rn(mz, double(g.z));
        first = double(__fdiv_rn(__fmul_rn(2.0f, __fadd_rn(g.w, dm)), A.theta));
        A.ndisp[k] = dm;
    }
    const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(ox, ox), __dmul_rn(oy, oy)), __dmul_rn(oz, oz)));
    A.open_r[k] = float(__dadd_rn(first, r));
}

__global__ void k_moments(MomentArgs A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= live_nodes(A.nn, A.nn_dev)) return;
    const int4 q = A.n_i4[k];
    if (!(q.w & 1)) return;
    double M = 0, sx = 0, sy = 0, sz = 0;
    float dm = 0.f;
    if (q.y <= kLeafMax) {  // the leaf's particles loaded together, summed in order
        double4 pm[kLeafMax];
        float pd[kLeafMax];
#pragma unroll
        for (int t = 0; t < kLeafMax; ++t) {
            pm[t] = make_double4(0.0, 0.0, 0.0, 0.0);
            pd[t] = 0.f;
            if (t < q.y) {
                const int i = q.x + t;
                if (!A.refit) {
                    const int j = A.perm[i];
                    pm[t] = make_double4(A.pos[3 * size_t(j)], A.pos[3 * size_t(j) + 1], A.pos[3 * size_t(j) + 2],
                                         A.mass ? A.mass[j] : 1.0);
                } else {
                    const float4 p = A.p4[i];
                    pm[t] = make_double4(double(p.x), double(p.y), double(p.z), double(p.w));
                    pd[t] = A.pdisp[i];
                }
            }
        }
#pragma unroll
        for (int t = 0; t < kLeafMax; ++t) {
            if (t < q.y) {  // cpp/nbody.cpp:124-131 (build), :285-289 (refit: float x float exact)
                const double m = pm[t].w;
                M = __dadd_rn(M, m);
                sx = __dadd_rn(sx, __dmul_rn(m, pm[t].x));
                sy = __dadd_rn(sy, __dmul_rn(m, pm[t].y));
                sz = __dadd_rn(sz, __dmul_rn(m, pm[t].z));
                dm = fmaxf(dm, pd[t]);
            }
        }
    } else
    for (int i = q.x; i < q.x + q.y; ++i) {
        if (!A.refit) {  // cpp/nbody.cpp:124-131
            const int j = A.perm[i];
            const double m = A.mass ? A.mass[j] : 1.0;
            M = __dadd_rn(M, m);
            sx = __dadd_rn(sx, __dmul_rn(m, A.pos[3 * size_t(j)]));
            sy = __dadd_rn(sy, __dmul_rn(m, A.pos[3 * size_t(j) + 1]));
            sz = __dadd_rn(sz, __dmul_rn(m, A.pos[3 * size_t(j) + 2]));
        } else {  // cpp/nbody.cpp:285-289 (float x float products are exact in float64)
            const float4 p = A.p4[i];
            const double m = double(p.w);
            M = __dadd_rn(M, m);
            sx = __dadd_rn(sx, m * double(p.x));
            sy = __dadd_rn(sy, m * double(p.y));
            sz = __dadd_rn(sz, m * double(p.z));
            dm = fmaxf(dm, A.pdisp[i]);
        }
    }
    finalize(A, k, M, sx, sy, sz, dm);
    __threadfence();
    int p = A.parent[k];
    while (p >= 0) {
        const int arrived = atomicAdd(&A.counter[p], 1);
        if (arrived != A.nchild[p] - 1) return;
        __threadfence();
        double PM = 0, px = 0, py = 0, pz = 0;
        float pd = 0.f;
        const int nc = A.nchild[p];
        float4 cms[8];
        float cds[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) {  // the children's records in flight together
            cms[c] = make_float4(0.f, 0.f, 0.f, 0.f);
            cds[c] = 0.f;
            if (c < nc) {
                const int ch = A.kids[8 * size_t(p) + c];
                cms[c] = __ldcg(&A.mom[ch]);
                if (A.refit) cds[c] = __ldcg(&A.ndisp[ch]);
            }
        }
#pragma unroll
        for (int c = 0; c < 8; ++c) {  // octant order
            if (c < nc) {
                const double m = double(cms[c].w);
                PM = __dadd_rn(PM, m);
                px = __dadd_rn(px, m * double(cms[c].x));
                py = __dadd_rn(py, m * double(cms[c].y));
                pz = __dadd_rn(pz, m * double(cms[c].z));
                pd = fmaxf(pd, cds[c]);
            }
        }
        finalize(A, p, PM, px, py, pz, pd);
        __threadfence();
        p = A.parent[p];
    }
}

// Relative opening radius of a quadrupole node: the walk accepts the node for a group sphere
// (centre c, radius R) when |com - c| - R exceeds rho * (alpha * min |a_old|)^(-1/5), i.e. when
// the octupole-order estimate M b^3 / r^5 of the truncation error is at most alpha times the
// group's smallest previous acceleration (the relative criterion of Springel 2005, GADGET-2,
// to the next order). b bounds the distance of the node's mass from its centre of mass.
// rho = M^(1/5) b^(3/5) in logarithms, so no intermediate overflows in float32. The second
// radius, (M b^2)^(1/4), is the quadrupole-order one: beyond rho_q (alpha_q a_min)^(-1/4) the
// node's quadrupole term itself is below alpha_q a_min and the walk takes its monopole alone.
__device__ __forceinline__ float2 rel_radii(float m, float ox, float oy, float oz, float half) {
    if (!(m > 0.f)) return make_float2(0.f, 0.f);
    const float lm = log2f(m), lb = log2f(sqrtf(ox * ox + oy * oy + oz * oz) + 1.7320508f * half);
    return make_float2(exp2f(0.2f * lm + 0.6f * lb), exp2f(0.25f * lm + 0.5f * lb));
}

// Traceless quadrupole Q = sum m (3 d d - |d|^2 I) and trace T = sum m |d|^2 about a centre.
struct QuadSum {
    KahanF xx, yy, xy, xz, yz, tr;
    __device__ __forceinline__ void point(float m, float dx, float dy, float dz) {
        const float r2 = dx * dx + dy * dy + dz * dz;
        xx.add(m * (3.f * dx * dx - r2));
        yy.add(m * (3.f * dy * dy - r2));
        xy.add(3.f * m * dx * dy);
        xz.add(3.f * m * dx * dz);
        yz.add(3.f * m * dy * dz);
        tr.add(m * r2);
    }
};

// Mixed form: monopole and traceless quadrupole in one bottom-up pass, float32 with
// Kahan-compensated sums, directly in the breadth-first walk layout (the children of a node
// are contiguous there, in octant order, so a parent reads them with independent loads). A
// leaf sums its particles; the last child to finish a parent (arrival counter) combines the
// children's masses and centres, then their quadrupoles shifted by the parallel-axis term.
// open_r = 2 (half + displacement) / theta + |com - cell centre| in float32, and the relative
// opening radii. Used by the build (pdisp null: no displacement) and by the refit (pdisp: the
// displacement of each particle since the build). Thread per breadth-first node.
struct RefitBfsArgs {
    int span;
    const int* nn_dev;
    float theta;
    const int* wparent;
    const float4* wgeo;
    int* counter;
    float4* wa;   // com, m
    float4* wb;   // open_r, first, code, rho
    float4* wq;   // Qxx, Qyy, Qxy, Qxz
    float2* wt;   // Qyz, T
    float* wrq;   // quadrupole-order radius
    float* ndisp; // breadth-first
    const float4* p4;
    const float* pdisp;  // null: no displacement (the build)
};

// Writes node b's monopole, opening radii and displacement bound (g: its cell, loaded early).
__device__ __forceinline__ void finalize_bfs(const RefitBfsArgs& A, int b, const float4 g, float m, float cx,
                                             float cy, float cz, float dm) {
    A.wa[b] = make_float4(cx, cy, cz, m);
    const float ox = cx - g.x, oy = cy - g.y, oz = cz - g.z;
    A.wb[b].x = 2.f * (g.w + dm) / A.theta + sqrtf(ox * ox + oy * oy + oz * oz);
    const float2 rr = rel_radii(m, ox, oy, oz, g.w + dm);
    A.wb[b].w = rr.x;
    A.wrq[b] = rr.y;
    A.ndisp[b] = dm;
}

__device__ __forceinline__ float4 leaf_centre(const KahanF& M, const KahanF& sx, const KahanF& sy, const KahanF& sz) {
    const float inv = M.s > 0.f ? 1.f / M.s : 0.f;
    return make_float4(sx.s * inv, sy.s * inv, sz.s * inv, M.s);
}

// Compensated sum over the 8 lanes of an aligned lane group (all 32 lanes take part): Knuth's
// two-sum at each of the three butterfly steps, the rounding errors carried in a second float.
// Both lanes of a pair compute the same bits, so the 8 lanes end with identical values.
__device__ __forceinline__ float group8_sum(float v) {
    float s = v, e = 0.f;
#pragma unroll
    for (int off = 4; off; off >>= 1) {
        const float o = __shfl_xor_sync(0xffffffffu, s, off);
        const float oe = __shfl_xor_sync(0xffffffffu, e, off);
        const float t = s + o;
        const float bp = t - s;
        const float err = (s - (t - bp)) + (o - bp);
        s = t;
        e = (e + oe) + err;
    }
    return s + e;
}

__device__ __forceinline__ float group8_max(float v) {
#pragma unroll
    for (int off = 4; off; off >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, off));
    return v;
}

// The arrival of a finished node at its parent p (child range c0, nc: structure fields, loaded
// before the atomic). The counter is an acquire-release atomic: it publishes this thread's
// records of the node and, for the last child, makes its siblings' records visible. Returns
// whether this arrival completed p.
__device__ __forceinline__ bool arrive(const RefitBfsArgs& A, int p, int nc) {
    return atom_add_acq_rel(&A.counter[p], 1) == nc - 1;
}

// Threads take the nodes from the end of the breadth-first layout (the deepest first), so the
// deep subtrees are summed and climbed by the first blocks and the last blocks hold the shallow
// nodes, whose climbs to the root are short. A leaf's thread sums its particles (sequential
// Kahan sums); a parent is combined by a group of 8 lanes of the warp whose lane completed it,
// lane c loading child c, so that all of a parent's records arrive with one memory latency and
// the sums are pairwise with compensation. 64 registers: 4 blocks per SM.
__global__ void __launch_bounds__(kThreads, 4) k_refit_bfs_quad32(RefitBfsArgs A) {
    const int b = live_nodes(A.span, A.nn_dev) - 1 - int(blockIdx.x * blockDim.x + threadIdx.x);
    const int lane = threadIdx.x & 31;
    int p = -1, pc0 = 0, pnc = 0;  // a parent that this lane's arrival completed, its child range
    const float4 wb = b >= 0 ? A.wb[b] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int first = __float_as_int(wb.y), code = __float_as_int(wb.z);
    if (b >= 0 && code < 0) {  // a leaf (internal nodes are reached by the climb)
        const int cnt = -code;
        const float4 g = __ldg(&A.wgeo[b]);
        const int par = __ldg(&A.wparent[b]);
        int c0 = 0, nc = 0;
        if (par >= 0) {
            const int* pbi = reinterpret_cast<const int*>(A.wb) + 4 * size_t(par);
            c0 = __ldg(pbi + 1);
            nc = __ldg(pbi + 2);
        }
        QuadSum S;
        if (cnt <= kLeafMax) {  // the leaf's particles loaded once, together (one memory latency)
            float4 pp[kLeafMax];
            float pd[kLeafMax];
#pragma unroll
            for (int t = 0; t < kLeafMax; ++t) {
                pp[t] = t < cnt ? A.p4[first + t] : make_float4(0.f, 0.f, 0.f, 0.f);
                pd[t] = t < cnt && A.pdisp ? A.pdisp[first + t] : 0.f;
            }
            KahanF M, sx, sy, sz;
            float dm = 0.f;
#pragma unroll
            for (int t = 0; t < kLeafMax; ++t) {
                if (t < cnt) {
                    M.add(pp[t].w);
                    sx.add(pp[t].w * pp[t].x);
                    sy.add(pp[t].w * pp[t].y);
                    sz.add(pp[t].w * pp[t].z);
                    dm = fmaxf(dm, pd[t]);
                }
            }
            const float4 c = leaf_centre(M, sx, sy, sz);
            finalize_bfs(A, b, g, c.w, c.x, c.y, c.z, dm);
#pragma unroll
            for (int t = 0; t < kLeafMax; ++t)
                if (t < cnt) S.point(pp[t].w, pp[t].x - c.x, pp[t].y - c.y, pp[t].z - c.z);
        } else {  // depth-48 leaves of coincident points
            KahanF M, sx, sy, sz;
            float dm = 0.f;
            for (int i = first; i < first + cnt; ++i) {
                const float4 q = A.p4[i];
                M.add(q.w);
                sx.add(q.w * q.x);
                sy.add(q.w * q.y);
                sz.add(q.w * q.z);
                if (A.pdisp) dm = fmaxf(dm, A.pdisp[i]);
            }
            const float4 c = leaf_centre(M, sx, sy, sz);
            finalize_bfs(A, b, g, c.w, c.x, c.y, c.z, dm);
            for (int i = first; i < first + cnt; ++i) {
                const float4 q = A.p4[i];
                S.point(q.w, q.x - c.x, q.y - c.y, q.z - c.z);
            }
        }
        A.wq[b] = make_float4(S.xx.s, S.yy.s, S.xy.s, S.xz.s);
        A.wt[b] = make_float2(S.yz.s, S.tr.s);
        if (par >= 0 && arrive(A, par, nc)) {
            p = par;
            pc0 = c0;
            pnc = nc;
        }
    }
    // Climb. Each round the four groups of 8 lanes take up to four of the warp's completed
    // parents (group k the one held by the k-th lane holding one); the group's lane 0 writes
    // the parent and arrives at the grandparent, and a completed grandparent goes back to the
    // lane that held the parent. Each round serves at least one parent and a parent precedes
    // its children in the layout, so the loop ends.
    const int grp = lane >> 3, c = lane & 7;
    for (;;) {
        const unsigned pend = __ballot_sync(0xffffffffu, p >= 0);
        if (pend == 0u) break;
        unsigned rest = pend;  // the holders from the grp-th on (lowest lanes first)
        for (int k = 0; k < grp; ++k) rest &= rest - 1u;
        const int src = rest ? __ffs(int(rest)) - 1 : 0;
        int q = __shfl_sync(0xffffffffu, p, src);
        const int q0 = __shfl_sync(0xffffffffu, pc0, src);
        const int qn = __shfl_sync(0xffffffffu, pnc, src);
        if (!rest) q = -1;
        __syncwarp();  // orders the holder's acquiring arrival before its group's loads
        float4 cm = make_float4(0.f, 0.f, 0.f, 0.f), qc = cm, g = cm;
        float2 yt = make_float2(0.f, 0.f);
        float dmc = 0.f;
        int gp = -1, gc0 = 0, gnc = 0;
        if (q >= 0) {
            if (c < qn) {
                cm = __ldcg(&A.wa[q0 + c]);
                dmc = __ldcg(&A.ndisp[q0 + c]);
                qc = __ldcg(&A.wq[q0 + c]);
                yt = __ldcg(&A.wt[q0 + c]);
            }
            if (c == 0) {
                g = __ldg(&A.wgeo[q]);
                gp = __ldg(&A.wparent[q]);
                if (gp >= 0) {
                    const int* pbi = reinterpret_cast<const int*>(A.wb) + 4 * size_t(gp);
                    gc0 = __ldg(pbi + 1);
                    gnc = __ldg(pbi + 2);
                }
            }
        }
        // children past qn (and groups without a parent) add zeros
        const float M = group8_sum(cm.w);
        const float sx = group8_sum(cm.w * cm.x), sy = group8_sum(cm.w * cm.y), sz = group8_sum(cm.w * cm.z);
        const float dm = group8_max(dmc);
        const float inv = M > 0.f ? 1.f / M : 0.f;
        const float cx = sx * inv, cy = sy * inv, cz = sz * inv;
        const float dx = cm.x - cx, dy = cm.y - cy, dz = cm.z - cz;
        const float r2 = dx * dx + dy * dy + dz * dz, m = cm.w;
        const float xx = group8_sum(qc.x + m * (3.f * dx * dx - r2));
        const float yy = group8_sum(qc.y + m * (3.f * dy * dy - r2));
        const float xy = group8_sum(qc.z + 3.f * m * dx * dy);
        const float xz = group8_sum(qc.w + 3.f * m * dx * dz);
        const float yz = group8_sum(yt.x + 3.f * m * dy * dz);
        const float tr = group8_sum(yt.y + m * r2);
        int np = -1;
        if (q >= 0 && c == 0) {
            finalize_bfs(A, q, g, M, cx, cy, cz, dm);
            A.wq[q] = make_float4(xx, yy, xy, xz);
            A.wt[q] = make_float2(yz, tr);
            if (gp >= 0 && arrive(A, gp, gnc)) np = gp;
        }
        // back to the holders: the k-th holder (k < 4) was served by group k
        const int rank = __popc(pend & lanemask_lt());
        const int from = 8 * min(rank, 3);
        const int np_ = __shfl_sync(0xffffffffu, np, from);
        const int nc0_ = __shfl_sync(0xffffffffu, gc0, from);
        const int nnc_ = __shfl_sync(0xffffffffu, gnc, from);
        if (p >= 0 && rank < 4) {
            p = np_;
            pc0 = nc0_;
            pnc = nnc_;
        }
    }
}

// ---------------------------------------------------------------------------- groups + layout

__global__ void k_group_flag(int span, const int* __restrict__ nn_dev, int gmax, const int4* __restrict__ n_i4,
                             const int* __restrict__ parent, int* __restrict__ flag) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= span) return;
    if (k >= live_nodes(span, nn_dev)) {  // past the live nodes: no group (the scan covers span)
        flag[k] = 0;
        return;
    }
    const int4 q = n_i4[k];
    const bool candidate = q.y <= gmax || (q.w & 1);
    const int p = parent[k];
    flag[k] = candidate && (p < 0 || n_i4[p].y > gmax) ? 1 : 0;
}

__global__ void k_group_write(int span, const int* __restrict__ nn_dev, const int* __restrict__ flag,
                              const int* __restrict__ scan, int* __restrict__ groups) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= live_nodes(span, nn_dev)) return;
    if (flag[k]) groups[scan[k]] = k;
}

// breadth-first order = stable sort by depth; slots past the live nodes sort last
__global__ void k_bfs_keys(int span, const int* __restrict__ nn_dev, const int4* __restrict__ n_i4,
                           uint64_t* __restrict__ key, int* __restrict__ val) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= span) return;
    key[k] = k < live_nodes(span, nn_dev) ? uint64_t(n_i4[k].w >> 8) : 255u;
    val[k] = k;
}

__global__ void k_bfs_index(int span, const int* __restrict__ nn_dev, const int* __restrict__ val,
                            int* __restrict__ bfs) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= live_nodes(span, nn_dev)) return;
    bfs[val[b]] = b;
}

__global__ void k_walk_fill(int nn, const int4* __restrict__ n_i4, const int* __restrict__ nchild,
                            const int* __restrict__ bfs, const float4* __restrict__ mom,
                            const float* __restrict__ open_r, const float4* __restrict__ geo,
                            float4* __restrict__ wa, float4* __restrict__ wb,
                            float4* __restrict__ wgeo, int* __restrict__ leaf_of,
                            const int* __restrict__ parent, int* __restrict__ wparent, const int* __restrict__ nn_dev) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= live_nodes(nn, nn_dev)) return;
    const int4 q = n_i4[k];
    const int b = bfs[k];
    int first, code;
    if (q.w & 1) {
        first = q.x;
        code = -q.y;
        if (leaf_of)
            for (int i = q.x; i < q.x + q.y; ++i) leaf_of[i] = b;
    } else {
        first = bfs[k + 1];
        code = nchild[k];
    }
    // mom null (mixed-form build, neighbour-search trees): no moments here (the mixed form
    // writes them into this layout afterwards)
    wa[b] = mom ? mom[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    wb[b] = make_float4(mom ? open_r[k] : 0.f, __int_as_float(first), __int_as_float(code), 0.f);
    if (wgeo) wgeo[b] = geo[k];
    if (wparent) wparent[b] = parent[k] < 0 ? -1 : bfs[parent[k]];
}

// ---------------------------------------------------------------------------- deep cells

// Positions of cells that still hold > 8 particles at level 21 get extension keys.
// Extension keys are read (by cpl and digit) only at positions whose level-21 key equals a
// neighbour's in sorted order, so the others are skipped: they hold stale words that nothing
// reads. Shared positions outside deep runs get zeros.
__global__ void k_deep_keys(int n, const uint64_t* __restrict__ k0, const int* __restrict__ perm,
                            const double* __restrict__ pos, const RootBox* __restrict__ rootp,
                            uint64_t* __restrict__ k1, uint64_t* __restrict__ k2,
                            int* __restrict__ starts, int* __restrict__ nstarts, int L) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t ki = k0[i];
    if (!((i > 0 && k0[i - 1] == ki) || (i + 1 < n && k0[i + 1] == ki))) return;
    bool deep = false;
    for (int j = max(0, i - L); j <= i && !deep; ++j)
        deep = j + L < n && k0[j] == k0[j + L];
    uint64_t a = 0, b = 0;
    if (deep) {
        const RootBox R = *rootp;
        const int p = perm[i];
        uint64_t c0;
        exact_keys(pos[3 * size_t(p)], pos[3 * size_t(p) + 1], pos[3 * size_t(p) + 2], R, kDepthMax, c0, a, b);
        if (i == 0 || k0[i - 1] != k0[i]) starts[atomicAdd(nstarts, 1)] = i;
    }
    k1[i] = a;
    k2[i] = b;
}

// One block per deep run: stable sort of (k1, k2) inside the run (ties keep index order).
__global__ void k_deep_sort(int n, const uint64_t* __restrict__ k0, uint64_t* __restrict__ k1,
                            uint64_t* __restrict__ k2, int* __restrict__ perm,
                            const int* __restrict__ starts, const int* __restrict__ nstarts,
                            uint32_t* status) {
    extern __shared__ unsigned char smem[];
    uint64_t* s1 = reinterpret_cast<uint64_t*>(smem);
    uint64_t* s2 = s1 + kDeepRunMax;
    int* sp = reinterpret_cast<int*>(s2 + kDeepRunMax);
    for (int r = blockIdx.x; r < *nstarts; r += gridDim.x) {
        const int b = starts[r];
        __shared__ int s_len;
        if (threadIdx.x == 0) {
            int e = b + 1;
            while (e < n && k0[e] == k0[b]) ++e;
            s_len = e - b;
        }
        __syncthreads();
        const int len = s_len;
        if (len > kDeepRunMax) {
            // sorted already when every extension key is equal (coincident particles)
            bool sorted = true;
            for (int i = b + 1 + threadIdx.x; i < b + len; i += blockDim.x)
                if (k1[i] < k1[i - 1] || (k1[i] == k1[i - 1] && k2[i] < k2[i - 1])) sorted = false;
            if (__syncthreads_or(!sorted) && threadIdx.x == 0) raise_status(status, GF_ERR_DEEP_CELL);
            __syncthreads();
            continue;
        }
        int P = 1;
        while (P < len) P <<= 1;
        for (int t = threadIdx.x; t < P; t += blockDim.x) {
            if (t < len) {
                s1[t] = k1[b + t];
                s2[t] = k2[b + t];
                sp[t] = perm[b + t];
            } else {
                s1[t] = ~0ull;
                s2[t] = ~0ull;
                sp[t] = 0x7fffffff;
            }
        }
        __syncthreads();
        for (int size = 2; size <= P; size <<= 1) {
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int t = threadIdx.x; t < P; t += blockDim.x) {
                    const int u = t ^ stride;
                    if (u > t) {
                        const bool up = (t & size) == 0;
                        const bool gt = s1[t] > s1[u] || (s1[t] == s1[u] && (s2[t] > s2[u] ||
                                                          (s2[t] == s2[u] && sp[t] > sp[u])));
                        if (gt == up) {
                            uint64_t x = s1[t]; s1[t] = s1[u]; s1[u] = x;
                            x = s2[t]; s2[t] = s2[u]; s2[u] = x;
                            const int y = sp[t]; sp[t] = sp[u]; sp[u] = y;
                        }
                    }
                }
                __syncthreads();
            }
        }
        for (int t = threadIdx.x; t < len; t += blockDim.x) {
            k1[b + t] = s1[t];
            k2[b + t] = s2[t];
            perm[b + t] = sp[t];
        }
        __syncthreads();
    }
}

}  // namespace

// ------------------------------------------------------------------------------- host side

static Octree g_tree;
Octree& gravity_tree() { return g_tree; }
static Octree* g_last_walked = nullptr;
Octree*& last_walked() { return g_last_walked; }

void Octree::reserve_graph_build() {
    if (!valid || n <= 0) throw Error(GF_ERR_ARG, "a captured rebuild needs a regular build first");
    key1.get<uint64_t>(n);
    key2.get<uint64_t>(n);
    pdisp.get<float>(n);
    node_owner.get<int>(node_cap);
    work.get<int4>(std::max(size_t(node_cap), size_t(n)) + 1);
    sphere.get<float4>(std::max(size_t(node_cap), size_t(n)) + 1);
    if (quad) item_gam.get<float2>(std::max(size_t(node_cap), size_t(n)) + 1);
    gweight.get<int>(std::max(node_cap, 1));
    reserve_scan_sort(std::max(n, node_cap), &scratch);
    deep_sort_attr();
}

void Octree::deep_sort_attr() {
    static bool attr = false;
    if (!attr) {
        const size_t sm = size_t(kDeepRunMax) * (2 * sizeof(uint64_t) + sizeof(int));
        GF_CUDA(cudaFuncSetAttribute(k_deep_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm)));
        attr = true;
    }
}

void Octree::build(int n_, const double* pos, const double* mass, double theta, cudaStream_t s, bool graph_safe) {
    Context& C = ctx();
    ProfScope ps(want_knn ? kStKnnTree : kStTreeBuild, s);
    if (graph_safe && (!valid || n != n_ || node_cap <= 0))
        throw Error(GF_ERR_ARG, "a captured rebuild needs a regular build of the same particle set first");
    n = n_;
    theta_f = float(theta);
    if (!graph_safe) valid = false;
    if (!h_counts) GF_CUDA(cudaMallocHost(&h_counts, sizeof(TreeCounts)));
    TreeCounts* cnt = counts.get<TreeCounts>(1);
    RootBox* R = root.get<RootBox>(1);
    GF_CUDA(cudaMemsetAsync(cnt, 0, sizeof(TreeCounts), s));

    const int grid = div_up(n, kThreads);
    const int nparts = std::min(4 * C.sms, std::max(1, grid));
    int* nb = nbase.get<int>(std::max(size_t(n) + 1, size_t(nparts) * 14 + 16));
    double* part = reinterpret_cast<double*>(nb);  // bbox partials, consumed before the scan
    k_bbox<<<nparts, kThreads, 0, s>>>(pos, n, part, R, C.d_status, &cnt->bbox_done);
    GF_CHECK_LAUNCH();

    uint64_t* k0 = key.get<uint64_t>(n);
    int* pm = perm.get<int>(n);
    k_keys<<<grid, kThreads, 0, s>>>(pos, n, R, k0, pm);
    GF_CHECK_LAUNCH();
    {
        ProfScope pso(want_knn ? kStCount : kStTreeSort, s);
        radix_sort_pairs(k0, pm, key_alt.get<uint64_t>(n), perm_alt.get<int>(n), n, 0, 63, s, &scratch);
    }

    int8_t* c9 = cpl9.get<int8_t>(n);
    int8_t* ld = ldepth.get<int8_t>(n);
    int8_t* ds = dsplit.get<int8_t>(n);
    int* ns = nstart.get<int>(n);
    KeyView K{k0, nullptr, nullptr};
    // Deep cells (> 8 particles in one level-21 cell) need extension keys. A regular build
    // finds out on the host; a captured one always computes them (zero outside deep runs,
    // where they leave every common-prefix length the tree uses unchanged).
    bool deep = graph_safe;
    if (!graph_safe) {
        k_cpl9<<<grid, kThreads, 0, s>>>(K, n, c9, cnt, leaf_max);
        GF_CHECK_LAUNCH();
        k_nstart<<<grid, kThreads, 0, s>>>(K, n, c9, ld, ds, ns, leaf_max);
        GF_CHECK_LAUNCH();
        exclusive_scan(ns, nb, n, &cnt->total_nodes, s, &scratch);
        GF_CUDA(cudaMemcpyAsync(h_counts, cnt, sizeof(TreeCounts), cudaMemcpyDeviceToHost, s));
        GF_CUDA(cudaStreamSynchronize(s));
        deep = h_counts->deep != 0;
    }
    if (deep) {
        uint64_t* e1 = key1.get<uint64_t>(n);
        uint64_t* e2 = key2.get<uint64_t>(n);
        int* starts = reinterpret_cast<int*>(key_alt.get<uint64_t>(n));  // scratch
        int* nst = &cnt->deep_runs;
        k_deep_keys<<<grid, kThreads, 0, s>>>(n, k0, pm, pos, R, e1, e2, starts, nst, leaf_max);
        GF_CHECK_LAUNCH();
        deep_sort_attr();
        const size_t sm = size_t(kDeepRunMax) * (2 * sizeof(uint64_t) + sizeof(int));
        k_deep_sort<<<2 * C.sms, 512, sm, s>>>(n, k0, e1, e2, pm, starts, nst, C.d_status);
        GF_CHECK_LAUNCH();
        K = KeyView{k0, e1, e2};
        k_cpl9<<<grid, kThreads, 0, s>>>(K, n, c9, cnt, leaf_max);
        GF_CHECK_LAUNCH();
        k_nstart<<<grid, kThreads, 0, s>>>(K, n, c9, ld, ds, ns, leaf_max);
        GF_CHECK_LAUNCH();
        exclusive_scan(ns, nb, n, &cnt->total_nodes, s, &scratch);
        if (!graph_safe) {
            GF_CUDA(cudaMemcpyAsync(h_counts, cnt, sizeof(TreeCounts), cudaMemcpyDeviceToHost, s));
            GF_CUDA(cudaStreamSynchronize(s));
        }
    }
    if (!graph_safe) {
        nn = h_counts->total_nodes;
        // headroom: later synchronisation-free rebuilds (captured or not) build inside it
        if (nn > node_cap) node_cap = nn + nn / 2 + 1024;
    }
    const int cap = node_cap;
    // node kernels cover [0, span) and read the live count on the device
    const int span = graph_safe ? cap : nn;
    const int* nn_dev = &cnt->total_nodes;
    const int ngrid = div_up(span, kThreads);

    int4* i4 = n_i4.get<int4>(cap);
    double4* cd = n_cd.get<double4>(cap);
    float4* geo = n_geo.get<float4>(cap);
    int* par = n_parent.get<int>(cap);
    {
        ProfScope pse(want_knn ? kStCount : kStTreeEmit, s);
        int* own = node_owner.get<int>(cap);
        k_node_owner<<<grid, kThreads, 0, s>>>(n, ns, nb, own, cap);
        GF_CHECK_LAUNCH();
        k_emit<<<ngrid, kThreads, 0, s>>>(K, n, span, R, ld, ds, nb, own, cnt, i4, cd, geo, par, cap);
        GF_CHECK_LAUNCH();
    }
    if (graph_safe) {  // more nodes than the buffers hold: flag, and leave an empty tree
        k_node_cap_check<<<1, 1, 0, s>>>(cnt, cap, C.d_status);
        GF_CHECK_LAUNCH();
    }
    int* nch = n_nchild.get<int>(cap);
    int* ctr = n_counter.get<int>(cap);
    int* kid = n_kids.get<int>(8 * size_t(cap));
    k_nchild<<<ngrid, kThreads, 0, s>>>(span, nn_dev, i4, nch, ctr, kid);
    GF_CHECK_LAUNCH();
    k_leaf_sort<<<ngrid, kThreads, 0, s>>>(span, nn_dev, i4, pm);
    GF_CHECK_LAUNCH();

    float4* pp = p4.get<float4>(n);
    double* xb = xbuild.get<double>(3 * size_t(n));
    k_gather<<<grid, kThreads, 0, s>>>(n, pm, pos, mass, nullptr, pp, nullptr,
                                       want_knn ? plo.get<float4>(n) : nullptr, 0, xb);
    GF_CHECK_LAUNCH();

    float4* mom = n_mom.get<float4>(cap);
    float* opr = n_open.get<float>(cap);
    float* ndp = n_disp.get<float>(cap);
    if (want_knn) {
        // a neighbour-search tree needs geometry only: no moments (the walk layout's mass and
        // opening-radius fields stay unused)
    } else if (quad) {
        // mixed form: moments in the breadth-first walk layout, after it is laid out (below)
    } else {
        MomentArgs A{};
        A.nn = span;
        A.nn_dev = nn_dev;
        A.refit = false;
        A.theta = theta_f;
        A.n_i4 = i4;
        A.parent = par;
        A.nchild = nch;
        A.kids = kid;
        A.counter = ctr;
        A.n_cd = cd;
        A.n_geo = geo;
        A.mom = mom;
        A.open_r = opr;
        A.ndisp = ndp;
        A.perm = pm;
        A.pos = pos;
        A.mass = mass;
        ProfScope psm(kStTreeMoments, s);
        k_moments<<<ngrid, kThreads, 0, s>>>(A);
        GF_CHECK_LAUNCH();
    }

    int* gf_ = gflag.get<int>(cap);
    int* gs = gscan.get<int>(cap);
    k_group_flag<<<ngrid, kThreads, 0, s>>>(span, nn_dev, group_max, i4, par, gf_);
    GF_CHECK_LAUNCH();
    exclusive_scan(gf_, gs, span, &cnt->num_groups, s, &scratch);
    k_group_write<<<ngrid, kThreads, 0, s>>>(span, nn_dev, gf_, gs, groups.get<int>(cap));
    GF_CHECK_LAUNCH();

    uint64_t* bk = bfs_key.get<uint64_t>(cap);
    int* bv = bfs_val.get<int>(cap);
    k_bfs_keys<<<ngrid, kThreads, 0, s>>>(span, nn_dev, i4, bk, bv);
    GF_CHECK_LAUNCH();
    radix_sort_pairs(bk, bv, bfs_key_alt.get<uint64_t>(cap), bfs_val_alt.get<int>(cap), span, 0, 8, s, &scratch);
    int* bfs = n_bfs.get<int>(cap);
    k_bfs_index<<<ngrid, kThreads, 0, s>>>(span, nn_dev, bv, bfs);
    GF_CHECK_LAUNCH();
    // breadth-first geometry and parents: the neighbour search, and the mixed form's refit
    const bool bfs_geo = want_knn || quad;
    const bool bfs_moments = quad && !want_knn;
    k_walk_fill<<<ngrid, kThreads, 0, s>>>(span, i4, nch, bfs, bfs_moments ? nullptr : mom, opr, geo,
                                           w_a.get<float4>(cap), w_b.get<float4>(cap),
                                           bfs_geo ? w_geo.get<float4>(cap) : nullptr,
                                           want_knn ? leaf_of.get<int>(n) : nullptr, par,
                                           bfs_geo ? w_parent.get<int>(cap) : nullptr, nn_dev);
    GF_CHECK_LAUNCH();
    if (bfs_moments) {  // mixed form: float32 monopole + quadrupole moments in one bottom-up pass
        GF_CUDA(cudaMemsetAsync(ctr, 0, sizeof(int) * size_t(span), s));
        RefitBfsArgs A{span, nn_dev, theta_f, w_parent.as<int>(), w_geo.as<float4>(), ctr, w_a.as<float4>(),
                       w_b.as<float4>(), w_q.get<float4>(cap), w_t.get<float2>(cap), w_rq.get<float>(cap), ndp, pp,
                       nullptr};
        ProfScope psm(kStTreeMoments, s);
        k_refit_bfs_quad32<<<ngrid, kThreads, 0, s>>>(A);
        GF_CHECK_LAUNCH();
    }
    valid = true;
    if (!g_no_alloc) {  // outside a capture: the live node count, for outgrowing()
        if (!h_live) GF_CUDA(cudaMallocHost(&h_live, sizeof(int)));
        if (!live_ev) GF_CUDA(cudaEventCreateWithFlags(&live_ev, cudaEventDisableTiming));
        GF_CUDA(cudaMemcpyAsync(h_live, &cnt->total_nodes, sizeof(int), cudaMemcpyDeviceToHost, s));
        GF_CUDA(cudaEventRecord(live_ev, s));
        live_pending = true;
    }
}

bool Octree::outgrowing() {
    if (!live_pending) return false;
    const cudaError_t e = cudaEventQuery(live_ev);
    if (e == cudaErrorNotReady) {
        (void)cudaGetLastError();  // not an error: the copy is still on its way
        return false;
    }
    GF_CUDA(e);
    live_pending = false;
    return *h_live > node_cap - node_cap / 8;
}

// Node kernels cover node_cap and read the live node count on the device, so a refit stays
// valid after a rebuild inside a captured graph (whose node count the host never sees).
void Octree::refit(const double* pos, const double* mass, cudaStream_t s, cudaStream_t s_moments,
                   cudaEvent_t gathered) {
    ProfScope ps(kStTreeRefit, s);
    const int grid = div_up(n, kThreads);
    const int span = std::max(node_cap, nn);
    const int ngrid = div_up(span, kThreads);
    const int* nn_dev = &counts.as<TreeCounts>()->total_nodes;
    float4* pp = p4.as<float4>();
    float* pd = pdisp.get<float>(n);
    k_gather<<<grid, kThreads, 0, s>>>(n, perm.as<int>(), pos, mass, xbuild.as<double>(), pp, pd,
                                       want_knn ? plo.get<float4>(n) : nullptr, quad ? 1 : 0);
    GF_CHECK_LAUNCH();
    if (s_moments) {  // the moments on their own stream, after the gather
        GF_CUDA(cudaEventRecord(gathered, s));
        GF_CUDA(cudaStreamWaitEvent(s_moments, gathered, 0));
        s = s_moments;
    }
    int* ctr = n_counter.as<int>();
    GF_CUDA(cudaMemsetAsync(ctr, 0, sizeof(int) * size_t(span), s));
    if (quad) {  // mixed form: straight into the walk layout
        RefitBfsArgs A{span, nn_dev, theta_f, w_parent.as<int>(), w_geo.as<float4>(), ctr, w_a.as<float4>(),
                       w_b.as<float4>(), w_q.as<float4>(), w_t.as<float2>(), w_rq.as<float>(), n_disp.as<float>(), pp,
                       pd};
        k_refit_bfs_quad32<<<ngrid, kThreads, 0, s>>>(A);
        GF_CHECK_LAUNCH();
        return;
    } else {
        MomentArgs A{};
        A.nn = span;
        A.nn_dev = nn_dev;
        A.refit = true;
        A.theta = theta_f;
        A.n_i4 = n_i4.as<int4>();
        A.parent = n_parent.as<int>();
        A.nchild = n_nchild.as<int>();
        A.kids = n_kids.as<int>();
        A.counter = ctr;
        A.n_cd = n_cd.as<double4>();
        A.n_geo = n_geo.as<float4>();
        A.mom = n_mom.as<float4>();
        A.open_r = n_open.as<float>();
        A.ndisp = n_disp.as<float>();
        A.p4 = pp;
        A.pdisp = pd;
        k_moments<<<ngrid, kThreads, 0, s>>>(A);
        GF_CHECK_LAUNCH();
    }
    k_walk_fill<<<ngrid, kThreads, 0, s>>>(span, n_i4.as<int4>(), n_nchild.as<int>(), n_bfs.as<int>(),
                                           n_mom.as<float4>(), n_open.as<float>(), n_geo.as<float4>(),
                                           w_a.as<float4>(), w_b.as<float4>(),
                                           want_knn ? w_geo.as<float4>() : nullptr,
                                           want_knn ? leaf_of.as<int>() : nullptr, n_parent.as<int>(),
                                           want_knn ? w_parent.as<int>() : nullptr, nn_dev);
    GF_CHECK_LAUNCH();
}

}  // namespace gf
