// gf_walk.cu — group tree walk + interaction-list evaluation (cpp/nbody.cpp:323-411).
//
// One warp per walk group (the reference's groups: shallowest nodes with <= 64 particles),
// persistent blocks pulling groups from an atomic counter (the reference's dynamic
// schedule). Per group:
//   * bounding sphere of its massive particles (float32, cpp/nbody.cpp:350-366) — computed
//     once per call in k_group_prep together with the active count;
//   * walk: the reference tests nodes one at a time along depth-first `next` links; here
//     the warp tests up to 32 nodes at once, taken from a shared-memory stack of child
//     ranges (children are contiguous in the breadth-first walk layout). A node is visited
//     iff all its ancestors were opened, so the set of accepted nodes and opened leaves —
//     the interaction list — is exactly the reference's; only the summation order differs;
//   * accepted monopoles and opened-leaf particles are appended to a shared-memory tile of
//     256 float4 entries, evaluated by the warp whenever it fills: each active particle of
//     the group owns 1..32 lanes (lanes split the tile when the group is small, two
//     particles per lane when it has more than 32 active particles);
//   * pair term as cpp/nbody.cpp:398-402 in float32: a += m d / (|d|^2 + eps^2)^(3/2).
// The mixed form (QUAD) walks work items (groups, runs of sibling groups, or chunks of a
// group's active particles), accepts nodes by the geometric or the relative criterion,
// keeps a second tile of quadrupole nodes (far accepted nodes may join the monopole tile),
// evaluates both tiles with 4 particles per lane and adds each tile's partial sums to Kahan
// totals.
// Accelerations are written as float64 into acc[3*k] for original index k (active only).
#include <algorithm>

#include "gf_tree.cuh"

namespace gf {

namespace {

constexpr int kWalkWarps = 4;
constexpr int kStackCap = 1024;   // child ranges per warp
constexpr int kTileCap = 256;     // interaction entries per warp
// Nodes tested per lane and round of the walk (their loads are issued together, so one
// round's memory latency covers them all): 2 for the mixed form's full evaluations (10 %
// faster at 1M than 1), 1 for the reference form (2 measured 3 % slower); 8 for walks of a
// few items (block time steps), which are bound by the latency of their rounds, not by work.

// Work list: groups with at least one active particle and a massive member, as work items
// {first particle, particle count, active particles to evaluate, rank of the first of them
// among the group's active particles}.
//   chunk == 0: one item per group with the reference's sphere (all massive members);
//   chunk  > 0: the group's active particles in tree order, cut into items of <= chunk,
//               each with the bounding sphere of its own particles. Sparse active sets
//               (block time steps) then spread over many warps with tight spheres instead of
//               one warp walking a whole group for a few particles.
//   merged items (mixed form, chunk == 0): consecutive sibling groups merged into items of
//               <= merge_cap particles, written in tree order by k_item_flag / k_item_fill;
//   aold != null: per item, gam = (alpha * a_min)^(-1/5) with a_min the smallest previous
//               |acceleration| among the item's particles (relative opening criterion; 0, i.e.
//               geometric only, when that minimum is not positive).
__device__ __forceinline__ float aold_mag(const double* aold, int k) {
    const double x = aold[3 * size_t(k)], y = aold[3 * size_t(k) + 1], z = aold[3 * size_t(k) + 2];
    return float(sqrt(x * x + y * y + z * z));
}

// (alpha a_min)^(-1/5) and (alpha_q a_min)^(-1/4) (0 where off or a_min is not positive)
__device__ __forceinline__ float2 rel_gamma(float alpha, float alpha_q, float amin) {
    if (!(alpha > 0.f && amin > 0.f && amin < 3e38f)) return make_float2(0.f, 0.f);
    return make_float2(exp2f(-0.2f * log2f(alpha * amin)), alpha_q > 0.f ? exp2f(-0.25f * log2f(alpha_q * amin)) : 0.f);
}

// One work item over the particles [b, e) of the tree (a group, or a run of sibling groups):
// its active count, the bounding sphere of its massive particles and, with aold, its scale of
// the relative criterion; an item without active or massive particles is not valid.
struct ItemStats {
    int nact;
    float4 sph;
    float2 gam;
    bool valid;
};

// act_sphere: the sphere bounds the active particles (the item's targets) instead of the massive
// ones (items merged by active count, whose inactive members are not evaluated).
__device__ __forceinline__ ItemStats item_stats(int b, int e, const float4* __restrict__ p4,
                                                const int* __restrict__ perm, const uint8_t* __restrict__ active,
                                                const double* __restrict__ aold, float alpha, float alpha_q,
                                                bool act_sphere = false) {
    const int lane = threadIdx.x & 31;
    ItemStats st;
    st.valid = false;
    int nact = 0;
    float x0 = 1e30f, y0 = 1e30f, z0 = 1e30f, x1 = -1e30f, y1 = -1e30f, z1 = -1e30f;
    float amin = INFINITY;
    for (int i = b + lane; i < e; i += 32) {
        const bool a = active ? active[perm[i]] != 0 : true;
        nact += __popc(__ballot_sync(__activemask(), a));
        if (aold && a) amin = fminf(amin, aold_mag(aold, perm[i]));
        const float4 p = p4[i];
        if (act_sphere ? a : p.w > 0) {
            x0 = fminf(x0, p.x); x1 = fmaxf(x1, p.x);
            y0 = fminf(y0, p.y); y1 = fmaxf(y1, p.y);
            z0 = fminf(z0, p.z); z1 = fmaxf(z1, p.z);
        }
    }
    st.nact = __shfl_sync(0xffffffffu, nact, 0);
    if (st.nact == 0) return st;
    x0 = warp_min(x0); y0 = warp_min(y0); z0 = warp_min(z0);
    x1 = warp_max(x1); y1 = warp_max(y1); z1 = warp_max(z1);
    if (x0 > x1) return st;  // massless
    const float bx = 0.5f * (x0 + x1), by = 0.5f * (y0 + y1), bz = 0.5f * (z0 + z1);
    float br2 = 0.f;
    for (int i = b + lane; i < e; i += 32) {
        const float4 p = p4[i];
        if (act_sphere ? active[perm[i]] != 0 : p.w > 0) {
            const float dx = p.x - bx, dy = p.y - by, dz = p.z - bz;
            br2 = fmaxf(br2, dx * dx + dy * dy + dz * dz);
        }
    }
    br2 = warp_max(br2);
    amin = warp_min(amin);
    // float32 rounding of the centre: pad so every target stays inside
    st.sph = make_float4(bx, by, bz, act_sphere ? sqrtf(br2) * (1.f + 1e-6f) : sqrtf(br2));
    st.gam = aold ? rel_gamma(alpha, alpha_q, amin) : make_float2(0.f, 0.f);
    st.valid = true;
    return st;
}

// Appends a valid item to the work list (in the order the warps get there).
__device__ __forceinline__ void emit_item(int b, int e, const float4* __restrict__ p4, const int* __restrict__ perm,
                                          const uint8_t* __restrict__ active, TreeCounts* cnt,
                                          int4* __restrict__ work, float4* __restrict__ sphere,
                                          const double* __restrict__ aold, float alpha, float alpha_q,
                                          float2* __restrict__ gam) {
    const int lane = threadIdx.x & 31;
    const ItemStats st = item_stats(b, e, p4, perm, active, aold, alpha, alpha_q);
    if (!st.valid) return;
    int slot = 0;
    if (lane == 0) slot = atomicAdd(&cnt->num_work, 1);
    slot = __shfl_sync(0xffffffffu, slot, 0);
    if (lane == 0) {
        work[slot] = make_int4(b, e - b, st.nact, 0);
        sphere[slot] = st.sph;
        if (gam) gam[slot] = st.gam;
    }
}

// Merged items: each run of consecutive sibling groups (contiguous in tree order) is cut
// greedily into items of at most `merge` weight (a heavier group alone); the weight of a group
// is its particle count, or gw[g] where given (its active particles). A run holds at most 8
// groups (the octree fan-out), so lanes 0..15 load groups g-8 .. g+7; the warp finds the run
// around group g and replays the cut from the run's first group. Returns the weight of the item
// that g starts (-1 if g starts none) and, in b and len, its first particle and particle count.
// With status: a run longer than the fan-out (groups g-8 .. g all siblings, which the 8-child
// node layout rules out) raises GF_ERR_CAPACITY instead of being cut silently.
__device__ __forceinline__ int cut_at(const int* __restrict__ groups, const int4* __restrict__ n_i4,
                                      const int* __restrict__ parent, const int* __restrict__ gw, int ng,
                                      int merge, int g, int& b, int& len, uint32_t* status = nullptr) {
    const int lane = threadIdx.x & 31;
    const int idx = g - 8 + lane;
    int pg = -2, cg = 0, bg = 0, wg = 0;
    if (lane < 16 && idx >= 0 && idx < ng) {
        const int nd = groups[idx];
        const int4 q = n_i4[nd];
        pg = parent[nd];
        cg = q.y;
        bg = q.x;
        wg = gw ? gw[idx] : q.y;
    }
    const int par = __shfl_sync(0xffffffffu, pg, 8);
    b = __shfl_sync(0xffffffffu, bg, 8);
    const unsigned same = __ballot_sync(0xffffffffu, pg == par);
    if (status && (same & 0xffu) == 0xffu && lane == 0) raise_status(status, GF_ERR_CAPACITY);
    const unsigned below = ~same & 0xffu;     // lanes 0..7 outside the run
    const unsigned above = ~same & 0xfe00u;   // lanes 9..15 outside the run
    const int first = below ? 32 - __clz(below) : 0;
    const int last = above ? __ffs(above) - 1 : 16;
    int start = first, rw = 0, rl = 0, mine = -1;
    len = 0;
    for (int l = first; l < last; ++l) {
        const int w = __shfl_sync(0xffffffffu, wg, l);
        const int c = __shfl_sync(0xffffffffu, cg, l);
        if (l > start && rw + w <= merge) {
            rw += w;
            rl += c;
            continue;
        }
        if (l > start) {  // the item [start, l) closes
            if (start == 8) {
                mine = rw;
                len = rl;
            }
            start = l;
        }
        rw = w;
        rl = c;
    }
    if (start == 8) {  // the run's last item
        mine = rw;
        len = rl;
    }
    return mine;
}

// Active particles per group (items merged by active count).
__global__ void k_group_nact(const int* __restrict__ groups, const int4* __restrict__ n_i4,
                             const int* __restrict__ perm, const uint8_t* __restrict__ active,
                             const TreeCounts* cnt, int* __restrict__ gw) {
    const int lane = threadIdx.x & 31;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int ng = cnt->num_groups;
    for (int g = wid; g < ng; g += nw) {
        const int4 q = n_i4[groups[g]];
        int c = 0;
        for (int i = q.x + lane; i < q.x + q.y; i += 32) c += active[perm[i]] != 0 ? 1 : 0;
        c = warp_sum(c);
        if (lane == 0) gw[g] = c;
    }
}

// flag[g] = 1 when group g starts a merged item of positive weight (g < span; 0 past the live
// group count)
__global__ void k_item_flag(const int* __restrict__ groups, const int4* __restrict__ n_i4,
                            const int* __restrict__ parent, const int* __restrict__ gw, const TreeCounts* cnt,
                            int merge, int span, int* __restrict__ flag, uint32_t* status) {
    const int lane = threadIdx.x & 31;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int ng = cnt->num_groups;
    for (int g = wid; g < ng; g += nw) {
        int b, len;
        const int f = cut_at(groups, n_i4, parent, gw, ng, merge, g, b, len, status) > 0 ? 1 : 0;
        if (lane == 0) flag[g] = f;
    }
    // past the live groups (the scan covers span): zeros, a thread per entry
    for (int t = ng + blockIdx.x * blockDim.x + threadIdx.x; t < span; t += gridDim.x * blockDim.x) flag[t] = 0;
}

// The merged items in tree order: item of group g at slot[g] (the scan of the flags). An item
// without active or massive particles keeps its slot with no particles to evaluate. act_sphere
// (walks of an active set): the sphere bounds the item's active particles, the only ones it
// evaluates.
__global__ void k_item_fill(const int* __restrict__ groups, const int4* __restrict__ n_i4,
                            const int* __restrict__ parent, const int* __restrict__ gw, bool act_sphere,
                            const TreeCounts* cnt, int merge,
                            const int* __restrict__ flag, const int* __restrict__ slot,
                            const float4* __restrict__ p4, const int* __restrict__ perm,
                            const uint8_t* __restrict__ active, const double* __restrict__ aold,
                            float alpha, float alpha_q, int4* __restrict__ work, float4* __restrict__ sphere,
                            float2* __restrict__ gam) {
    const int lane = threadIdx.x & 31;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int ng = cnt->num_groups;
    for (int g = wid; g < ng; g += nw) {
        if (!flag[g]) continue;
        int b, count;
        cut_at(groups, n_i4, parent, gw, ng, merge, g, b, count);
        const ItemStats st = item_stats(b, b + count, p4, perm, active, aold, alpha, alpha_q, act_sphere);
        if (lane == 0) {
            const int k = slot[g];
            work[k] = make_int4(b, count, st.valid ? st.nact : 0, 0);
            sphere[k] = st.valid ? st.sph : make_float4(0.f, 0.f, 0.f, 0.f);
            if (gam) gam[k] = st.valid ? st.gam : make_float2(0.f, 0.f);
        }
    }
}

__global__ void k_group_prep(const int* __restrict__ groups, const int4* __restrict__ n_i4,
                             const float4* __restrict__ p4, const int* __restrict__ perm,
                             const uint8_t* __restrict__ active, TreeCounts* cnt,
                             int4* __restrict__ work, float4* __restrict__ sphere, int chunk,
                             const double* __restrict__ aold, float alpha, float alpha_q,
                             float2* __restrict__ gam) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = lanemask_lt();
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int ng = cnt->num_groups;
    for (int g = wid; g < ng; g += nw) {
        const int node = groups[g];
        const int4 q = n_i4[node];
        const int b = q.x, e = q.x + q.y;
        if (chunk > 0) {
            // pass over the group per item: rank of each active particle by ballot
            int r0 = 0;
            for (;;) {  // items [r0, r0 + chunk)
                float x0 = 1e30f, y0 = 1e30f, z0 = 1e30f, x1 = -1e30f, y1 = -1e30f, z1 = -1e30f;
                float amin = INFINITY;
                int rank_base = 0, in_item = 0;
                for (int i0 = b; i0 < e; i0 += 32) {
                    const int i = i0 + lane;
                    const bool a = i < e && active[perm[i]] != 0;
                    const unsigned m = __ballot_sync(0xffffffffu, a);
                    const int rank = rank_base + __popc(m & lt);
                    if (a && rank >= r0 && rank < r0 + chunk) {
                        const float4 p = p4[i];
                        x0 = fminf(x0, p.x); x1 = fmaxf(x1, p.x);
                        y0 = fminf(y0, p.y); y1 = fmaxf(y1, p.y);
                        z0 = fminf(z0, p.z); z1 = fmaxf(z1, p.z);
                        if (aold) amin = fminf(amin, aold_mag(aold, perm[i]));
                        ++in_item;
                    }
                    rank_base += __popc(m);
                    if (rank_base >= r0 + chunk) break;
                }
                const int P = warp_sum(in_item);
                if (P == 0) break;
                x0 = warp_min(x0); y0 = warp_min(y0); z0 = warp_min(z0);
                x1 = warp_max(x1); y1 = warp_max(y1); z1 = warp_max(z1);
                const float bx = 0.5f * (x0 + x1), by = 0.5f * (y0 + y1), bz = 0.5f * (z0 + z1);
                float br2 = 0.f;
                int rb = 0;
                for (int i0 = b; i0 < e && rb < r0 + chunk; i0 += 32) {
                    const int i = i0 + lane;
                    const bool a = i < e && active[perm[i]] != 0;
                    const unsigned m = __ballot_sync(0xffffffffu, a);
                    const int rank = rb + __popc(m & lt);
                    if (a && rank >= r0 && rank < r0 + chunk) {
                        const float4 p = p4[i];
                        const float dx = p.x - bx, dy = p.y - by, dz = p.z - bz;
                        br2 = fmaxf(br2, dx * dx + dy * dy + dz * dz);
                    }
                    rb += __popc(m);
                }
                br2 = warp_max(br2);
                amin = warp_min(amin);
                int slot = 0;
                if (lane == 0) slot = atomicAdd(&cnt->num_work, 1);
                slot = __shfl_sync(0xffffffffu, slot, 0);
                if (lane == 0) {
                    work[slot] = make_int4(b, q.y, P, r0);
                    // float32 rounding of the centre: pad so every member stays inside
                    sphere[slot] = make_float4(bx, by, bz, sqrtf(br2) * (1.f + 1e-6f));
                    if (gam) gam[slot] = aold ? rel_gamma(alpha, alpha_q, amin) : make_float2(0.f, 0.f);
                }
                if (P < chunk) break;
                r0 += chunk;
            }
            continue;
        }
        emit_item(b, e, p4, perm, active, cnt, work, sphere, aold, alpha, alpha_q, gam);
    }
}

// Shared memory of one warp. QUAD (mixed form) adds a tile of accepted nodes with their
// quadrupoles; particles of opened leaves always go to the monopole tile. SMALL: the mixed
// form's interaction tiles at 128 particle and 64 node entries instead of 256 and 96 (fewer
// entries per evaluation pass, 40 % less shared memory per warp).
template <bool QUAD, int NPL, bool SMALL = false>
struct WarpSmem {
    static constexpr int kStack = QUAD ? 768 : kStackCap;
    static constexpr int kTile = (QUAD && (NPL > 2 || SMALL)) ? 128 : kTileCap;  // particle entries
    static constexpr int kNodeTile = QUAD ? (SMALL ? 64 : 96) : 1;
    static constexpr int kBatch = QUAD ? 128 : 64;  // active particles evaluated per walk
    int stack[kStack];
    float4 tile[kTile];
    float4 ntA[kNodeTile];   // centre of mass, mass
    float4 ntQ[kNodeTile];   // Qxx, Qyy, Qxy, Qxz
    float2 ntYZ[kNodeTile];  // Qyz, T
    int lanemap[QUAD ? 32 * NPL : 1];  // slot -> node of a round (mixed form)
    int slot_pos[kBatch];
};

// |d|^2 + eps^2 as one fused chain seeded with eps^2 (three FMAs)
__device__ __forceinline__ float soft_r2(float ex, float ey, float ez, float eps2) {
    return fmaf(ex, ex, fmaf(ey, ey, fmaf(ez, ez, eps2)));
}

__device__ __forceinline__ void pair_acc(const float4 e, float x, float y, float z, float eps2,
                                         float& ax, float& ay, float& az) {
    const float ex = e.x - x, ey = e.y - y, ez = e.z - z;
    const float r2 = soft_r2(ex, ey, ez, eps2);
    const float inv = rsqrtf(r2);
    const float f = e.w * inv * inv * inv;
    ax += f * ex;
    ay += f * ey;
    az += f * ez;
}

// the same pair with the softened potential -m / sqrt(|d|^2 + eps^2) (energy diagnostics;
// a particle's pair with itself, d = 0, adds nothing)
__device__ __forceinline__ void pair_acc_pot(const float4 e, float x, float y, float z, float eps2,
                                             float& ax, float& ay, float& az, float& ph) {
    const float ex = e.x - x, ey = e.y - y, ez = e.z - z;
    const float r2 = soft_r2(ex, ey, ez, eps2);
    const float inv = rsqrtf(r2);
    const float mi = e.w * inv;
    const float f = mi * inv * inv;
    ax += f * ex;
    ay += f * ey;
    az += f * ez;
    ph -= (ex != 0.f || ey != 0.f || ez != 0.f) ? mi : 0.f;  // no self term
}

// Second-order expansion of the Plummer-softened field of a node about its centre of mass,
// at d = com - x, r^2 = |d|^2 + eps^2, Q the traceless quadrupole and T = sum m |y|^2:
//   a = M d / r^3 - Q d / r^5 + (5/2) (d.Q.d) d / r^7 - (5/2) T eps^2 d / r^7.
// The last term comes from the trace of the second moment, which the softened potential
// (unlike 1/r) does not annihilate; it matters for cells accepted within a few eps.
// c_t = (5/2) T eps^2 is the node's constant of that term (the caller computes it once per node
// for all the particles it serves).
__device__ __forceinline__ void quad_acc(const float4 e, const float4 q, float qyz, float c_t, float x, float y,
                                         float z, float eps2, float& ax, float& ay, float& az) {
    const float dx = e.x - x, dy = e.y - y, dz = e.z - z;
    const float r2 = soft_r2(dx, dy, dz, eps2);
    const float inv = rsqrtf(r2);
    const float inv2 = inv * inv;
    const float inv3 = inv2 * inv;
    const float inv5 = inv3 * inv2;
    const float inv7 = inv5 * inv2;
    const float qzz = -(q.x + q.y);
    const float qdx = q.x * dx + q.z * dy + q.w * dz;
    const float qdy = q.z * dx + q.y * dy + qyz * dz;
    const float qdz = q.w * dx + qyz * dy + qzz * dz;
    const float dqd = dx * qdx + dy * qdy + dz * qdz;
    const float f = fmaf(fmaf(2.5f, dqd, -c_t), inv7, e.w * inv3);
    ax += f * dx - inv5 * qdx;
    ay += f * dy - inv5 * qdy;
    az += f * dz - inv5 * qdz;
}

// Evaluates the tile entries [0, fill) for the lane's particle(s); POT also sums potentials.
template <bool POT>
__device__ __forceinline__ void eval_tile(const float4* tile, int fill, bool two, int r, int sub, float eps2,
                                          float x0, float y0, float z0, float x1, float y1, float z1,
                                          float& ax0, float& ay0, float& az0, float& ax1, float& ay1,
                                          float& az1, float& ph0, float& ph1) {
    if constexpr (POT) {
        if (two) {
            for (int j = 0; j < fill; ++j) {
                const float4 e = tile[j];
                pair_acc_pot(e, x0, y0, z0, eps2, ax0, ay0, az0, ph0);
                pair_acc_pot(e, x1, y1, z1, eps2, ax1, ay1, az1, ph1);
            }
        } else {
            for (int j = sub; j < fill; j += r) pair_acc_pot(tile[j], x0, y0, z0, eps2, ax0, ay0, az0, ph0);
        }
        return;
    }
    if (two) {
#pragma unroll 2
        for (int j = 0; j < fill; ++j) {
            const float4 e = tile[j];
            pair_acc(e, x0, y0, z0, eps2, ax0, ay0, az0);
            pair_acc(e, x1, y1, z1, eps2, ax1, ay1, az1);
        }
    } else if (r == 1) {
#pragma unroll 4
        for (int j = 0; j < fill; ++j) pair_acc(tile[j], x0, y0, z0, eps2, ax0, ay0, az0);
    } else {
#pragma unroll 4
        for (int j = sub; j < fill; j += r) pair_acc(tile[j], x0, y0, z0, eps2, ax0, ay0, az0);
    }
}

// Mixed form: entries ksub, ksub + m, ... of both tiles for the lane's PPL (4) particles (each
// entry loaded once from shared memory serves the PPL); the tile's partial sums go to Kahan
// totals.
template <int PPL>
__device__ __forceinline__ void eval_quad(const float4* tile, const float4* ntA, const float4* ntQ,
                                          const float2* ntYZ, int fill, int fillN, int ksub, int m, float eps2,
                                          const float (&x)[4], const float (&y)[4], const float (&z)[4],
                                          KahanF (&kx)[4], KahanF (&ky)[4], KahanF (&kz)[4]) {
    float px[PPL], py[PPL], pz[PPL];
#pragma unroll
    for (int t = 0; t < PPL; ++t) px[t] = py[t] = pz[t] = 0.f;
    for (int j = ksub; j < fill; j += m) {
        const float4 e = tile[j];
#pragma unroll
        for (int t = 0; t < PPL; ++t) pair_acc(e, x[t], y[t], z[t], eps2, px[t], py[t], pz[t]);
    }
    for (int j = ksub; j < fillN; j += m) {
        const float4 e = ntA[j], q = ntQ[j];
        const float2 yt = ntYZ[j];
        const float c_t = 2.5f * yt.y * eps2;
#pragma unroll
        for (int t = 0; t < PPL; ++t) quad_acc(e, q, yt.x, c_t, x[t], y[t], z[t], eps2, px[t], py[t], pz[t]);
    }
#pragma unroll
    for (int t = 0; t < PPL; ++t) {
        kx[t].add(px[t]);
        ky[t].add(py[t]);
        kz[t].add(pz[t]);
    }
}

// POT (monopole form only): also the softened potential of every walked particle, into pot.
// Blocks per SM: shared memory allows 4 of the mixed form's and 6 of the reference form's;
// 5 keeps the latter free of register spills; the wide-round variant needs more registers.
// WARPS (block shape) and SMALL (tile size) are the mixed walk's tunable launch shape: the
// register bound keeps 16 warps per SM whatever the block shape.
template <bool QUAD, bool POT = false, int NPL = (QUAD ? 2 : 1), int WARPS = kWalkWarps, bool SMALL = false>
__global__ void __launch_bounds__(WARPS * 32, QUAD ? (NPL > 2 ? 1 : 16 / WARPS) : 5) k_walk(
    const float4* __restrict__ wa, const float4* __restrict__ wb, const float4* __restrict__ wq,
    const float2* __restrict__ wt, const float* __restrict__ wrq, const float4* __restrict__ p4,
    const int* __restrict__ perm, const uint8_t* __restrict__ active, const int4* __restrict__ work,
    const float4* __restrict__ sphere, const float2* __restrict__ gam, TreeCounts* cnt, int nn, float eps2,
    double* __restrict__ acc, uint32_t* status, int stride, double* __restrict__ pot = nullptr) {
    static_assert(!(QUAD && POT), "potentials come from the monopole walk");
    using Smem = WarpSmem<QUAD, NPL, SMALL>;
    constexpr int kNodesPerLane = NPL;
    constexpr int kRound = 32 * kNodesPerLane;
    __shared__ Smem smem_all[WARPS];
    Smem& S = smem_all[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const unsigned lt = lanemask_lt();
    // Tickets go to items through a stride permutation: ticket t -> item (t mod stride) *
    // ceil(nwork / stride) + t / stride, so the warps at work at one time spread over `stride`
    // regions of a work list in tree order, each taken in order (1: the list's own order).
    const int nwork = cnt->num_work;
    const int per = (nwork + stride - 1) / stride;
    const int ntick = per * stride;

    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(&cnt->walk_next, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= ntick) break;
        const int g = (t % stride) * per + t / stride;
        if (g >= nwork) continue;
        const int4 w = work[g];
        const float4 sph = sphere[g];
        // relative criterion: accept a node when its distance from the sphere exceeds both
        // open_r (geometric) and rho * gm (rho = B.w: 0 outside quadrupole trees); take an
        // accepted node as a monopole when that distance also exceeds rho_q * gq (gq > 0)
        const float2 gg = QUAD ? gam[g] : make_float2(0.f, 0.f);
        const float gm = gg.x, gq = gg.y;
        const int b = w.x, count = w.y, Pall = w.z, r0 = w.w;
        // Items hold <= kBatch particles except depth-48 leaves of coincident points; those
        // are evaluated in batches, each batch walking the tree again.
        for (int pb = 0; pb < Pall; pb += Smem::kBatch) {
        const int P = min(Smem::kBatch, Pall - pb);

        // compact the active particles of this batch into slots
        int nslot = 0;
        for (int i0 = 0; i0 < count; i0 += 32) {
            const int i = b + i0 + lane;
            const bool a = i0 + lane < count && (active ? active[perm[i]] != 0 : true);
            const unsigned m = __ballot_sync(0xffffffffu, a);
            const int rank = nslot + __popc(m & lt);
            if (a && rank >= r0 + pb && rank < r0 + pb + P) S.slot_pos[rank - r0 - pb] = i;
            nslot += __popc(m);
        }
        __syncwarp();

        // Lane mapping.
        //   monopole (reference form): r lanes per particle splitting the entries (r = 1 and
        //     two slots per lane when P > 32);
        //   QUAD (mixed form): every lane holds 4 particles, so each entry read from shared
        //     memory serves 4 interactions; L = ceil(P / 4) lanes cover the batch and
        //     m = 32 / L groups of L lanes split the entries (the 4-particle slots of lane
        //     q hold particles 4q .. 4q + 3). (A second evaluation loop with 3 per lane, for
        //     batches that leave lanes idle, slowed every batch by ~10 %: it is not kept.)
        constexpr int kPpl = QUAD ? 4 : 2;
        constexpr int ppl = kPpl;
        int r = 1, sub = 0, m = 1, ksub = 0, L = 1;
        bool lane_on = true;
        int slot[kPpl];
        if (QUAD) {
            L = (P + ppl - 1) / ppl;
            m = max(1, 32 / L);
            ksub = lane / L;
            lane_on = ksub < m;
            const int q = lane - ksub * L;
#pragma unroll
            for (int t = 0; t < kPpl; ++t) slot[t] = t < ppl ? ppl * q + t : P;  // P: no particle
        } else {
            if (P <= 16) r = P <= 1 ? 32 : P <= 2 ? 16 : P <= 4 ? 8 : P <= 8 ? 4 : 2;
            slot[0] = lane / r;
            slot[1] = slot[0] + 32;
            sub = lane % r;
        }
        float x[kPpl], y[kPpl], z[kPpl];
        bool has[kPpl];
#pragma unroll
        for (int t = 0; t < kPpl; ++t) {
            has[t] = lane_on && slot[t] < P && (QUAD || t == 0 || P > 32);
            x[t] = y[t] = z[t] = 0.f;
            if (has[t]) {
                const float4 p = p4[S.slot_pos[slot[t]]];
                x[t] = p.x; y[t] = p.y; z[t] = p.z;
            }
        }
        // reference form: one float32 running sum per component; mixed form: each tile's
        // partial sums are added to Kahan-compensated totals
        float ax[kPpl], ay[kPpl], az[kPpl], ph[kPpl];
        KahanF kx[kPpl], ky[kPpl], kz[kPpl];
#pragma unroll
        for (int t = 0; t < kPpl; ++t) ax[t] = ay[t] = az[t] = ph[t] = 0.f;
        const bool two = P > 32;

        int fill = 0, fillN = 0;
        unsigned long long listlen = 0, nodelen = 0;
#define GF_WALK_FLUSH()                                                                              \
    do {                                                                                             \
        listlen += fill + fillN;                                                                     \
        nodelen += fillN;                                                                            \
        __syncwarp();                                                                                \
        if constexpr (QUAD) {                                                                        \
            if (lane_on) eval_quad<4>(S.tile, S.ntA, S.ntQ, S.ntYZ, fill, fillN, ksub, m, eps2, x, y, z, \
                                      kx, ky, kz);                                                   \
        } else {                                                                                     \
            eval_tile<POT>(S.tile, fill, two, r, sub, eps2, x[0], y[0], z[0], x[1], y[1], z[1],      \
                           ax[0], ay[0], az[0], ax[1], ay[1], az[1], ph[0], ph[1]);                  \
        }                                                                                            \
        __syncwarp();                                                                                \
        fill = 0;                                                                                    \
        fillN = 0;                                                                                   \
    } while (0)

        int sp = 1;
        if (lane == 0) S.stack[0] = (0 << 4) | 1;  // root: range (first 0, count 1)
        bool overflow = false;
        __syncwarp();
        // every node is popped at most once per walk: more rounds than nodes is a bug
        for (int rounds = 0; sp > 0; ++rounds) {
            if (rounds > nn) {
                overflow = true;
                break;
            }
            // pop up to kRound nodes from the top ranges (kNodesPerLane per lane: their loads
            // are issued together, so one round's memory latency covers them all)
            int nodes[kNodesPerLane];
            int nnodes;
            if constexpr (!QUAD) {
                nnodes = pop_round<kNodesPerLane>(S.stack, sp, nodes);
            } else {  // the slots' nodes staged in shared memory (shorter round latency)
                const int k = min(sp, 32);
                int e = 0, c = 0;
                if (lane < k) {
                    e = S.stack[sp - 1 - lane];
                    c = e & 15;
                }
                const int incl = warp_incl_scan(c);
                const int excl = incl - c;
                const unsigned fullm = __ballot_sync(0xffffffffu, lane < k && incl <= kRound);
                const int nfull = __popc(fullm);
                nnodes = __shfl_sync(0xffffffffu, incl, k - 1);
                int take = c;
                if (nfull < k) {  // range `nfull` is split: the rest stays on the stack
                    nnodes = kRound;
                    if (lane == nfull) {
                        take = kRound - excl;
                        S.stack[sp - 1 - lane] = (((e >> 4) + take) << 4) | (c - take);
                    }
                }
                __syncwarp();
                if (lane < k && lane <= nfull) {
                    const int first = e >> 4;
                    for (int t = 0; t < take && excl + t < kRound; ++t) S.lanemap[excl + t] = first + t;
                }
                sp -= nfull;
                __syncwarp();
#pragma unroll
                for (int i = 0; i < kNodesPerLane; ++i) {
                    const int slot = lane + 32 * i;
                    nodes[i] = slot < nnodes ? S.lanemap[slot] : -1;
                }
                __syncwarp();
            }
            float4 As[kNodesPerLane], Bs[kNodesPerLane];
            float RQs[kNodesPerLane];
#pragma unroll
            for (int i = 0; i < kNodesPerLane; ++i) {
                As[i] = make_float4(0.f, 0.f, 0.f, 0.f);
                Bs[i] = As[i];
                RQs[i] = 0.f;
                if (nodes[i] >= 0) {
                    As[i] = wa[nodes[i]];
                    Bs[i] = wb[nodes[i]];
                    if (QUAD && gq > 0.f) RQs[i] = wrq[nodes[i]];
                }
            }
#pragma unroll
            for (int i = 0; i < kNodesPerLane; ++i) {
            if (32 * i >= nnodes) break;  // warp-uniform
            const int node = nodes[i];
            const bool valid = node >= 0;
            const float4 A = As[i], B = Bs[i];
            const float dx = A.x - sph.x, dy = A.y - sph.y, dz = A.z - sph.z;
            const float t = (QUAD ? fmaxf(B.x, B.w * gm) : B.x) + sph.w;
            const float dd2 = dx * dx + dy * dy + dz * dz;
            const bool accept = valid && (dd2 > t * t);
            const float tq = RQs[i] * gq + sph.w;
            const bool mono = QUAD && accept && gq > 0.f && dd2 > tq * tq;  // quadrupole below alpha_q a_min
            const int first = __float_as_int(B.y), code = __float_as_int(B.z);
            const bool leaf = valid && !accept && code < 0;
            const bool open = valid && !accept && code > 0;

            // The loads this slot needs are issued here, ahead of the pushes and appends that
            // do not depend on them: an accepted quadrupole node's moments, and the first 32
            // particles of the round's opened leaves (concatenated in lane order; entry o goes
            // to lane o, which finds its leaf by a binary search over the inclusive sums).
            float4 qv = make_float4(0.f, 0.f, 0.f, 0.f);
            float2 yv = make_float2(0.f, 0.f);
            if (QUAD && accept && !mono) {
                qv = wq[node];
                yv = wt[node];
            }
            const bool anyleaf = __any_sync(0xffffffffu, leaf);
            int lincl = 0, lexcl = 0, ltot = 0;
            float4 lp = make_float4(0.f, 0.f, 0.f, 0.f);
            if (anyleaf) {
                const int lc = leaf ? -code : 0;
                lincl = warp_incl_scan(lc);
                lexcl = lincl - lc;
                ltot = __shfl_sync(0xffffffffu, lincl, 31);
                int src = 0;
#pragma unroll
                for (int step = 16; step; step >>= 1) {
                    const int v = __shfl_sync(0xffffffffu, lincl, src + step - 1);
                    if (v <= lane) src += step;
                }
                const int f = __shfl_sync(0xffffffffu, first, src);
                const int x = __shfl_sync(0xffffffffu, lexcl, src);
                if (lane < ltot) lp = p4[f + (lane - x)];
            }

            // opened internal nodes: push their child ranges
            const unsigned om = __ballot_sync(0xffffffffu, open);
            const int npush = __popc(om);
            if (sp + npush > Smem::kStack) {
                overflow = true;
                break;
            }
            if (open) S.stack[sp + __popc(om & lt)] = (first << 4) | code;
            sp += npush;

            // accepted nodes: monopole (reference) or monopole + quadrupole (mixed) entries;
            // the mixed form's far nodes (mono) join the monopole tile of the leaf particles
            if (QUAD) {
                const unsigned qm = __ballot_sync(0xffffffffu, accept && !mono);
                const int nq = __popc(qm);
                if (fillN + nq > Smem::kNodeTile) GF_WALK_FLUSH();
                if (accept && !mono) {
                    const int slot_n = fillN + __popc(qm & lt);
                    S.ntA[slot_n] = A;
                    S.ntQ[slot_n] = qv;
                    S.ntYZ[slot_n] = yv;
                }
                fillN += nq;
                const unsigned mm = __ballot_sync(0xffffffffu, mono);
                const int nm = __popc(mm);
                if (nm) {
                    if (fill + nm > Smem::kTile) GF_WALK_FLUSH();
                    if (mono) S.tile[fill + __popc(mm & lt)] = A;
                    fill += nm;
                }
            } else {
                const unsigned am = __ballot_sync(0xffffffffu, accept);
                const int na = __popc(am);
                if (fill + na > Smem::kTile) GF_WALK_FLUSH();
                if (accept) S.tile[fill + __popc(am & lt)] = A;
                fill += na;
            }

            // opened leaves: their particles, the first 32 from the loads above
            if (anyleaf) {
            const int n0 = min(32, ltot);
            if (fill + n0 > Smem::kTile) GF_WALK_FLUSH();
            if (lane < n0) S.tile[fill + lane] = lp;
            fill += n0;
            for (int done = n0; done < ltot;) {
                if (fill == Smem::kTile) GF_WALK_FLUSH();
                const int chunk = min(Smem::kTile - fill, ltot - done);
                // warp-cooperative copy: entry o of the concatenated leaves goes to lane o % 32,
                // which finds its leaf by a binary search over the inclusive sums (32 loads in
                // flight at once instead of each leaf's particles one after another)
                for (int base = 0; base < chunk; base += 32) {
                    const int o = done + base + lane;
                    int src = 0;
#pragma unroll
                    for (int step = 16; step; step >>= 1) {
                        const int v = __shfl_sync(0xffffffffu, lincl, src + step - 1);
                        if (v <= o) src += step;
                    }
                    const int f = __shfl_sync(0xffffffffu, first, src);
                    const int x = __shfl_sync(0xffffffffu, lexcl, src);
                    if (base + lane < chunk) S.tile[fill + base + lane] = p4[f + (o - x)];
                }
                fill += chunk;
                done += chunk;
            }
            }  // any leaf
            __syncwarp();
            }  // nodes of the lane
            if (overflow) break;
        }
        if (overflow) {
            if (lane == 0) raise_status(status, GF_ERR_WALK_STACK);
            break;
        }
        GF_WALK_FLUSH();
#undef GF_WALK_FLUSH
        if (lane == 0) {
            atomicAdd(&cnt->pairs, listlen * (unsigned long long)P);
            if (QUAD) atomicAdd(&cnt->qpairs, nodelen * (unsigned long long)P);
        }
        if constexpr (QUAD) {
            // sum the m entry groups of every particle in a fixed order (the tile is free now)
            float* red = reinterpret_cast<float*>(S.tile);  // m groups x ppl L slots x 3 <= 384 floats
            if (lane_on) {
#pragma unroll
                for (int t = 0; t < kPpl; ++t) {
                    if (t < ppl) {
                        float* o = red + 3 * (ksub * ppl * L + slot[t]);
                        o[0] = kx[t].s;
                        o[1] = ky[t].s;
                        o[2] = kz[t].s;
                    }
                }
            }
            __syncwarp();
            for (int p = lane; p < P; p += 32) {
                float sx = 0.f, sy = 0.f, sz = 0.f;
                for (int kk = 0; kk < m; ++kk) {
                    const float* o = red + 3 * (kk * ppl * L + p);
                    sx += o[0];
                    sy += o[1];
                    sz += o[2];
                }
                const int kp = perm[S.slot_pos[p]];
                acc[3 * size_t(kp)] = sx;
                acc[3 * size_t(kp) + 1] = sy;
                acc[3 * size_t(kp) + 2] = sz;
            }
        } else {
            // combine the partial sums of the lanes that share a particle
            for (int o = r >> 1; o > 0; o >>= 1) {
                ax[0] += __shfl_xor_sync(0xffffffffu, ax[0], o);
                ay[0] += __shfl_xor_sync(0xffffffffu, ay[0], o);
                az[0] += __shfl_xor_sync(0xffffffffu, az[0], o);
                if (POT) ph[0] += __shfl_xor_sync(0xffffffffu, ph[0], o);
            }
            if (has[0] && sub == 0) {
                const int kp = perm[S.slot_pos[slot[0]]];
                acc[3 * size_t(kp)] = ax[0];
                acc[3 * size_t(kp) + 1] = ay[0];
                acc[3 * size_t(kp) + 2] = az[0];
                if (POT) pot[kp] = ph[0];
            }
            if (has[1]) {
                const int kp = perm[S.slot_pos[slot[1]]];
                acc[3 * size_t(kp)] = ax[1];
                acc[3 * size_t(kp) + 1] = ay[1];
                acc[3 * size_t(kp) + 2] = az[1];
                if (POT) pot[kp] = ph[1];
            }
        }
        __syncwarp();
        }  // batches
    }
}

}  // namespace

void Octree::prepare_walk(const uint8_t* active, cudaStream_t s, int chunk, const double* aold, float alpha,
                          float alpha_q) {
    Context& C = ctx();
    TreeCounts* cnt = counts.as<TreeCounts>();
    GF_CUDA(cudaMemsetAsync(&cnt->num_work, 0, 2 * sizeof(int), s));  // num_work, walk_next
    GF_CUDA(cudaMemsetAsync(&cnt->pairs, 0, 2 * sizeof(unsigned long long), s));  // pairs, qpairs
    ProfScope ps(kStGroupPrep, s);
    // items: one per group (<= nodes), or at most one per active particle with chunks
    const size_t cap = std::max(size_t(node_cap), size_t(n)) + 1;
    active_ptr = active;
    // chunk > kChunkMax (active sets): runs of sibling groups merged by active count
    const bool by_active = active && chunk > kChunkMax;
    if ((quad && merge_cap > 0 && !(active && chunk > 0)) || by_active) {
        // merged items in tree order (flag, scan, fill), walked 4 regions at a time: 2 % faster
        // per evaluation than the order of appending warps, 6 % faster than 1 region, 9 % than 8
        const int span = std::max(node_cap, 1);
        int* fl = gflag.get<int>(span);
        int* sl = gscan.get<int>(span);
        const int blocks = std::min(div_up(span, 8), 16 * C.sms);
        const int cap_w = by_active ? merged_active_cap(chunk) : merge_cap;
        int* gw = nullptr;
        if (by_active) {
            gw = gweight.get<int>(span);
            k_group_nact<<<blocks, 256, 0, s>>>(groups.as<int>(), n_i4.as<int4>(), perm.as<int>(), active, cnt, gw);
            GF_CHECK_LAUNCH();
        }
        k_item_flag<<<blocks, 256, 0, s>>>(groups.as<int>(), n_i4.as<int4>(), n_parent.as<int>(), gw, cnt, cap_w,
                                           span, fl, C.d_status);
        GF_CHECK_LAUNCH();
        exclusive_scan(fl, sl, span, &cnt->num_work, s, &scratch);
        k_item_fill<<<blocks, 256, 0, s>>>(groups.as<int>(), n_i4.as<int4>(), n_parent.as<int>(), gw,
                                           active != nullptr, cnt, cap_w, fl,
                                           sl, p4.as<float4>(), perm.as<int>(), active,
                                           alpha > 0.f ? aold : nullptr, alpha, alpha_q, work.get<int4>(cap),
                                           sphere.get<float4>(cap), quad ? item_gam.get<float2>(cap) : nullptr);
        GF_CHECK_LAUNCH();
        walk_stride = 4;
        return;
    }
    walk_stride = 1;
    // The grid also fixes the order of this work list (each warp appends its groups' items as
    // it goes), which the walk follows; 4 blocks per SM was the best of 2 to 8 for the merged
    // items before they were written in tree order. Items of an active set: as many blocks as
    // fit on the SMs, so that the warps' passes over the groups (most without a particle due)
    // are short.
    static int prep_fit = 0;
    if (!prep_fit) GF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&prep_fit, k_group_prep, 256, 0));
    const int prep_blocks = (active && chunk > 0 ? std::max(prep_fit, 4) : 4) * C.sms;
    k_group_prep<<<prep_blocks, 256, 0, s>>>(groups.as<int>(), n_i4.as<int4>(), p4.as<float4>(),
                                          perm.as<int>(), active, cnt, work.get<int4>(cap),
                                          sphere.get<float4>(cap), active ? chunk : 0,
                                          quad && alpha > 0.f ? aold : nullptr, alpha, alpha_q,
                                          quad ? item_gam.get<float2>(cap) : nullptr);
    GF_CHECK_LAUNCH();
}

namespace {

// Launch shapes of the mixed walk (2 nodes per lane and round): warps per block and tile size.
// Every shape keeps its static shared memory under 48 KB per block (8 warps of the large tiles
// would not).

template <int WARPS, bool SMALL>
void launch_quad_walk(const Octree& T, const uint8_t* active, float eps2, double* acc, cudaStream_t s) {
    static int bps = 0;
    if (!bps) {
        GF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_walk<true, false, 2, WARPS, SMALL>, WARPS * 32,
                                                              0));
        bps = std::max(1, bps);
    }
    k_walk<true, false, 2, WARPS, SMALL><<<bps * ctx().sms, WARPS * 32, 0, s>>>(
        T.w_a.as<float4>(), T.w_b.as<float4>(), T.w_q.as<float4>(), T.w_t.as<float2>(), T.w_rq.as<float>(),
        T.p4.as<float4>(), T.perm.as<int>(), active, T.work.as<int4>(), T.sphere.as<float4>(),
        T.item_gam.as<float2>(), T.counts.as<TreeCounts>(), T.node_cap, eps2, acc, ctx().d_status, T.walk_stride);
}

}  // namespace

void Octree::walk(double eps, double* acc, cudaStream_t s, double* pot, int npl, int shape) {
    Context& C = ctx();
    const float eps2 = float(eps * eps);
    static int bps_mono = 0, bps_quad = 0;
    if (!bps_mono) {
        GF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps_mono, k_walk<false>, kWalkWarps * 32, 0));
        GF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps_quad, k_walk<true>, kWalkWarps * 32, 0));
        bps_mono = std::max(1, bps_mono);
        bps_quad = std::max(1, bps_quad);
    }
    ProfScope ps(kStWalk, s);
    last_walked() = this;
    if (pot) {
        if (quad) throw Error(GF_ERR_ARG, "potentials come from the monopole walk");
        k_walk<false, true><<<bps_mono * C.sms, kWalkWarps * 32, 0, s>>>(
            w_a.as<float4>(), w_b.as<float4>(), nullptr, nullptr, nullptr, p4.as<float4>(), perm.as<int>(), active_ptr,
            work.as<int4>(), sphere.as<float4>(), nullptr, counts.as<TreeCounts>(), node_cap, eps2, acc, C.d_status,
            walk_stride, pot);
    } else if (quad && npl > 2) {
        k_walk<true, false, 8><<<bps_quad * C.sms, kWalkWarps * 32, 0, s>>>(
            w_a.as<float4>(), w_b.as<float4>(), w_q.as<float4>(), w_t.as<float2>(), w_rq.as<float>(), p4.as<float4>(),
            perm.as<int>(), active_ptr, work.as<int4>(), sphere.as<float4>(), item_gam.as<float2>(),
            counts.as<TreeCounts>(), node_cap, eps2, acc, C.d_status, walk_stride);
    } else if (quad) {
        switch (shape) {
            case 1: launch_quad_walk<2, false>(*this, active_ptr, eps2, acc, s); break;
            case 2: launch_quad_walk<4, true>(*this, active_ptr, eps2, acc, s); break;
            case 3: launch_quad_walk<2, true>(*this, active_ptr, eps2, acc, s); break;
            default: launch_quad_walk<4, false>(*this, active_ptr, eps2, acc, s); break;
        }
    } else {
        k_walk<false><<<bps_mono * C.sms, kWalkWarps * 32, 0, s>>>(
            w_a.as<float4>(), w_b.as<float4>(), nullptr, nullptr, nullptr, p4.as<float4>(), perm.as<int>(), active_ptr,
            work.as<int4>(), sphere.as<float4>(), nullptr, counts.as<TreeCounts>(), node_cap, eps2, acc, C.d_status,
            walk_stride);
    }
    GF_CHECK_LAUNCH();
}

}  // namespace gf
