// gf_tree.cuh — device octree: Morton-key build that reproduces the reference's tree,
// refit, walk groups and the walk layout.
#pragma once

#include "gf_common.cuh"

namespace gf {

constexpr int kLeafMax = 8;      // cpp/nbody.cpp:33
constexpr int kGroupMax = 64;    // cpp/nbody.cpp:34
constexpr int kDepthMax = 48;    // cpp/nbody.cpp:35
constexpr int kKeyLevels = 21;   // levels held by one 63-bit Morton key word
constexpr int kDeepRunMax = 4096;
// launch shapes of the mixed walk: warps per block x interaction tiles (particle / node
// entries per warp): 0 = 4 x 256/96, 1 = 2 x 256/96, 2 = 4 x 128/64, 3 = 2 x 128/64
constexpr int kNumWalkShapes = 4;

// Root cube and the fixed-point grid used by the fast key path.
struct RootBox {
    double c[3];
    double half;
    double lo[3];     // c - half
    double inv_w;     // 2^21 / (2 half): grid units per unit length
    double margin;    // grid units: closer than this to a cell wall -> exact path
    double inv_w32;   // inv_w * 2^32: 32.32 fixed-point grid units per unit length
    uint32_t m_lo, m_hi;  // fixed-point fraction window that is at least `margin` from a wall
};

// Small device-side counters read back once per build.
struct TreeCounts {
    int total_nodes;
    int deep;         // some level-21 cell holds more than kLeafMax particles
    int num_groups;
    int num_work;
    int walk_next;    // dynamic scheduler of the walk
    int deep_runs;    // level-21 cells holding more than the leaf capacity (their first positions)
    int reserved;
    int bbox_done;    // blocks of the bounding-box pass that have written their partials
    unsigned long long pairs;   // list interactions evaluated by the last walk (all kinds)
    unsigned long long qpairs;  // of which with quadrupole nodes (mixed form)
};

struct Octree {
    int n = 0;        // particles
    int nn = 0;       // nodes
    int ng = 0;       // groups
    int max_depth = 0;
    int node_cap = 0; // node buffers are sized to this (grows with headroom, never shrinks)
    float theta_f = 0.7f;
    bool valid = false;
    const uint8_t* active_ptr = nullptr;  // active flags of the current walk (device)

    // particles (tree order unless noted)
    DevBuf key, key_alt, perm, perm_alt, key1, key2, p4, xbuild, pdisp;
    DevBuf cpl9, ldepth, dsplit, nstart, nbase, node_owner;
    // nodes, depth-first (preorder) order
    DevBuf n_i4;      // int4 {start, count, next, leaf | depth << 8}
    DevBuf n_mom;     // float4 {cx, cy, cz, m}
    DevBuf n_open;    // float open_r
    DevBuf n_geo;     // float4 {gx, gy, gz, half}
    DevBuf n_cd;      // double4 {centre, half} (build only)
    DevBuf n_parent, n_nchild, n_counter, n_disp, n_bfs;
    DevBuf n_kids;    // children of each node in octant order (8 slots per node)
    // walk layout, breadth-first order: children of a node are contiguous
    DevBuf w_a;       // float4 {cx, cy, cz, m}
    DevBuf w_b;       // float4 {open_r, first (int bits), code (int bits), rho};
                      //   code > 0: internal, `code` children from BFS index `first`;
                      //   code < 0: leaf, -code particles from tree position `first`;
                      //   rho (quadrupole trees, else 0) = (M b^3)^(1/5), b = |com - cell centre|
                      //   + sqrt(3) (half + displacement): the relative opening radius
    DevBuf w_geo;     // float4 {gx, gy, gz, half} of the cell, breadth-first order
    DevBuf w_q;       // float4 {Qxx, Qyy, Qxy, Qxz} (quadrupole trees)
    DevBuf w_t;       // float2 {Qyz, T = sum m |d|^2 about the centre of mass} (quadrupole trees)
    DevBuf w_rq;      // float (M b^2)^(1/4): the quadrupole-order radius (quadrupole trees)
    DevBuf bfs_key, bfs_key_alt, bfs_val, bfs_val_alt;
    // neighbour search extras (tree order): float32 remainders x - float(x) and the
    // breadth-first index of each particle's leaf
    DevBuf plo, leaf_of, w_parent;
    bool want_knn = false;
    int group_max = kGroupMax;   // walk groups: shallowest nodes with <= group_max particles
    int merge_cap = 0;           // quadrupole trees: walk items = runs of consecutive sibling
                                 // groups of <= merge_cap particles (0: one item per group)
    int leaf_max = kLeafMax;     // leaf capacity (the reference's 8 for gravity trees)
    bool quad = false;           // also build quadrupole moments (mixed-precision form)
    bool kahan = false;          // walk: compensated accumulation of the tile sums
    // groups and walk work list (gweight: active particles per group, for items merged by
    // active count)
    DevBuf gflag, gscan, groups, work, sphere, gweight;
    DevBuf item_gam;  // per work item: float2 {(alpha a_min)^(-1/5), (alpha_q a_min)^(-1/4)}, 0 = off
    int walk_stride = 1;  // regions of the work list the walk takes at a time (prepare_walk sets it)
    DevBuf root, counts;
    ScanScratch scratch;  // this tree's scan / sort scratch (trees may build on different streams)
    TreeCounts* h_counts = nullptr;  // pinned
    // node count of the last build outside a captured graph, copied to the host behind it
    // (read once the copy is done): a synchronisation-free rebuild bounds the tree by node_cap,
    // so the caller does a regular build (which re-sizes the node buffers) once the tree grows
    // close to it
    int* h_live = nullptr;           // pinned
    cudaEvent_t live_ev = nullptr;
    bool live_pending = false;
    bool outgrowing();

    // graph_safe: no host synchronisation and no allocation (inside a captured CUDA graph):
    // needs a regular build of the same particle set first (node_cap from it; a tree that
    // outgrows node_cap raises GF_ERR_CAPACITY and is left empty).
    void build(int n, const double* pos, const double* mass, double theta, cudaStream_t s,
               bool graph_safe = false);
    void reserve_graph_build();
    void deep_sort_attr();
    // Node kernels read the live node count on the device (valid after captured rebuilds).
    // s_moments (with the event `gathered`): the moments run on that stream once the gathered
    // positions are ready, and the caller joins it before reading them (the walk items, which
    // need the positions only, can be prepared on s meanwhile).
    void refit(const double* pos, const double* mass, cudaStream_t s, cudaStream_t s_moments = nullptr,
               cudaEvent_t gathered = nullptr);
    // Work list of groups with at least one active particle (active may be null); chunk in
    // 1..kChunkMax cuts each group's active particles into items of <= chunk with their own
    // spheres; chunk in kChunkMax+1..kChunkCodeMax (active sets) merges runs of sibling groups
    // into items of <= merged_active_cap(chunk) active particles, each with the bounding
    // sphere of its active particles.
    // aold (quadrupole trees, may be null): the previous accelerations (n,3) in original order,
    // for the relative opening criterion with tolerance alpha.
    // alpha_q > 0: accepted nodes whose quadrupole term is below alpha_q a_min are taken as
    // monopoles.
    void prepare_walk(const uint8_t* active, cudaStream_t s, int chunk = 0, const double* aold = nullptr,
                      float alpha = 0.f, float alpha_q = 0.f);
    // pot (monopole trees, may be null): softened potentials of the walked particles
    // npl: nodes per lane and round of the mixed walk (2, or 8 for walks of a few items)
    // shape: launch shape of the mixed walk with npl 2 (kNumWalkShapes)
    void walk(double eps, double* acc, cudaStream_t s, double* pot = nullptr, int npl = 2, int shape = 0);
};

// Walk item codes (prepare_walk's chunk): 1..kChunkMax chunks of one group's active particles,
// kChunkMax+1..kChunkCodeMax sibling-group runs merged by active count.
constexpr int kChunkMax = 64;
constexpr int kChunkCodeMax = 96;
__host__ __device__ inline int merged_active_cap(int chunk) { return 2 * (chunk - kChunkMax); }

Octree& gravity_tree();
// The tree walked most recently (for the pair counter).
Octree*& last_walked();

}  // namespace gf
