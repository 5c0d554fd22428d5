// gf_sph.cuh — internal entry points shared by the C ABI (gf_capi.cu).
#pragma once

#include "gf_tree.cuh"

namespace gf {

struct SphScratch {
    DevBuf pr2, cs;
};

void sph_kernel_values(int n, const double* r, const double* h, double* w, double* dw, cudaStream_t s);

// nb: (n, ld) neighbour indices, the first k of each row used.
template <class Idx>
void sph_forces(SphScratch& S, int n, int k, int ld, const double* pos, const double* vel, const double* mass,
                const Idx* nb, const double* h, const double* u, double gamma, double alpha,
                double beta, double* rho, double* acc, double* dudt, double* dt_i, cudaStream_t s,
                float* divv = nullptr, Subset sub = Subset());

// Inputs of the learned smoothing-length guess inside a neighbour search: X (n x 4) receives
// the features; with use_mlp the network's predicted distance of the k-th nearest, times a
// small margin, gives the starting radius (the library uses it for searches without a
// previous h); dk (if set) receives the converged distances of the k-th nearest, the training
// targets.
struct HGuess {
    const int* gidx;      // caller index -> global particle index (null: identity)
    const double* hprev;  // previous h per global index (null: none)
    const float* divv;    // previous velocity divergence per global index (null: none)
    float* X;             // n x 4 features (out)
    float* Y;             // n predictions (scratch)
    float* rg;            // n starting radii (scratch)
    bool use_mlp;
    float* dk;            // n distances of the k-th nearest (out, training targets), or null
};

// log h of the cell-density start (radius side (k / count)^(1/3), over the 2.5 that relates a
// previous h to its search radius) from the first feature f0 = log(count / side^3): the
// stand-in for the previous h of a particle that has none.
__host__ __device__ inline float cold_log_h(float f0, int k) {
    return (logf(float(k)) - f0) * (1.0f / 3.0f) - logf(2.5f);
}

struct Sph32Scratch {
    DevBuf A, B, C, D;
};

// Mixed-precision sph_forces (float32 arithmetic, Kahan sums; float64 in and out). order
// (optional): the visiting order of the particles. sub (both forms): only these particles get
// new density, forces and Courant step (the others keep theirs, and serve as neighbours).
template <class Idx>
void sph_forces32(Sph32Scratch& S, int n, int k, int ld, const int* order, const double* pos, const double* vel,
                  const double* mass, const Idx* nb, const double* h, const double* u, double gamma, double alpha,
                  double beta, double* rho, double* acc, double* dudt, double* dt_i, cudaStream_t s,
                  float* divv = nullptr, Subset sub = Subset());

void knn_from_candidates(int n, int m, const double* pos, const int64_t* cand, int k, int64_t* nb,
                         double* dist, int* d_ok, cudaStream_t s);

// Exact float64 k nearest neighbours of every point (itself included), ascending; builds
// the point octree in T. r_guess (caller order, optional): starting search radius.
// Outputs either nb/dist (n,k) int64/float64, or nb32 (n, ld32) int32 plus the distance of
// neighbour `dsel_col` in dsel (n,) — or, with dsel_idx, that neighbour's index (the caller
// measures its float64 distance; -1 for a failed query). same_set: the points are those of the
// last search on T, moved (the tree is rebuilt without a host synchronisation).
void knn_exact(Octree& T, int n, const double* pos, int k, const float* r_guess, int64_t* nb,
               double* dist, unsigned long long* d_iters, cudaStream_t s, int* nb32 = nullptr,
               int ld32 = 0, double* dsel = nullptr, int dsel_col = -1, const HGuess* hg = nullptr,
               bool same_set = false, int* dsel_idx = nullptr);

void direct_sum(int n, const double* pos, const double* mass, int nt, const int64_t* targets,
                double* acc, double eps, cudaStream_t s);

// Seeded initial conditions on the device (gf_ic.cu): kind 0 the rotating 1/r cloud, 1 the
// disk + 1/r halo (+ Plummer clumps); prm: the 13 values documented at gf_ic_generate_dev.
void ic_generate(int kind, int n_gas, int n_dm, uint64_t seed, const double* prm, double* pos, double* vel,
                 double* mass, int8_t* kind_out, double* u, cudaStream_t s);

void render_splat(int n, const double* pos, const uint8_t* group, int ngroups, const double* rot,
                  const double* center, double scale, int W, int H, float* img, cudaStream_t s);
void render_tonemap(int W, int H, int ngroups, const float* img, const float* glow, int gw, int gh,
                    const float* colors, float inv_ref, float K, float exposure, uint8_t* out,
                    cudaStream_t s);

}  // namespace gf
