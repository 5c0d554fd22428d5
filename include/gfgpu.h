/* gfgpu.h — C ABI of libgfgpu.so, the GB300 (sm_103a) gravity + SPH force library.
 *
 * Drop-in for the force path of HugoGW/Galaxy_formation:
 *   - the five extern "C" exports of cpp/nbody.cpp (bound with ctypes in
 *     galaxy_formation/engine.py:30-35), with identical names and signatures;
 *   - the SPH entry points of galaxy_formation/sph.py (sph_forces, knn_from_candidates and
 *     the k-d tree query inside NeighbourFinder.find), as plain-pointer C functions.
 *
 * Conventions. Pointers of the reference-compatible functions are HOST pointers (the
 * library copies to and from the GPU). Functions with the `_dev` suffix take DEVICE
 * pointers and a CUDA stream (cudaStream_t passed as void*, NULL = the library's stream;
 * cudaStreamLegacy, (void*)1, for the legacy default stream);
 * they enqueue work and return without synchronising unless stated. Arrays are
 * C-contiguous: positions (n,3) float64 row-major, etc.
 *
 * Errors. The reference's functions return void and have no error channel
 * (cpp/nbody.cpp:415-441). Every entry point here records a status: the int-returning
 * ones return it, and gf_last_status() returns the status of the last call (0 = ok,
 * otherwise a bitwise OR of GF_ERR_*); gf_last_error() gives a message. Kernels never
 * trap on bad input; they set a status bit and skip the offending work.
 */
#ifndef GFGPU_H
#define GFGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status bits */
#define GF_OK 0
#define GF_ERR_CUDA 1         /* a CUDA runtime call failed (message in gf_last_error) */
#define GF_ERR_ARG 2          /* invalid argument (negative size, null pointer, ...)  */
#define GF_ERR_NONFINITE 4    /* a position was NaN or infinite                        */
#define GF_ERR_WALK_STACK 8   /* tree-walk stack overflow: some accelerations skipped  */
#define GF_ERR_DEEP_CELL 16   /* more than 4096 particles share one cell below level 21 */
#define GF_ERR_KNN 32         /* neighbour search did not converge for some particles  */
#define GF_ERR_NO_DEVICE 64   /* no CUDA device                                        */
#define GF_ERR_CAPACITY 128   /* a fixed-capacity buffer was too small                 */
#define GF_ERR_TIMEOUT 256    /* a bounded device-side wait gave up (results invalid)   */

/* ---- drop-ins for cpp/nbody.cpp (signatures identical to the reference) ---------------- */

/* Replaces nbody_num_threads (cpp/nbody.cpp:417): returns the number of SMs of the GPU
 * (the library's unit of parallelism), 0 when no GPU is usable. */
int nbody_num_threads(void);

/* Replaces nbody_accel_active (cpp/nbody.cpp:422-425). Barnes-Hut accelerations (G = 1,
 * Plummer softening eps, opening angle theta) of the active particles (active[i] != 0, or
 * all when active is NULL), written into acc (n,3); other rows of acc are left untouched.
 * The octree always holds every particle and is kept on the GPU between calls:
 * rebuild = 0 refits the previous tree (same cells, new moments, opening radii enlarged
 * by the largest displacement since the build), unless n changed. Same tree, groups,
 * interaction lists and float32 arithmetic as the reference. */
void nbody_accel_active(int n, const double* pos, const double* mass, double* acc,
                        double theta, double eps, const uint8_t* active, int rebuild);

/* Replaces nbody_accel_direct (cpp/nbody.cpp:428-441): exact O(N^2) float64 sum. */
void nbody_accel_direct(int n, const double* pos, const double* mass, double* acc,
                        double eps);

/* Replaces nbody_render (cpp/nbody.cpp:445-469): orthographic bilinear deposit of the
 * first n particles into img (ngroups, H, W), float32. */
void nbody_render(int n, const double* pos, const uint8_t* group, int ngroups,
                  const double* rot, const double* center, double scale, int W, int H,
                  float* img);

/* Replaces nbody_tonemap (cpp/nbody.cpp:474-503): log tone map + glow + soft saturation
 * of the per-group images to 8-bit RGB out (H, W, 3). */
void nbody_tonemap(int W, int H, int ngroups, const float* img, const float* glow, int gw,
                   int gh, const float* colors, float inv_ref, float K, float exposure,
                   uint8_t* out);

/* ---- status ------------------------------------------------------------------------- */

/* Status of the last call (GF_OK or GF_ERR_* bits); synchronises the library stream. No
 * reference counterpart: the reference has no error channel (cpp/nbody.cpp:415-441). */
int gf_last_status(void);
/* Message of the last failure ("" when none). No reference counterpart. */
const char* gf_last_error(void);
/* Number of octree nodes and walk groups of the current gravity tree (for tests). */
int gf_tree_size(int* num_nodes, int* num_groups);
/* Copies the current gravity tree out in the reference's depth-first node order
 * (cpp/nbody.cpp:38-45 layout, split): ints (nn,4) = start, count, next, leaf;
 * floats (nn,9) = cx, cy, cz, m, open_r, gx, gy, gz, half; order (n,) tree position ->
 * particle index (cpp/nbody.cpp:62 idx); groups (ng,) node ids (cpp/nbody.cpp:235-243).
 * Host pointers. No reference counterpart (test hook). */
int gf_tree_export(int32_t* ints, float* floats, int32_t* order, int32_t* groups);
/* Rebuilds the gravity tree from pos / mass (host pointers) inside a captured CUDA graph —
 * the synchronisation-free build that the batched form (gf_sim_blocks) replays — and runs
 * it once. The tree must already hold n particles (e.g. from nbody_accel_active with
 * rebuild), whose node buffers bound the new tree (GF_ERR_CAPACITY if it outgrows them).
 * No reference counterpart (test hook: gf_tree_export then shows the captured build). */
int gf_tree_rebuild_captured(int n, const double* pos, const double* mass, double theta);

/* ---- device-resident gravity -------------------------------------------------------- */

/* nbody_accel_active on device pointers (same semantics). */
int gf_accel_active_dev(int n, const double* pos, const double* mass, double* acc,
                        double theta, double eps, const uint8_t* active, int rebuild,
                        void* stream);
/* nbody_accel_direct on device pointers. */
int gf_accel_direct_dev(int n, const double* pos, const double* mass, double* acc,
                        double eps, void* stream);
/* Direct float64 sum for nt target particles (indices into pos) against all n sources;
 * acc is (nt,3). Host pointers. Same arithmetic as nbody_accel_direct
 * (cpp/nbody.cpp:428-441), for error reports at sizes where O(N^2) is too slow. */
int gf_accel_direct_targets(int n, const double* pos, const double* mass, int nt,
                            const int64_t* targets, double* acc, double eps);

/* ---- SPH (galaxy_formation/sph.py) --------------------------------------------------- */

/* Vectorised kernel(r, h) and kernel_grad(r, h) of sph.py:31-54 (either output may be
 * NULL). Host pointers. */
int gf_sph_kernel(int n, const double* r, const double* h, double* w, double* dw);

/* Replaces sph_forces (sph.py:57-106): density, pressure + artificial-viscosity
 * acceleration, du/dt and Courant time step of n gas particles with k neighbours each
 * (nb (n,k) local indices, the particle itself included). Host pointers; outputs rho (n),
 * acc (n,3), dudt (n), dt_i (n). float64 arithmetic as in the reference. */
int gf_sph_forces(int n, int k, const double* pos, const double* vel, const double* mass,
                  const int64_t* nb, const double* h, const double* u, double gamma,
                  double alpha, double beta, double* rho, double* acc, double* dudt,
                  double* dt_i);
/* sph_forces in the mixed-precision form (no reference counterpart): the same formulas in
 * float32 arithmetic with hi/lo split positions and Kahan-compensated neighbour sums;
 * float64 inputs and outputs, host pointers, same arguments as gf_sph_forces. */
int gf_sph_forces_mixed(int n, int k, const double* pos, const double* vel, const double* mass,
                        const int64_t* nb, const double* h, const double* u, double gamma,
                        double alpha, double beta, double* rho, double* acc, double* dudt,
                        double* dt_i);

/* Particles accepted by gf_sph_forces_noalloc_dev (its fixed scratch: 16 bytes each). */
#define GF_SPH_NOALLOC_MAX_N 262144

/* sph_forces on device pointers. Every neighbour row is checked on the device before it is
 * read through: a particle whose row holds an index outside [0, n) gets NaN outputs (and so
 * do the particles that have it as a neighbour), and GF_ERR_ARG is reported by the next
 * synchronising call (e.g. gf_last_status). */
int gf_sph_forces_dev(int n, int k, const double* pos, const double* vel, const double* mass,
                      const int64_t* nb, const double* h, const double* u, double gamma,
                      double alpha, double beta, double* rho, double* acc, double* dudt,
                      double* dt_i, void* stream);

/* gf_sph_forces_dev without any device allocation (no reference counterpart: the reference
 * runs on the CPU and never faces this). For callers that cannot call cudaMalloc — a host
 * whose memory pool owns the GPU, or a step loop that must not allocate because
 * cudaMalloc/cudaFree synchronise the device. Inputs and outputs are the caller's device
 * buffers; the per-particle scratch is a fixed array inside the library, so n is limited to
 * GF_SPH_NOALLOC_MAX_N (larger n returns GF_ERR_CAPACITY without launching anything). The
 * first call on a device looks up that array's device address (cudaGetSymbolAddress); make
 * that first call before any stream capture. All calls share the one array: calls that
 * overlap on the GPU (different streams, or different host threads) race and must be
 * serialised by the caller. stream: cudaStream_t as void*, NULL = the legacy default
 * stream. Returns GF_OK or GF_ERR_* bits; enqueues work without synchronising. Neighbour
 * rows are checked on the device as in gf_sph_forces_dev; with no status word to write, a
 * row holding an index outside [0, n) shows only as NaN outputs of its particle (and of the
 * particles that have it as a neighbour). The fixed array's device address is looked up
 * once per device and kept for the life of the process: it does not survive
 * cudaDeviceReset or a reset of the device's primary context. */
int gf_sph_forces_noalloc_dev(int n, int k, const double* pos, const double* vel,
                              const double* mass, const int64_t* nb, const double* h,
                              const double* u, double gamma, double alpha, double beta,
                              double* rho, double* acc, double* dudt, double* dt_i, void* stream);

/* Replaces knn_from_candidates (sph.py:109-135): the k nearest of each particle among its
 * m candidates (cand (n,m) local indices, -1 = none), ascending, into nb (n,k) and dist
 * (n,k). Returns 1 when every particle had at least k candidates, 0 otherwise (rows of
 * such particles are left untouched), or -GF_ERR_* on failure. Host pointers. */
int gf_knn_from_candidates(int n, int m, const double* pos, const int64_t* cand, int k,
                           int64_t* nb, double* dist);

/* Replaces cKDTree(pos).query(pos, k) inside NeighbourFinder.find (sph.py:165-166): the
 * exact k nearest points of every point (itself included), ascending distance, into dist
 * (n,k) and nb (n,k). 1 <= k <= 64, k <= n. Host pointers. */
int gf_knn(int n, const double* pos, int k, double* dist, int64_t* nb);
/* Total search-radius iterations of the last gf_knn call, summed over particles (the
 * neighbour-count iteration). No reference counterpart. */
long long gf_knn_iterations(void);

/* ---- fused force evaluation (galaxy_formation/simulation.py:61-95) ------------------- */

/* One GalaxyFormation.accelerations(active, rebuild, sph, fresh_nb) call on device
 * pointers: Barnes-Hut gravity of the active particles (into a persistent internal
 * acc_grav), then, when sph != 0, the hydro step of simulation.py:74-95 for every particle
 * with kind == 0 (gas): neighbour search (fresh_nb != 0: full 48-candidate search; else
 * Verlet reselection among the cached candidates, falling back to a full search as
 * sph.py:155-166 does), h = max(d_32 / 2, eps / 2), sph_forces, scatter. Outputs acc (n,3)
 * = acc_grav + acc_sph and dt_ind (n,) = min(0.3 sqrt(eps / |a|), dt_courant). kind is
 * (n,) int8 (0 gas, 1 star, 2 dark matter), u (n,) specific internal energy. State (tree,
 * neighbour cache, acc_grav, acc_sph, dt_courant) persists between calls and is reset when
 * n changes. */
int gf_accelerations_dev(int n, const double* pos, const double* vel, const double* mass,
                         const int8_t* kind, const double* u, double theta, double eps,
                         double gamma, double alpha, double beta, const uint8_t* active,
                         int rebuild, int sph, int fresh_nb, double* acc, double* dt_ind,
                         void* stream);
/* gf_accelerations_dev on host pointers (copies in and out, synchronises). */
int gf_accelerations(int n, const double* pos, const double* vel, const double* mass,
                     const int8_t* kind, const double* u, double theta, double eps, double gamma,
                     double alpha, double beta, const uint8_t* active, int rebuild, int sph,
                     int fresh_nb, double* acc, double* dt_ind);
/* ---- initial conditions on the device ------------------------------------------------ */

/* Seeded particle sets generated on the GPU (the reference builds its initial cloud on the
 * host, galaxy_formation/initial_conditions.py:25-68; the disk + halo snapshot has no
 * reference counterpart). kind 0: the rotating cloud of initial_conditions.py:33-68 (both
 * species in a 1/r sphere of radius R0, rotation from the spin parameter, 10 % velocity
 * dispersion, no bulk motion, gas at u_gas); kind 1: a 1/r dark-matter halo, an exponential
 * gas disk (scale length rd truncated at 12 rd, sech^2 height z0) holding disk_frac of the
 * gas, of which n_clumps Plummer spheres (each clump_frac of the gas, radius a_clump, centres
 * in the disk) are carved out, the rest of the gas in the 1/r sphere; circular velocities
 * from the enclosed mass plus 10 % dispersion; gas energies log-uniform in [u_lo, u_hi].
 * params (code units, 13 values): M_tot, f_baryon, R0, spin, u_gas, disk_frac, rd, z0,
 * n_clumps, clump_frac, a_clump, u_lo, u_hi. Outputs: pos (n,3), vel (n,3), mass (n),
 * kind (n) (0 gas first, then 2 dark matter), u (n), n = n_gas + n_dm. Every draw is a
 * function of (seed, particle index, draw number), so a set depends only on its arguments.
 * The sets match the host generators (galaxy_formation_gb300/synthetic.py) in distribution,
 * not bit for bit. _dev: device pointers, enqueued on stream. */
int gf_ic_generate_dev(int kind, int n_gas, int n_dm, unsigned long long seed, const double* params,
                       int nparams, double* pos, double* vel, double* mass, int8_t* kind_out, double* u,
                       void* stream);
/* gf_ic_generate_dev into host arrays (copies out, synchronises). */
int gf_ic_generate(int kind, int n_gas, int n_dm, unsigned long long seed, const double* params, int nparams,
                   double* pos, double* vel, double* mass, int8_t* kind_out, double* u);

/* ---- the step loop (galaxy_formation/simulation.py:114-149) ----------------------------- */

/* Loads a particle set onto the GPU (host pointers, copied) and computes its initial
 * accelerations, as GalaxyFormation.__init__ does (simulation.py:51-54). kind: 0 gas,
 * 1 star, 2 dark matter. */
int gf_sim_init(int n, const double* pos, const double* vel, const double* mass,
                const int8_t* kind, const double* u, double theta, double eps, double gamma,
                double alpha, double beta);
/* One long step of the hierarchical kick-drift-kick leapfrog of GalaxyFormation.step
 * (simulation.py:114-149), device-resident, without the sub-grid physics hooks
 * (_thermodynamics, _stars). taken: its length; substeps: sub-steps done (1 for a global
 * step). */
int gf_sim_step(double dt_max, double* taken, int* substeps);
/* The batched form of the step loop (no reference counterpart): block time steps. Each
 * particle sits on a power-of-two level j (step 2^j delta, delta = min dt_ind, j =
 * floor(log2(dt_ind / delta)) clamped to [0, nlev-1]); a block is 2^(nlev-1) finest
 * sub-steps, at each of which only the particles due (s mod 2^j == 0) get new forces
 * (gravity on the refitted tree, SPH with the neighbours' last densities) and kicks. The
 * inner sub-steps of a block run as one captured CUDA graph; block boundaries rebuild the
 * tree and search neighbours afresh. updates: particle-updates done (forces computed). */
int gf_sim_blocks(int nblocks, int nlev, double* updates);
/* Launch shape of gf_sim_blocks per sub-step bin (bin b = sub-steps whose index has b
 * trailing zero bits, i.e. levels 0..b due): chunk[b] = active particles per walk item
 * (0: the reference's walk groups with their spheres; 1..64: items of <= chunk[b] active
 * particles of one group in tree order, each with its own bounding sphere; 65..96: runs of
 * consecutive sibling groups merged into items of <= 2 (chunk[b] - 64) active particles, each
 * with the bounding sphere of its active particles), plus 100 to walk with 8 nodes
 * per lane and round instead of 2 (mixed form; for bins of a few items, whose walks are bound
 * by the latency of their rounds), plus 1000 x s to walk with launch shape s
 * (GF_OPT_WALK_SHAPE, 2 per lane only); bins past nbins reuse chunk[nbins-1]; chunk NULL =
 * groups everywhere. rebuild_every > 0 rebuilds the tree inside the captured block every
 * that many sub-steps (0: refit only). */
int gf_sim_block_config(const int* chunk, int nbins, int rebuild_every);
/* Autotuner of that launch shape on the current state: times the gravity walk of each bin's
 * active set per chunk candidate, walk width and launch shape, then one block per rebuild
 * cadence; keeps
 * the fastest and writes them to chunk (nlev-1 entries, in gf_sim_block_config's encoding) /
 * rebuild_every; graph_ms = the best block's graph time. Positions, velocities and time are restored afterwards (the next block starts with
 * a full evaluation). */
int gf_sim_block_autotune(int nlev, int* chunk, int* rebuild_every, double* graph_ms);
/* Fraction of the particles on each level 0..nlev-1 of the current block. */
int gf_sim_levels(int nlev, double* frac);
/* Particle-updates of the last gf_sim_step: particles that received freshly computed forces
 * (the active set of every force evaluation, plus all gas whenever SPH ran). */
double gf_sim_updates(void);
/* Conserved quantities of the current state, float64 (no reference counterpart): out[8] =
 * kinetic, potential, thermal (sum m u of the gas), total energy, angular momentum Lx, Ly, Lz,
 * time. The potential is 1/2 sum m phi with phi the softened potential of a monopole
 * Barnes-Hut walk at opening angle theta (a tree of its own); between blocks of
 * gf_sim_blocks the velocities are synchronised first (the next block's opening half-kick
 * taken off). */
int gf_sim_diagnostics(double theta, double* out);
/* Copies the state out (host pointers; any may be NULL): pos, vel, acc (n,3), dt_ind (n),
 * and the simulated time t. */
int gf_sim_read(double* pos, double* vel, double* acc, double* dt_ind, double* t);
/* Copies the specific internal energies u (n) of the simulation state out. */
int gf_sim_read_u(double* u);
/* out[3] = t, dt_grav, dt_gas of the step loop (the time and the global step limits that the
 * next gf_sim_step starts from). */
int gf_sim_read_scalars(double* out);
/* Density and du/dt of the last SPH evaluation per particle (n each; NaN outside its gas
 * set): the inputs of the next thermal update. */
int gf_sim_read_hydro(double* rho, double* dudt);
/* Exact resume of a checkpoint (no reference counterpart): after gf_sim_init of the saved
 * particle set (pos, vel, mass, kind, u at the end of a step), overwrites the state that
 * gf_sim_init recomputed with the saved one: accelerations acc (n,3) and dt_ind (n) of the
 * last evaluations, birth and no_cool_until, the last SPH evaluation's rho and du/dt (as
 * gf_sim_read_hydro gives them; these four may be NULL), t, dt_grav and dt_gas; the tree of
 * the next sub-steps is the one gf_sim_init built at the same positions. The run then goes on
 * as if it had not stopped. */
int gf_sim_restore(const double* acc, const double* dt_ind, const double* birth, const double* no_cool_until,
                   const double* rho, const double* dudt, double t, double dt_grav, double dt_gas);
/* Thermal update at the start of every step and sub-step of gf_sim_step, as
 * GalaxyFormation._thermodynamics (simulation.py:97-104) on the gas of the last SPH
 * evaluation: mode 0 = off (default), 1 = u += dt du/dt floored at u_floor (compression and
 * shock heating), 2 = 1 then radiative cooling of a primordial gas (cooling.py:34-43),
 * except for particles inside a supernova bubble (no_cool_until > t, from gf_sim_stars).
 * gf_sim_blocks applies the same update to each gas particle over its own step, at the
 * sub-steps where it is due, before its evaluation there.
 * units (mode > 0): 8 positive constants in this order: u_per_K, u_floor, RHO_CGS, X_H,
 * M_H, MYR, SEC_PER_MYR, U_CGS (galaxy_formation/units.py, simulation.py:40-42). */
int gf_sim_thermo(int mode, const double* units);
/* Star formation and supernova feedback after every step and sub-step of gf_sim_step, as
 * GalaxyFormation._stars (simulation.py:106-110, star_formation.py:35-65), on the device:
 * gas of the last SPH evaluation with rho > rho_sf and T < 3e4 K becomes a star (kind 1,
 * birth = t) when its uniform draw is below 1 - exp(-sf_eff dt / t_ff); each new star then
 * heats its fb_ngb nearest gas particles and blocks their cooling for fb_myr. The draws are
 * those of NumPy's Generator(PCG64): rng_state holds its bit generator's state and increment
 * (128-bit each) as 4 words: state high, state low, inc high, inc low; the dense particle of
 * rank r (ascending particle index) takes the stream's draw r + 1 and the stream advances by
 * the number of dense particles per call, exactly as rng.uniform(size=p.size), so the same
 * generator state gives the reference's stars. params (10, positive): rho_sf (code units),
 * sf_eff, fb_eff, fb_ngb (1..64), fb_myr / MYR (code units), E_SN_PER_MSUN (erg), MSUN,
 * MSUN_G, U_CGS, u_per_K. on = 0 turns it off (default). Block steps (gf_sim_blocks) form no
 * stars; their thermal update honours the bubbles. */
int gf_sim_stars(int on, const double* params, const uint64_t* rng_state);
/* Copies kind (n, int8), birth and no_cool_until (n, float64; inf / -inf where unset) and the
 * advanced PCG64 state (4 words) out; any may be NULL. Returns the number of stars formed
 * since gf_sim_init, or -GF_ERR_* on failure. */
long long gf_sim_read_stars(int8_t* kind, double* birth, double* no_cool_until, uint64_t* rng_state);
/* cooling.py:24-31 (host pointers): lam[i] = Lambda(T[i]) in erg cm^3 / s, 0 at or below
 * 1e4 K. */
int gf_cooling_function(int n, const double* T, double* lam);
/* cooling.py:34-43 elementwise (host pointers), with a step dt[i] per particle and blocked
 * (may be NULL) as the reference's bubble mask; units as for gf_sim_thermo (the first two are
 * not used: u_floor is passed explicitly). */
int gf_cool(int n, const double* u, const double* T, const double* rho, const double* dt,
            const uint8_t* blocked, double u_floor, const double* units, double* out);

/* Options of the fused force evaluation (no reference counterpart):
 *   GF_OPT_SPH_FLOAT32  0 = float64 SPH arithmetic (the reference's, default);
 *                       1 = mixed precision: float32 arithmetic with hi/lo split positions
 *                           and Kahan-compensated neighbour sums. */
#define GF_OPT_SPH_FLOAT32 0
/*   GF_OPT_GRAVITY_QUAD 0 = the reference's monopole Barnes-Hut (default);
 *                       1 = mixed form: nodes carry traceless quadrupoles (float32, Kahan
 *                           sums), accepted nodes are evaluated to quadrupole order and the
 *                           walk adds its tile sums with Kahan compensation. The fused path
 *                           keeps its own tree; nbody_accel_active is never affected. */
#define GF_OPT_GRAVITY_QUAD 1
/*   GF_OPT_HGUESS       start of the neighbour-count iteration of a full search:
 *                       0 = 2.5 x the previous h (default), falling back to the density of the
 *                       particle's tree cell when there is none (the first search of a particle
 *                       set); 1 = the cell density only; 2 = 2.5 x the previous h, and the
 *                       learned guess (gf_mlp_*) where there is none. The iteration always runs
 *                       to the exact 48 nearest, so only the iteration count changes. */
#define GF_OPT_HGUESS 2
/*   GF_OPT_COLLECT      capacity (rows) of a device buffer that every later full search with a
 *                       previous h fills with (features, log distance of the 48th nearest) pairs
 *                       for training, two rows per gas particle: its features, and the features it
 *                       would have without a previous h; setting it clears the buffer;
 *                       gf_get_option returns the rows kept. */
#define GF_OPT_COLLECT 3
/*   GF_OPT_WALK_CHUNK   walks of an active subset (gf_accel_active*, gf_accelerations with an
 *                       active mask): 0 = the reference's groups and spheres (default);
 *                       1..64 = items of <= that many active particles in tree order, each
 *                       with the bounding sphere of its own particles (no reference
 *                       counterpart: same opening criterion per particle, tighter spheres);
 *                       65..96 = runs of sibling groups merged into items of <= 2 (value - 64)
 *                       active particles, each with the sphere of its active particles. */
#define GF_OPT_WALK_CHUNK 4
/*   GF_OPT_WALK_GROUP   mixed form (GF_OPT_GRAVITY_QUAD = 1): walk groups are the shallowest
 *                       nodes holding <= this many particles, 8..128 (default 64, the
 *                       reference's kGroupMax of cpp/nbody.cpp:34, which the monopole walk
 *                       always keeps). */
#define GF_OPT_WALK_GROUP 5
/*   GF_OPT_GRAVITY_REL  mixed form (GF_OPT_GRAVITY_QUAD = 1): relative opening criterion with
 *                       tolerance alpha (0 = off, default; e.g. 2.5e-3). A node is accepted
 *                       for a walk group when its distance from the group's sphere exceeds
 *                       both the geometric radius at theta = 1 and (M b^3 / (alpha a_min))^(1/5),
 *                       where M b^3 bounds the node's octupole and a_min is the group's
 *                       smallest |gravity| of the previous evaluation of the same particle
 *                       set. Until the gravity of every particle has been evaluated once
 *                       (the first call, a new particle count, or after setting this option)
 *                       the geometric criterion at the caller's theta is used. Set the option
 *                       again before evaluating an unrelated particle set of the same size. */
#define GF_OPT_GRAVITY_REL 6
/*   GF_OPT_WALK_MERGE   mixed form: walk items are runs of consecutive sibling walk groups
 *                       (contiguous in tree order) holding <= this many particles, 0..128
 *                       (0 = one item per group, default). Each item has the bounding sphere
 *                       of its own particles and is walked once: fewer, larger walks. */
#define GF_OPT_WALK_MERGE 7
/*   GF_OPT_GRAVITY_REL_MONO  with the relative criterion on: an accepted node whose quadrupole
 *                       term, estimated as M b^2 / r^4, is below this tolerance times the
 *                       group's a_min is evaluated as a monopole alone (0 = off, default;
 *                       e.g. 1.5e-4). Far nodes then cost a monopole's arithmetic. */
#define GF_OPT_GRAVITY_REL_MONO 8
/*   GF_OPT_WALK_SHAPE   mixed form: launch shape of the walk (2 nodes per lane and round),
 *                       warps per block x interaction tiles (particle / node entries per
 *                       warp): 0 = 4 x 256/96 (default), 1 = 2 x 256/96, 2 = 4 x 128/64,
 *                       3 = 2 x 128/64. gf_force_autotune and gf_sim_block_autotune choose it. */
#define GF_OPT_WALK_SHAPE 9
/*   GF_OPT_FORGET_H     (any value) the next full neighbour search starts without the previous
 *                       smoothing lengths, as the first search of a particle set does. */
#define GF_OPT_FORGET_H 10
int gf_set_option(int key, double value);
/* Current value of an option (-1 for an unknown key). */
double gf_get_option(int key);
/* ---- learned smoothing-length guess (no reference counterpart) ----------------------- */
/* A 4 -> 64 -> 64 -> 1 ReLU MLP with bfloat16 weights and float32 accumulation predicting the log
 * distance of the 48th nearest gas neighbour (a full search starts at 1.06 times it)
 * from (log cell density, log previous h, leaf count, velocity divergence), standardised by
 * gf_mlp_set_norm; a particle without a previous h enters with the h its cell density implies
 * and a divergence of 0. Parameters: flat float32 vector of 4545 values, W1 (64x4), b1, W2 (64x64),
 * b2, w3 (64), b3. */
int gf_mlp_init(int seed);
int gf_mlp_set_params(const float* params);
int gf_mlp_get_params(float* params);
int gf_mlp_set_norm(const float* mean4, const float* std4, double t_mean, double t_std);
/* Predictions of n samples (X: n x 4), host pointers. Inference rounds the layer-2 inputs to
 * bfloat16 and runs layer 2 on the tensor cores (tcgen05) once the first call has checked
 * them against the CUDA-core kernel. */
int gf_mlp_predict(int n, const float* X, float* Y);
/* 1: inference uses the tensor cores; 0: the CUDA-core kernel (the check disagreed);
 * -1: not checked yet (no prediction since the weights were set). */
int gf_mlp_tensor_cores(void);
/* Gradient of 0.5 mean((y - t)^2) (standardised target t) over the n samples w.r.t. the flat
 * parameters, host pointers. */
int gf_mlp_gradient(int n, const float* X, const float* T, float* grad);
/* Copies up to max_rows collected training pairs (X rows of 4, T) to the host; returns the
 * rows copied (with X and T NULL: the rows available). */
long long gf_mlp_collected(float* X, float* T, long long max_rows);
/* Adam steps on random minibatches of the collected pairs; loss: the last minibatch's
 * mean loss in standardised units. */
int gf_mlp_train(int steps, int batch, double lr, double* loss);

/* Scalars of the last force evaluation: gas count, dt_grav = 0.3 sqrt(eps / max |a|),
 * dt_gas = min Courant step (inf without hydro), search-radius iterations of the last full
 * neighbour search. Any pointer may be NULL. Synchronises the device. */
int gf_force_info(int* n_gas, double* dt_grav, double* dt_gas, long long* knn_iters);
/* Autotuner of the mixed form's walk (no reference counterpart): on the tree, work items and
 * error scale of the last fused evaluation (which must have used GF_OPT_GRAVITY_QUAD), times the
 * gravity walk for each item size (GF_OPT_WALK_MERGE in {0, 24, 32, 40, 48, 64}) and launch
 * shape (GF_OPT_WALK_SHAPE 0..3), three times each, and sets both options to the fastest
 * (median time). Outputs (any may be NULL): the chosen merge cap and shape and that walk's
 * time in ms. Synchronises the device. */
int gf_force_autotune(double eps, int* walk_merge, int* walk_shape, double* walk_ms);
/* The gas state of the last hydro step of the fused evaluation (simulation.py:74-95: the
 * arrays _hydro builds for sph_forces), in gas-local order = np.flatnonzero(kind == 0):
 * global index, smoothing length h, density, du/dt, Courant step dt_i, SPH acceleration
 * (ng,3), and the 32 neighbours of each row (local indices, the set of the 32 nearest, in no
 * particular order). After a block sub-step only the gas due was recomputed; the other rows
 * hold their last values. *n_gas receives ng (0 when the last call had <= 40 gas); cap is the
 * row capacity of the arrays; any pointer may be NULL. Synchronises the device. No reference
 * counterpart (a read-out for checks against a CPU restatement). */
int gf_force_read_gas(int cap, int* n_gas, int32_t* gidx, double* h, double* rho, double* dudt,
                      double* dt_i, double* acc_sph, int32_t* nb32);
/* Up to nout statistics of the fused evaluation, in this order: gas count, dt_grav, dt_gas,
 * search-radius iterations of the last full search, 0 (reserved), full searches so far,
 * Verlet reselections so far, nodes of the gas octree, nodes of the gravity octree.
 * Synchronises the device. */
int gf_force_stats(double* out, int nout);

/* ---- measurement hooks (no reference counterpart) ----------------------------------- */

/* Starts (on != 0) or stops a profiling session; starting clears previous records. While
 * on, every stage below is bracketed by CUDA events recorded on its launching stream. */
int gf_profile(int on);
/* Stage ids: 0 gravity tree build, 1 refit, 2 walk kernel, 3 walk work list, 4 neighbour
 * search kernel, 5 gas octree build, 6 SPH density kernel, 7 SPH force kernel, 8 Verlet
 * reselection, 9 whole force evaluation, 10 radix sort of the gravity tree's keys, 11 node
 * emission of the gravity tree, 12 moments pass of the gravity tree build. Total milliseconds and number of launches
 * recorded in the session; synchronises the device. */
int gf_profile_stage(int stage, double* total_ms, int* launches);
/* Kernels launched by the library since it was loaded. */
long long gf_launch_count(void);
/* The library's own CUDA stream (cudaStream_t as void*), on which the host-pointer entry
 * points and the step loops run (NULL when no GPU is usable). */
void* gf_stream(void);
/* Particle-list pair interactions evaluated by the most recent gravity walk (synchronises). */
long long gf_walk_pairs(void);
/* Of those, the interactions with quadrupole nodes (mixed form; 0 for the monopole walk). */
long long gf_walk_quad_pairs(void);
/* Measures the float32 FFMA throughput of the GPU (TFLOP/s, an FMA counting 2 flops): the
 * roofline peak of the float32 walk. */
int gf_fp32_peak(double* tflops);

#ifdef __cplusplus
}
#endif

#endif /* GFGPU_H */
