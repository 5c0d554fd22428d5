// gf_capi.cu — extern "C" entry points of libgfgpu.so (declared in include/gfgpu.h).
//
// Host-pointer entry points keep the reference's calling convention (cpp/nbody.cpp:415-505
// via galaxy_formation/engine.py; galaxy_formation/sph.py): they copy inputs to the GPU,
// run the kernels on the library stream, copy results back and synchronise. `_dev` entry
// points take device pointers and only enqueue work.
#include <cmath>
#include <cstring>
#include <vector>

#include "gf_hydro.cuh"
#include "gf_mlp.cuh"
#include "gf_thermo.cuh"

namespace gf {
namespace {

struct Staging {
    DevBuf pos, mass, acc, active, vel, h, u, nb, rho, dudt, dt, dist, cand, r, w, dw;
    DevBuf img, glow, colors, rot, center, group, out, targets, flags, kind, dt_ind;
    DevBuf mlpX, mlpY, mlpT, mlpG;
};
Staging g_st;
SphScratch g_sph;
Sph32Scratch g_sph32;
Octree g_knn_tree;
unsigned long long g_knn_iters = 0;

template <class F>
int guarded(F&& f) {
    Context& c = ctx();
    c.last_status = 0;
    c.last_error.clear();
    try {
        ensure_ready();
        f();
    } catch (const Error& e) {
        c.last_status |= e.code;
        c.last_error = e.what();
    } catch (const std::exception& e) {
        c.last_status |= GF_ERR_CUDA;
        c.last_error = e.what();
    }
    return c.last_status;
}

inline cudaStream_t pick(void* stream) {
    return stream ? static_cast<cudaStream_t>(stream) : ctx().stream;
}

template <class T>
T* upload(DevBuf& b, const T* host, size_t count, cudaStream_t s) {
    T* d = b.get<T>(count);
    if (count) GF_CUDA(cudaMemcpyAsync(d, host, sizeof(T) * count, cudaMemcpyHostToDevice, s));
    return d;
}

template <class T>
void download(T* host, const T* dev, size_t count, cudaStream_t s) {
    if (count) GF_CUDA(cudaMemcpyAsync(host, dev, sizeof(T) * count, cudaMemcpyDeviceToHost, s));
}

void require(bool ok, const char* what) {
    if (!ok) throw Error(GF_ERR_ARG, what);
}

void accel_active_device(int n, const double* pos, const double* mass, double* acc, double theta,
                         double eps, const uint8_t* active, int rebuild, cudaStream_t s) {
    Octree& T = gravity_tree();
    if (rebuild || !T.valid || T.n != n)
        T.build(n, pos, mass, theta, s);
    else
        T.refit(pos, mass, s);
    T.prepare_walk(active, s, force_engine().walk_chunk);
    T.walk(eps, acc, s);
}

}  // namespace
}  // namespace gf

using namespace gf;

extern "C" {

int nbody_num_threads(void) {
    try {
        ensure_ready();
        return ctx().sms;
    } catch (...) {
        return 0;
    }
}

void nbody_accel_active(int n, const double* pos, const double* mass, double* acc, double theta,
                        double eps, const uint8_t* active, int rebuild) {
    guarded([&] {
        require(n >= 0, "n < 0");
        if (n == 0) return;
        require(pos && mass && acc, "null array");
        require(n < (1 << 27), "n too large");
        cudaStream_t s = ctx().stream;
        double* d_pos = upload(g_st.pos, pos, 3 * size_t(n), s);
        double* d_mass = upload(g_st.mass, mass, size_t(n), s);
        double* d_acc = upload(g_st.acc, acc, 3 * size_t(n), s);
        const uint8_t* d_act = active ? upload(g_st.active, active, size_t(n), s) : nullptr;
        accel_active_device(n, d_pos, d_mass, d_acc, theta, eps, d_act, rebuild, s);
        download(acc, d_acc, 3 * size_t(n), s);
        collect_status(s);
    });
}

void nbody_accel_direct(int n, const double* pos, const double* mass, double* acc, double eps) {
    guarded([&] {
        require(n >= 0, "n < 0");
        if (n == 0) return;
        require(pos && mass && acc, "null array");
        cudaStream_t s = ctx().stream;
        double* d_pos = upload(g_st.pos, pos, 3 * size_t(n), s);
        double* d_mass = upload(g_st.mass, mass, size_t(n), s);
        double* d_acc = g_st.acc.get<double>(3 * size_t(n));
        direct_sum(n, d_pos, d_mass, n, nullptr, d_acc, eps, s);
        download(acc, d_acc, 3 * size_t(n), s);
        collect_status(s);
    });
}

void nbody_render(int n, const double* pos, const uint8_t* group, int ngroups, const double* rot,
                  const double* center, double scale, int W, int H, float* img) {
    guarded([&] {
        require(n >= 0 && ngroups >= 0 && W >= 0 && H >= 0, "negative size");
        require(img && rot && center && (n == 0 || (pos && group)), "null array");
        for (int i = 0; i < n; ++i) require(group[i] < ngroups, "group index >= ngroups");
        cudaStream_t s = ctx().stream;
        const double* d_pos = upload(g_st.pos, pos, 3 * size_t(n), s);
        const uint8_t* d_grp = upload(g_st.group, group, size_t(n), s);
        const double* d_rot = upload(g_st.rot, rot, 9, s);
        const double* d_cen = upload(g_st.center, center, 3, s);
        const size_t npx = size_t(ngroups) * W * H;
        float* d_img = g_st.img.get<float>(npx);
        render_splat(n, d_pos, d_grp, ngroups, d_rot, d_cen, scale, W, H, d_img, s);
        download(img, d_img, npx, s);
        collect_status(s);
    });
}

void nbody_tonemap(int W, int H, int ngroups, const float* img, const float* glow, int gw, int gh,
                   const float* colors, float inv_ref, float K, float exposure, uint8_t* out) {
    guarded([&] {
        require(W >= 0 && H >= 0 && ngroups >= 0 && gw >= 2 && gh >= 2, "bad size");
        require(img && glow && colors && out, "null array");
        cudaStream_t s = ctx().stream;
        const float* d_img = upload(g_st.img, img, size_t(ngroups) * W * H, s);
        const float* d_glow = upload(g_st.glow, glow, size_t(ngroups) * gw * gh, s);
        const float* d_col = upload(g_st.colors, colors, 3 * size_t(ngroups), s);
        uint8_t* d_out = g_st.out.get<uint8_t>(3 * size_t(W) * H);
        render_tonemap(W, H, ngroups, d_img, d_glow, gw, gh, d_col, inv_ref, K, exposure, d_out, s);
        download(out, d_out, 3 * size_t(W) * H, s);
        collect_status(s);
    });
}

namespace {
void ic_args_check(int kind, int n_gas, int n_dm, const double* params, int nparams) {
    require(kind == 0 || kind == 1, "kind must be 0 (cloud) or 1 (disk + halo)");
    require(n_gas >= 1 && n_dm >= 0 && (long long)n_gas + n_dm < (1ll << 30), "bad particle counts");
    require(params && nparams >= 13, "need 13 parameters");
    for (int i = 0; i < 13; ++i) require(std::isfinite(params[i]), "non-finite parameter");
    require(params[0] > 0 && params[1] > 0 && params[1] < 1 && params[2] > 0, "bad mass, baryon fraction or radius");
    if (kind == 1) {
        require(params[5] >= 0 && params[5] <= 1 && params[6] > 0 && params[7] > 0, "bad disk parameters");
        require(params[8] >= 0 && params[9] >= 0 && params[10] > 0, "bad clump parameters");
        require(params[11] > 0 && params[12] >= params[11], "bad energy range");
    }
}
}  // namespace

int gf_ic_generate_dev(int kind, int n_gas, int n_dm, unsigned long long seed, const double* params,
                       int nparams, double* pos, double* vel, double* mass, int8_t* kind_out, double* u,
                       void* stream) {
    return guarded([&] {
        ic_args_check(kind, n_gas, n_dm, params, nparams);
        require(pos && vel && mass && kind_out && u, "null array");
        ic_generate(kind, n_gas, n_dm, seed, params, pos, vel, mass, kind_out, u, pick(stream));
    });
}

int gf_ic_generate(int kind, int n_gas, int n_dm, unsigned long long seed, const double* params, int nparams,
                   double* pos, double* vel, double* mass, int8_t* kind_out, double* u) {
    return guarded([&] {
        ic_args_check(kind, n_gas, n_dm, params, nparams);
        require(pos && vel && mass && kind_out && u, "null array");
        const size_t n = size_t(n_gas) + size_t(n_dm);
        cudaStream_t s = ctx().stream;
        double* d_pos = g_st.pos.get<double>(3 * n);
        double* d_vel = g_st.vel.get<double>(3 * n);
        double* d_mass = g_st.mass.get<double>(n);
        int8_t* d_kind = g_st.kind.get<int8_t>(n);
        double* d_u = g_st.u.get<double>(n);
        ic_generate(kind, n_gas, n_dm, seed, params, d_pos, d_vel, d_mass, d_kind, d_u, s);
        download(pos, d_pos, 3 * n, s);
        download(vel, d_vel, 3 * n, s);
        download(mass, d_mass, n, s);
        download(kind_out, d_kind, n, s);
        download(u, d_u, n, s);
        collect_status(s);
    });
}

int gf_last_status(void) {
    Context& c = ctx();
    if (c.ready) {
        try {
            GF_CUDA(cudaDeviceSynchronize());
            collect_status(c.stream);
        } catch (const Error& e) {
            c.last_status |= e.code;
            c.last_error = e.what();
        }
    }
    return c.last_status;
}

const char* gf_last_error(void) { return ctx().last_error.c_str(); }

int gf_tree_size(int* num_nodes, int* num_groups) {
    return guarded([&] {
        Octree& T = gravity_tree();
        int nn = 0, ng = 0;
        if (T.valid) {  // device counts: also right after a captured rebuild
            GF_CUDA(cudaDeviceSynchronize());
            TreeCounts h;
            GF_CUDA(cudaMemcpy(&h, T.counts.as<TreeCounts>(), sizeof h, cudaMemcpyDeviceToHost));
            nn = h.total_nodes;
            ng = h.num_groups;
        }
        if (num_nodes) *num_nodes = nn;
        if (num_groups) *num_groups = ng;
    });
}

int gf_tree_export(int32_t* ints, float* floats, int32_t* order, int32_t* groups) {
    return guarded([&] {
        Octree& T = gravity_tree();
        require(T.valid, "no tree");
        GF_CUDA(cudaDeviceSynchronize());
        TreeCounts h;
        GF_CUDA(cudaMemcpy(&h, T.counts.as<TreeCounts>(), sizeof h, cudaMemcpyDeviceToHost));
        const int nn = h.total_nodes, n = T.n;
        std::vector<int4> i4(nn);
        std::vector<float4> mom(nn), geo(nn);
        std::vector<float> open(nn);
        GF_CUDA(cudaMemcpy(i4.data(), T.n_i4.p, sizeof(int4) * nn, cudaMemcpyDeviceToHost));
        GF_CUDA(cudaMemcpy(mom.data(), T.n_mom.p, sizeof(float4) * nn, cudaMemcpyDeviceToHost));
        GF_CUDA(cudaMemcpy(geo.data(), T.n_geo.p, sizeof(float4) * nn, cudaMemcpyDeviceToHost));
        GF_CUDA(cudaMemcpy(open.data(), T.n_open.p, sizeof(float) * nn, cudaMemcpyDeviceToHost));
        for (int k = 0; k < nn; ++k) {
            ints[4 * k] = i4[k].x;
            ints[4 * k + 1] = i4[k].y;
            ints[4 * k + 2] = i4[k].z;
            ints[4 * k + 3] = i4[k].w & 1;
            const float f[9] = {mom[k].x, mom[k].y, mom[k].z, mom[k].w, open[k],
                                geo[k].x, geo[k].y, geo[k].z, geo[k].w};
            std::memcpy(floats + 9 * size_t(k), f, sizeof f);
        }
        GF_CUDA(cudaMemcpy(order, T.perm.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
        GF_CUDA(cudaMemcpy(groups, T.groups.p, sizeof(int32_t) * h.num_groups, cudaMemcpyDeviceToHost));
    });
}

int gf_tree_rebuild_captured(int n, const double* pos, const double* mass, double theta) {
    return guarded([&] {
        Octree& T = gravity_tree();
        require(pos && mass, "null array");
        require(T.valid && T.n == n, "build the tree for n particles first");
        cudaStream_t s = ctx().stream;
        double* d_pos = upload(g_st.pos, pos, 3 * size_t(n), s);
        double* d_mass = upload(g_st.mass, mass, size_t(n), s);
        T.reserve_graph_build();
        GF_CUDA(cudaStreamSynchronize(s));
        Context& C = ctx();
        const bool prof = C.prof.on;
        C.prof.on = false;
        cudaGraph_t g = nullptr;
        GF_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeGlobal));
        g_no_alloc = true;
        try {
            T.build(n, d_pos, d_mass, theta, s, true);
        } catch (...) {
            g_no_alloc = false;
            cudaStreamEndCapture(s, &g);
            if (g) cudaGraphDestroy(g);
            C.prof.on = prof;
            throw;
        }
        g_no_alloc = false;
        C.prof.on = prof;
        GF_CUDA(cudaStreamEndCapture(s, &g));
        cudaGraphExec_t exec = nullptr;
        GF_CUDA(cudaGraphInstantiate(&exec, g, 0));
        GF_CUDA(cudaGraphDestroy(g));
        const cudaError_t e = cudaGraphLaunch(exec, s);
        cudaGraphExecDestroy(exec);
        GF_CUDA(e);
        collect_status(s);
    });
}

int gf_accel_active_dev(int n, const double* pos, const double* mass, double* acc, double theta,
                        double eps, const uint8_t* active, int rebuild, void* stream) {
    return guarded([&] {
        require(n >= 0, "n < 0");
        if (n == 0) return;
        require(pos && mass && acc, "null array");
        require(n < (1 << 27), "n too large");
        accel_active_device(n, pos, mass, acc, theta, eps, active, rebuild, pick(stream));
    });
}

int gf_accel_direct_dev(int n, const double* pos, const double* mass, double* acc, double eps,
                        void* stream) {
    return guarded([&] {
        require(n >= 0, "n < 0");
        if (n == 0) return;
        require(pos && mass && acc, "null array");
        direct_sum(n, pos, mass, n, nullptr, acc, eps, pick(stream));
    });
}

int gf_accel_direct_targets(int n, const double* pos, const double* mass, int nt,
                            const int64_t* targets, double* acc, double eps) {
    return guarded([&] {
        require(n >= 0 && nt >= 0, "negative size");
        if (n == 0 || nt == 0) return;
        require(pos && mass && targets && acc, "null array");
        for (int t = 0; t < nt; ++t) require(targets[t] >= 0 && targets[t] < n, "target out of range");
        cudaStream_t s = ctx().stream;
        const double* d_pos = upload(g_st.pos, pos, 3 * size_t(n), s);
        const double* d_mass = upload(g_st.mass, mass, size_t(n), s);
        const int64_t* d_t = upload(g_st.targets, targets, size_t(nt), s);
        double* d_acc = g_st.acc.get<double>(3 * size_t(nt));
        direct_sum(n, d_pos, d_mass, nt, d_t, d_acc, eps, s);
        download(acc, d_acc, 3 * size_t(nt), s);
        collect_status(s);
    });
}

int gf_sph_kernel(int n, const double* r, const double* h, double* w, double* dw) {
    return guarded([&] {
        require(n >= 0, "n < 0");
        if (n == 0) return;
        require(r && h && (w || dw), "null array");
        cudaStream_t s = ctx().stream;
        const double* d_r = upload(g_st.r, r, size_t(n), s);
        const double* d_h = upload(g_st.h, h, size_t(n), s);
        double* d_w = w ? g_st.w.get<double>(n) : nullptr;
        double* d_dw = dw ? g_st.dw.get<double>(n) : nullptr;
        sph_kernel_values(n, d_r, d_h, d_w, d_dw, s);
        if (w) download(w, d_w, size_t(n), s);
        if (dw) download(dw, d_dw, size_t(n), s);
        collect_status(s);
    });
}

int gf_sph_forces(int n, int k, const double* pos, const double* vel, const double* mass,
                  const int64_t* nb, const double* h, const double* u, double gamma, double alpha,
                  double beta, double* rho, double* acc, double* dudt, double* dt_i) {
    return guarded([&] {
        require(n >= 0 && k >= 0, "negative size");
        if (n == 0) return;
        require(pos && vel && mass && nb && h && u && rho && acc && dudt && dt_i, "null array");
        for (size_t t = 0; t < size_t(n) * k; ++t) require(nb[t] >= 0 && nb[t] < n, "neighbour out of range");
        cudaStream_t s = ctx().stream;
        const double* d_pos = upload(g_st.pos, pos, 3 * size_t(n), s);
        const double* d_vel = upload(g_st.vel, vel, 3 * size_t(n), s);
        const double* d_mass = upload(g_st.mass, mass, size_t(n), s);
        const int64_t* d_nb = upload(g_st.nb, nb, size_t(n) * k, s);
        const double* d_h = upload(g_st.h, h, size_t(n), s);
        const double* d_u = upload(g_st.u, u, size_t(n), s);
        double* d_rho = g_st.rho.get<double>(n);
        double* d_acc = g_st.acc.get<double>(3 * size_t(n));
        double* d_dudt = g_st.dudt.get<double>(n);
        double* d_dt = g_st.dt.get<double>(n);
        sph_forces<int64_t>(g_sph, n, k, k, d_pos, d_vel, d_mass, d_nb, d_h, d_u, gamma, alpha, beta,
                            d_rho, d_acc, d_dudt, d_dt, s);
        download(rho, d_rho, size_t(n), s);
        download(acc, d_acc, 3 * size_t(n), s);
        download(dudt, d_dudt, size_t(n), s);
        download(dt_i, d_dt, size_t(n), s);
        collect_status(s);
    });
}

int gf_sph_forces_mixed(int n, int k, const double* pos, const double* vel, const double* mass,
                        const int64_t* nb, const double* h, const double* u, double gamma, double alpha,
                        double beta, double* rho, double* acc, double* dudt, double* dt_i) {
    return guarded([&] {
        require(n >= 0 && k >= 0, "negative size");
        if (n == 0) return;
        require(pos && vel && mass && nb && h && u && rho && acc && dudt && dt_i, "null array");
        for (size_t t = 0; t < size_t(n) * k; ++t) require(nb[t] >= 0 && nb[t] < n, "neighbour out of range");
        cudaStream_t s = ctx().stream;
        const double* d_pos = upload(g_st.pos, pos, 3 * size_t(n), s);
        const double* d_vel = upload(g_st.vel, vel, 3 * size_t(n), s);
        const double* d_mass = upload(g_st.mass, mass, size_t(n), s);
        const int64_t* d_nb = upload(g_st.nb, nb, size_t(n) * k, s);
        const double* d_h = upload(g_st.h, h, size_t(n), s);
        const double* d_u = upload(g_st.u, u, size_t(n), s);
        double* d_rho = g_st.rho.get<double>(n);
        double* d_acc = g_st.acc.get<double>(3 * size_t(n));
        double* d_dudt = g_st.dudt.get<double>(n);
        double* d_dt = g_st.dt.get<double>(n);
        sph_forces32<int64_t>(g_sph32, n, k, k, nullptr, d_pos, d_vel, d_mass, d_nb, d_h, d_u, gamma, alpha, beta,
                              d_rho, d_acc, d_dudt, d_dt, s);
        download(rho, d_rho, size_t(n), s);
        download(acc, d_acc, 3 * size_t(n), s);
        download(dudt, d_dudt, size_t(n), s);
        download(dt_i, d_dt, size_t(n), s);
        collect_status(s);
    });
}

int gf_sph_forces_dev(int n, int k, const double* pos, const double* vel, const double* mass,
                      const int64_t* nb, const double* h, const double* u, double gamma, double alpha,
                      double beta, double* rho, double* acc, double* dudt, double* dt_i, void* stream) {
    return guarded([&] {
        require(n >= 0 && k >= 0, "negative size");
        if (n == 0) return;
        require(pos && vel && mass && nb && h && u && rho && acc && dudt && dt_i, "null array");
        sph_forces<int64_t>(g_sph, n, k, k, pos, vel, mass, nb, h, u, gamma, alpha, beta, rho, acc, dudt,
                            dt_i, pick(stream));
    });
}

int gf_knn_from_candidates(int n, int m, const double* pos, const int64_t* cand, int k, int64_t* nb,
                           double* dist) {
    int ok = 1;
    const int st = guarded([&] {
        require(n >= 0 && m >= 0 && k >= 1, "bad size");
        require(m <= 64 && k <= m, "need k <= m <= 64");
        if (n == 0) return;
        require(pos && cand && nb && dist, "null array");
        for (size_t t = 0; t < size_t(n) * m; ++t) require(cand[t] >= -1 && cand[t] < n, "candidate out of range");
        cudaStream_t s = ctx().stream;
        const double* d_pos = upload(g_st.pos, pos, 3 * size_t(n), s);
        const int64_t* d_cand = upload(g_st.cand, cand, size_t(n) * m, s);
        int64_t* d_nb = upload(g_st.nb, nb, size_t(n) * k, s);
        double* d_dist = upload(g_st.dist, dist, size_t(n) * k, s);
        int* d_ok = g_st.flags.get<int>(1);
        GF_CUDA(cudaMemcpyAsync(d_ok, &ok, sizeof(int), cudaMemcpyHostToDevice, s));
        knn_from_candidates(n, m, d_pos, d_cand, k, d_nb, d_dist, d_ok, s);
        download(nb, d_nb, size_t(n) * k, s);
        download(dist, d_dist, size_t(n) * k, s);
        download(&ok, d_ok, 1, s);
        collect_status(s);
    });
    return st ? -st : ok;
}

int gf_knn(int n, const double* pos, int k, double* dist, int64_t* nb) {
    return guarded([&] {
        require(n >= 1 && k >= 1 && k <= 64 && k <= n, "need 1 <= k <= min(64, n)");
        require(pos && dist && nb, "null array");
        require(n < (1 << 27), "n too large");
        cudaStream_t s = ctx().stream;
        const double* d_pos = upload(g_st.pos, pos, 3 * size_t(n), s);
        int64_t* d_nb = g_st.nb.get<int64_t>(size_t(n) * k);
        double* d_dist = g_st.dist.get<double>(size_t(n) * k);
        unsigned long long* d_it = g_st.flags.get<unsigned long long>(1);
        GF_CUDA(cudaMemsetAsync(d_it, 0, sizeof(unsigned long long), s));
        knn_exact(g_knn_tree, n, d_pos, k, nullptr, d_nb, d_dist, d_it, s);
        download(nb, d_nb, size_t(n) * k, s);
        download(dist, d_dist, size_t(n) * k, s);
        download(&g_knn_iters, d_it, 1, s);
        collect_status(s);
    });
}

long long gf_knn_iterations(void) { return (long long)g_knn_iters; }

static void force_args_check(int n, const void* pos, const void* vel, const void* mass, const void* kind,
                             const void* u, const void* acc, const void* dt_ind) {
    require(n >= 0, "n < 0");
    require(n < (1 << 27), "n too large");
    require(n == 0 || (pos && vel && mass && kind && u && acc && dt_ind), "null array");
}

int gf_accelerations_dev(int n, const double* pos, const double* vel, const double* mass,
                         const int8_t* kind, const double* u, double theta, double eps, double gamma,
                         double alpha, double beta, const uint8_t* active, int rebuild, int sph,
                         int fresh_nb, double* acc, double* dt_ind, void* stream) {
    return guarded([&] {
        force_args_check(n, pos, vel, mass, kind, u, acc, dt_ind);
        if (n == 0) return;
        ForceArgs a{n, pos, vel, mass, kind, u, theta, eps, gamma, alpha, beta, active, rebuild, sph,
                    fresh_nb, acc, dt_ind};
        force_engine().evaluate(a, pick(stream));
    });
}

int gf_accelerations(int n, const double* pos, const double* vel, const double* mass, const int8_t* kind,
                     const double* u, double theta, double eps, double gamma, double alpha, double beta,
                     const uint8_t* active, int rebuild, int sph, int fresh_nb, double* acc,
                     double* dt_ind) {
    return guarded([&] {
        force_args_check(n, pos, vel, mass, kind, u, acc, dt_ind);
        if (n == 0) return;
        cudaStream_t s = ctx().stream;
        // the gravity chain needs pos and mass (and kind for the gas flags) first; vel and u,
        // read only by the hydro chain, are copied on a second stream meanwhile
        static cudaStream_t s_late = nullptr;
        static cudaEvent_t ev_start = nullptr, ev_late = nullptr;
        if (!s_late) {
            GF_CUDA(cudaStreamCreateWithFlags(&s_late, cudaStreamNonBlocking));
            GF_CUDA(cudaEventCreateWithFlags(&ev_start, cudaEventDisableTiming));
            GF_CUDA(cudaEventCreateWithFlags(&ev_late, cudaEventDisableTiming));
        }
        GF_CUDA(cudaEventRecord(ev_start, s));  // after the previous call's work on s
        GF_CUDA(cudaStreamWaitEvent(s_late, ev_start, 0));
        double* d_pos = upload(g_st.pos, pos, 3 * size_t(n), s);
        double* d_mass = upload(g_st.mass, mass, size_t(n), s);
        int8_t* d_kind = upload(g_st.kind, kind, size_t(n), s);
        const uint8_t* d_act = active ? upload(g_st.active, active, size_t(n), s) : nullptr;
        double* d_vel = upload(g_st.vel, vel, 3 * size_t(n), s_late);
        double* d_u = upload(g_st.u, u, size_t(n), s_late);
        GF_CUDA(cudaEventRecord(ev_late, s_late));
        ForceArgs a{n, d_pos, d_vel, d_mass, d_kind, d_u, theta, eps, gamma, alpha, beta, d_act, rebuild, sph,
                    fresh_nb, g_st.acc.get<double>(3 * size_t(n)), g_st.dt_ind.get<double>(size_t(n))};
        a.late_inputs = ev_late;
        force_engine().evaluate(a, s);
        GF_CUDA(cudaStreamWaitEvent(s, ev_late, 0));  // the copies are done before the call returns
        download(acc, a.acc, 3 * size_t(n), s);
        download(dt_ind, a.dt_ind, size_t(n), s);
        collect_status(s);
    });
}

int gf_profile(int on) {
    return guarded([&] {
        GF_CUDA(cudaDeviceSynchronize());
        ctx().prof.clear();
        ctx().prof.on = on != 0;
    });
}

int gf_profile_stage(int stage, double* total_ms, int* launches) {
    return guarded([&] {
        require(stage >= 0 && stage < kStCount, "bad stage");
        GF_CUDA(cudaDeviceSynchronize());
        double t = 0;
        for (auto& pr : ctx().prof.recs[stage]) {
            float ms = 0;
            GF_CUDA(cudaEventElapsedTime(&ms, pr.first, pr.second));
            t += ms;
        }
        if (total_ms) *total_ms = t;
        if (launches) *launches = int(ctx().prof.recs[stage].size());
    });
}

long long gf_launch_count(void) { return ctx().launches; }

void* gf_stream(void) {
    try {
        ensure_ready();
        return ctx().stream;
    } catch (...) {
        return nullptr;
    }
}

int gf_fp32_peak(double* tflops) {
    return guarded([&] {
        require(tflops != nullptr, "null pointer");
        *tflops = fp32_peak_tflops();
    });
}

static long long walk_counter(bool quad_only) {
    unsigned long long p = 0;
    guarded([&] {
        Octree* T = last_walked();
        if (!T || !T->valid) return;
        GF_CUDA(cudaDeviceSynchronize());
        TreeCounts* c = T->counts.as<TreeCounts>();
        GF_CUDA(cudaMemcpy(&p, quad_only ? &c->qpairs : &c->pairs, sizeof p, cudaMemcpyDeviceToHost));
    });
    return (long long)p;
}

long long gf_walk_pairs(void) { return walk_counter(false); }

long long gf_walk_quad_pairs(void) { return walk_counter(true); }

int gf_set_option(int key, double value) {
    return guarded([&] {
        ForceEngine& F = force_engine();
        switch (key) {
            case GF_OPT_SPH_FLOAT32: F.sph_float32 = value != 0; break;
            case GF_OPT_GRAVITY_QUAD: F.gravity_quad = value != 0; break;
            case GF_OPT_HGUESS:
                require(value == 0 || value == 1 || value == 2, "h guess mode is 0, 1 or 2");
                F.hguess = int(value);
                break;
            case GF_OPT_COLLECT: {
                require(value >= 0 && value <= 2e8, "collect capacity out of range");
                F.collect_cap = (long long)value;
                F.collect_n = 0;
                if (F.collect_cap > 0) {
                    F.colX.get<float>(4 * size_t(F.collect_cap));
                    F.colT.get<float>(size_t(F.collect_cap));
                }
                break;
            }
            case GF_OPT_WALK_CHUNK:
                require(value >= 0 && value <= kChunkCodeMax, "walk chunk is 0..96");
                F.walk_chunk = int(value);
                break;
            case GF_OPT_WALK_GROUP:
                require(value >= 8 && value <= 128, "walk group is 8..128");
                F.walk_group = int(value);
                F.grav.valid = false;  // regroup at the next evaluation
                break;
            case GF_OPT_WALK_MERGE:
                require(value >= 0 && value <= 128, "walk merge is 0..128");
                F.walk_merge = int(value);
                break;
            case GF_OPT_GRAVITY_REL_MONO:
                require(value >= 0 && value < 1, "monopole tolerance is in [0, 1)");
                F.grav_rel_mono = value;
                break;
            case GF_OPT_FORGET_H:  // the next full search starts without previous smoothing lengths
                F.have_hprev = false;
                F.have_divv = false;
                break;
            case GF_OPT_WALK_SHAPE:
                require(value >= 0 && value < kNumWalkShapes && value == int(value), "walk shape is 0..3");
                F.walk_shape = int(value);
                break;
            case GF_OPT_GRAVITY_REL:
                require(value >= 0 && value < 1, "relative opening tolerance is in [0, 1)");
                F.grav_rel = value;
                F.have_aold = false;  // the next evaluation sets the error scale
                break;
            default: throw Error(GF_ERR_ARG, "unknown option");
        }
    });
}

double gf_get_option(int key) {
    ForceEngine& F = force_engine();
    switch (key) {
        case GF_OPT_SPH_FLOAT32: return F.sph_float32;
        case GF_OPT_GRAVITY_QUAD: return F.gravity_quad;
        case GF_OPT_HGUESS: return F.hguess;
        case GF_OPT_COLLECT: return double(F.collect_n);
        case GF_OPT_WALK_CHUNK: return F.walk_chunk;
        case GF_OPT_WALK_GROUP: return F.walk_group;
        case GF_OPT_GRAVITY_REL: return F.grav_rel;
        case GF_OPT_WALK_MERGE: return F.walk_merge;
        case GF_OPT_GRAVITY_REL_MONO: return F.grav_rel_mono;
        case GF_OPT_WALK_SHAPE: return F.walk_shape;
        default: return -1.0;
    }
}

int gf_sim_init(int n, const double* pos, const double* vel, const double* mass, const int8_t* kind,
                const double* u, double theta, double eps, double gamma, double alpha, double beta) {
    return guarded([&] {
        require(n > 0 && n < (1 << 27), "bad n");
        require(pos && vel && mass && kind && u, "null array");
        sim_init(n, pos, vel, mass, kind, u, theta, eps, gamma, alpha, beta);
        collect_status(ctx().stream);
    });
}

int gf_sim_step(double dt_max, double* taken, int* substeps) {
    return guarded([&] {
        require(dt_max > 0, "dt_max <= 0");
        const double D = sim_step(dt_max, substeps);
        if (taken) *taken = D;
        collect_status(ctx().stream);
    });
}

double gf_sim_updates(void) { return sim_updates(); }

int gf_sim_blocks(int nblocks, int nlev, double* updates) {
    return guarded([&] {
        require(nblocks >= 0 && nlev >= 1 && nlev <= 8, "need nblocks >= 0 and 1 <= nlev <= 8");
        require(simulation_ready(), "gf_sim_init first");
        const double u = block_run(nblocks, nlev);
        if (updates) *updates = u;
        collect_status(ctx().stream);
    });
}

int gf_sim_block_config(const int* chunk, int nbins, int rebuild_every) {
    return guarded([&] {
        require(!chunk || (nbins >= 1 && nbins <= 8), "need 1 <= nbins <= 8");
        require(rebuild_every >= 0, "rebuild_every < 0");
        if (chunk)
            for (int b = 0; b < nbins; ++b)
                require(chunk[b] >= 0 && chunk[b] % 100 <= kChunkCodeMax && chunk[b] % 1000 < 200 &&
                            chunk[b] / 1000 < kNumWalkShapes,
                        "chunk out of [0, 96] (+100, + 1000 x shape)");
        block_config(chunk, nbins, rebuild_every);
    });
}

int gf_sim_block_autotune(int nlev, int* chunk, int* rebuild_every, double* graph_ms) {
    return guarded([&] {
        require(nlev >= 2 && nlev <= 8, "need 2 <= nlev <= 8");
        require(simulation_ready(), "gf_sim_init first");
        block_autotune(nlev, chunk, rebuild_every, graph_ms);
        collect_status(ctx().stream);
    });
}

int gf_sim_levels(int nlev, double* frac) {
    return guarded([&] {
        require(nlev >= 1 && nlev <= 8 && frac, "bad arguments");
        block_levels(nlev, frac);
    });
}

int gf_sim_diagnostics(double theta, double* out) {
    return guarded([&] {
        require(out && theta > 0, "bad arguments");
        require(simulation_ready(), "gf_sim_init first");
        sim_diagnostics(theta, out);
        collect_status(ctx().stream);
    });
}

int gf_sim_read(double* pos, double* vel, double* acc, double* dt_ind, double* t) {
    return guarded([&] { sim_read(pos, vel, acc, dt_ind, t); });
}

int gf_sim_stars(int on, const double* params, const uint64_t* rng_state) {
    return guarded([&] {
        require(simulation_ready(), "no simulation (gf_sim_init)");
        if (on) {
            require(params != nullptr && rng_state != nullptr, "null argument");
            for (int i = 0; i < 10; ++i) require(std::isfinite(params[i]) && params[i] >= 0, "bad star parameter");
            require(params[3] >= 1 && params[3] <= 64, "fb_ngb is 1..64");
            require((rng_state[3] & 1) == 1, "a PCG64 increment is odd");
        }
        sim_stars(on, params, reinterpret_cast<const unsigned long long*>(rng_state));
    });
}

long long gf_sim_read_stars(int8_t* kind, double* birth, double* no_cool_until, uint64_t* rng_state) {
    long long formed = -1;
    const int st = guarded([&] {
        require(simulation_ready(), "no simulation (gf_sim_init)");
        formed = sim_read_stars(kind, birth, no_cool_until, reinterpret_cast<unsigned long long*>(rng_state));
    });
    return st ? -st : formed;
}

int gf_sim_read_scalars(double* out) {
    return guarded([&] {
        require(out != nullptr, "null array");
        require(simulation_ready(), "no simulation (gf_sim_init)");
        sim_scalars(out);
    });
}

int gf_sim_read_hydro(double* rho, double* dudt) {
    return guarded([&] {
        require(rho != nullptr && dudt != nullptr, "null array");
        require(simulation_ready(), "no simulation (gf_sim_init)");
        sim_read_hydro(rho, dudt);
    });
}

int gf_sim_restore(const double* acc, const double* dt_ind, const double* birth, const double* no_cool_until,
                   const double* rho, const double* dudt, double t, double dt_grav, double dt_gas) {
    return guarded([&] {
        require(simulation_ready(), "no simulation (gf_sim_init)");
        require(acc != nullptr && dt_ind != nullptr, "null array");
        require(std::isfinite(t) && dt_grav > 0 && dt_gas > 0, "bad scalars");
        sim_restore(acc, dt_ind, birth, no_cool_until, rho, dudt, t, dt_grav, dt_gas);
    });
}

int gf_sim_read_u(double* u) {
    return guarded([&] {
        require(u != nullptr, "null array");
        require(simulation_ready(), "no simulation (gf_sim_init)");
        sim_read_u(u);
    });
}

int gf_sim_thermo(int mode, const double* units) {
    return guarded([&] {
        require(mode >= 0 && mode <= 2, "thermal mode is 0, 1 or 2");
        require(mode == 0 || units != nullptr, "null units");
        if (mode) {
            for (int i = 0; i < 8; ++i) require(std::isfinite(units[i]) && units[i] > 0, "units must be positive");
        }
        sim_thermo(mode, units);
    });
}

int gf_cooling_function(int n, const double* T, double* lam) {
    return guarded([&] {
        require(n >= 0 && (n == 0 || (T && lam)), "bad arguments");
        cudaStream_t s = ctx().stream;
        const double* d_T = upload(g_st.r, T, size_t(n), s);
        double* d_l = g_st.w.get<double>(size_t(n));
        cooling_function(n, d_T, d_l, s);
        download(lam, d_l, size_t(n), s);
        collect_status(s);
    });
}

int gf_cool(int n, const double* u, const double* T, const double* rho, const double* dt, const uint8_t* blocked,
            double u_floor, const double* units, double* out) {
    return guarded([&] {
        require(n >= 0 && (n == 0 || (u && T && rho && dt && out)) && units, "bad arguments");
        cudaStream_t s = ctx().stream;
        const ThermoUnits U{units[0], units[1], units[2], units[3], units[4], units[5], units[6], units[7]};
        const double* d_u = upload(g_st.u, u, size_t(n), s);
        const double* d_T = upload(g_st.r, T, size_t(n), s);
        const double* d_rho = upload(g_st.rho, rho, size_t(n), s);
        const double* d_dt = upload(g_st.dt, dt, size_t(n), s);
        const uint8_t* d_b = blocked ? upload(g_st.flags, blocked, size_t(n), s) : nullptr;
        double* d_o = g_st.w.get<double>(size_t(n));
        cool(n, d_u, d_T, d_rho, d_dt, d_b, u_floor, U, d_o, s);
        download(out, d_o, size_t(n), s);
        collect_status(s);
    });
}

int gf_mlp_tensor_cores(void) { return mlp().tensor_cores; }

int gf_mlp_init(int seed) {
    return guarded([&] { mlp().init(unsigned(seed), ctx().stream); });
}

int gf_mlp_set_params(const float* p) {
    return guarded([&] {
        require(p != nullptr, "null params");
        mlp().set_params(p, ctx().stream);
        GF_CUDA(cudaStreamSynchronize(ctx().stream));
    });
}

int gf_mlp_get_params(float* p) {
    return guarded([&] {
        require(p != nullptr && mlp().ready, "no model");
        mlp().get_params(p, ctx().stream);
    });
}

int gf_mlp_set_norm(const float* mean4, const float* std4, double t_mean, double t_std) {
    return guarded([&] {
        require(mean4 && std4 && t_std > 0, "bad normalisation");
        MlpNorm& nm = mlp().norm;
        for (int i = 0; i < 4; ++i) {
            require(std4[i] > 0, "std <= 0");
            nm.mean[i] = mean4[i];
            nm.inv_std[i] = 1.f / std4[i];
        }
        nm.t_mean = float(t_mean);
        nm.t_std = float(t_std);
    });
}

int gf_mlp_predict(int n, const float* X, float* Y) {
    return guarded([&] {
        require(n >= 0 && (n == 0 || (X && Y)) && mlp().ready, "bad arguments or no model");
        if (n == 0) return;
        cudaStream_t s = ctx().stream;
        const float* dX = upload(g_st.mlpX, X, 4 * size_t(n), s);
        float* dY = g_st.mlpY.get<float>(n);
        mlp().predict(n, dX, dY, s);
        download(Y, dY, size_t(n), s);
        collect_status(s);
    });
}

int gf_mlp_gradient(int n, const float* X, const float* T, float* grad) {
    return guarded([&] {
        require(n > 0 && X && T && grad && mlp().ready, "bad arguments or no model");
        cudaStream_t s = ctx().stream;
        const float* dX = upload(g_st.mlpX, X, 4 * size_t(n), s);
        const float* dT = upload(g_st.mlpT, T, size_t(n), s);
        float* dG = g_st.mlpG.get<float>(kMlpParams);
        mlp().gradient(n, nullptr, dX, dT, dG, s);
        download(grad, dG, size_t(kMlpParams), s);
        collect_status(s);
    });
}

long long gf_mlp_collected(float* X, float* T, long long max_rows) {
    long long got = 0;
    guarded([&] {
        ForceEngine& F = force_engine();
        got = std::min<long long>(F.collect_n, std::max<long long>(0, max_rows));
        if (got > 0 && X) GF_CUDA(cudaMemcpy(X, F.colX.p, sizeof(float) * 4 * size_t(got), cudaMemcpyDeviceToHost));
        if (got > 0 && T) GF_CUDA(cudaMemcpy(T, F.colT.p, sizeof(float) * size_t(got), cudaMemcpyDeviceToHost));
        if (!X && !T) got = F.collect_n;
    });
    return got;
}

int gf_mlp_train(int steps, int batch, double lr, double* loss) {
    return guarded([&] {
        ForceEngine& F = force_engine();
        Mlp& M = mlp();
        require(M.ready && F.collect_n > 0, "no model or no collected data");
        require(steps >= 0 && batch > 0 && lr > 0, "bad training arguments");
        M.X.p = nullptr;  // the training set is the collected one (not owned)
        M.n_data = int(F.collect_n);
        cudaStream_t s = ctx().stream;
        const double l = train_on(M, F.colX.as<float>(), F.colT.as<float>(), steps, batch, lr, s);
        if (loss) *loss = l;
        collect_status(s);
    });
}

int gf_force_stats(double* out, int nout) {
    return guarded([&] {
        require(out && nout >= 0, "bad output");
        ForceEngine& F = force_engine();
        GF_CUDA(cudaDeviceSynchronize());
        const HydroScalars* h = F.scalars_h;
        TreeCounts kc{}, gc{};
        if (F.knn_tree.valid)
            GF_CUDA(cudaMemcpy(&kc, F.knn_tree.counts.p, sizeof kc, cudaMemcpyDeviceToHost));
        if (F.grav.valid)  // the device count: also right after a synchronisation-free rebuild
            GF_CUDA(cudaMemcpy(&gc, F.grav.counts.p, sizeof gc, cudaMemcpyDeviceToHost));
        const double v[9] = {h ? double(F.ng) : 0.0, h ? h->dt_grav : 0.0, h ? h->dt_gas : 0.0,
                             h ? double(h->knn_iters) : 0.0, 0.0, double(F.full_searches),
                             double(F.verlet_hits), double(F.knn_tree.nn), double(gc.total_nodes)};
        for (int i = 0; i < nout && i < 9; ++i) out[i] = v[i];
    });
}

int gf_force_autotune(double eps, int* walk_merge, int* walk_shape, double* walk_ms) {
    return guarded([&] {
        require(eps > 0 && std::isfinite(eps), "bad eps");
        GF_CUDA(cudaDeviceSynchronize());
        force_engine().autotune_walk(eps, ctx().stream, walk_merge, walk_shape, walk_ms);
        collect_status(ctx().stream);
    });
}

int gf_force_read_gas(int cap, int* n_gas, int32_t* gidx, double* h, double* rho, double* dudt, double* dt_i,
                      double* acc_sph, int32_t* nb32) {
    return guarded([&] {
        ForceEngine& F = force_engine();
        GF_CUDA(cudaDeviceSynchronize());
        const int ng = F.ng_valid;
        if (n_gas) *n_gas = ng;
        if (ng <= 0) return;
        require(cap >= ng || !(gidx || h || rho || dudt || dt_i || acc_sph || nb32),
                "output rows fewer than the gas particles");
        cudaStream_t s = ctx().stream;
        download(gidx, F.gidx.as<int32_t>(), gidx ? size_t(ng) : 0, s);
        download(h, F.h.as<double>(), h ? size_t(ng) : 0, s);
        download(rho, F.rho.as<double>(), rho ? size_t(ng) : 0, s);
        download(dudt, F.dudt.as<double>(), dudt ? size_t(ng) : 0, s);
        download(dt_i, F.dt_i.as<double>(), dt_i ? size_t(ng) : 0, s);
        download(acc_sph, F.gacc.as<double>(), acc_sph ? 3 * size_t(ng) : 0, s);
        if (nb32) {
            require(F.last_nb != nullptr, "no neighbour rows");
            GF_CUDA(cudaMemcpy2DAsync(nb32, 32 * sizeof(int32_t), F.last_nb, 48 * sizeof(int32_t),
                                      32 * sizeof(int32_t), size_t(ng), cudaMemcpyDeviceToHost, s));
        }
        GF_CUDA(cudaStreamSynchronize(s));
    });
}

int gf_force_info(int* n_gas, double* dt_grav, double* dt_gas, long long* knn_iters) {
    return guarded([&] {
        ForceEngine& F = force_engine();
        GF_CUDA(cudaDeviceSynchronize());
        const HydroScalars* h = F.scalars_h;
        if (n_gas) *n_gas = h ? F.ng : 0;
        if (dt_grav) *dt_grav = h ? h->dt_grav : 0.0;
        if (dt_gas) *dt_gas = h ? h->dt_gas : 0.0;
        if (knn_iters) *knn_iters = h ? (long long)h->knn_iters : 0;
    });
}

}  // extern "C"
