// gf_oracle.cpp — TEST INFRASTRUCTURE ONLY (the oracle).
//
// A CPU restatement of the reference algorithms on the force path, used to check the
// CUDA library and, in bench.py's `cpu_baseline` leg and `--impl reference` arm, as the
// timed CPU baseline ("port"). Nothing in the product links or calls this file.
//
// Parity is pinned: tests/test_oracle_pinned.py compares this restatement against the
// reference itself (cpp/nbody.cpp compiled from its own sources into oracle/_ref/, and
// galaxy_formation/sph.py run through a numba stand-in) via the fixtures under
// tests/golden/, generated by tests/golden/make_golden.py.
//
// What is restated (reference file:line):
//   Barnes-Hut octree build ........ cpp/nbody.cpp:76-150 (partition, child centres,
//                                    finalize, recursive build), :202-256 (bbox, root box,
//                                    groups, tree-order copy)
//   refit ........................... cpp/nbody.cpp:262-305
//   group walk + list evaluation .... cpp/nbody.cpp:323-411
//   direct sum ...................... cpp/nbody.cpp:428-441
//   SPH kernel / gradient ........... galaxy_formation/sph.py:31-54
//   SPH density + forces ............ galaxy_formation/sph.py:57-106
//   Verlet reselection .............. galaxy_formation/sph.py:109-135
//   exact k nearest neighbours ...... stands in for scipy.spatial.cKDTree.query
//                                     (galaxy_formation/sph.py:165-166); brute force.
//
// The parallel structure (OpenMP tasks over the top three levels of the octree) is this
// file's own; the tree it produces is the reference's: same cells, same depth-first node
// order, same `next` links, same groups, same single-precision moments.
//
// Build: see oracle/Makefile (g++ -O3 -ffast-math -fopenmp, no -march flags so that the
// same source builds on x86-64 and aarch64).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>
#include <omp.h>

namespace {

constexpr int kLeafMax = 8;     // cpp/nbody.cpp:33
constexpr int kGroupMax = 64;   // cpp/nbody.cpp:34
constexpr int kDepthMax = 48;   // cpp/nbody.cpp:35
constexpr int kTaskDepth = 3;   // subtrees below this depth are built by one OpenMP task

// 64-byte node record; field meaning follows cpp/nbody.cpp:38-45.
struct Node {
    float cx, cy, cz, m;
    float open_r;
    int32_t start, count, next, leaf;
    float gx, gy, gz, half;
};

struct Octree {
    int n = 0;
    float theta = 0.7f;
    const double* pos = nullptr;
    const double* mass = nullptr;
    std::vector<Node> nodes;
    std::vector<int32_t> order;         // tree position -> particle index
    std::vector<int32_t> scratch;
    std::vector<uint8_t> oct;
    std::vector<int32_t> groups;        // node ids of the walk groups, depth-first order
    std::vector<float> fx, fy, fz, fm;  // tree-order single-precision particles
    std::vector<double> pos_at_build;   // refit measures displacements from these
    std::vector<float> pdisp, ndisp;    // per-particle / per-node displacement (refit)
};

Octree g_oct;

// Stable 8-way split of order[b, e) around centre c (cpp/nbody.cpp:76-90): octant bit k is
// set when coordinate k is strictly greater than the centre.
void split8(Octree& T, int b, int e, const double c[3], int bounds[9]) {
    int cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const double* p = T.pos;
    for (int i = b; i < e; ++i) {
        const int j = T.order[i];
        const int o = int(p[3 * j] > c[0]) | (int(p[3 * j + 1] > c[1]) << 1) |
                      (int(p[3 * j + 2] > c[2]) << 2);
        T.oct[i] = uint8_t(o);
        ++cnt[o];
    }
    bounds[0] = b;
    for (int o = 0; o < 8; ++o) bounds[o + 1] = bounds[o] + cnt[o];
    int put[8];
    std::copy(bounds, bounds + 8, put);
    for (int i = b; i < e; ++i) T.scratch[put[T.oct[i]]++] = T.order[i];
    std::memcpy(&T.order[b], &T.scratch[b], sizeof(int32_t) * size_t(e - b));
}

// Moments -> node record (cpp/nbody.cpp:98-115): single-precision centre of mass and mass,
// opening radius 2 half / theta + |com - box centre| evaluated in double.
void set_node(Node& q, double M, double sx, double sy, double sz, const double c[3], double half,
              int b, int e, bool leaf, float theta) {
    const double inv = M > 0 ? 1.0 / M : 0.0;
    const double mx = sx * inv, my = sy * inv, mz = sz * inv;
    q.cx = float(mx);
    q.cy = float(my);
    q.cz = float(mz);
    q.m = float(M);
    const double ox = mx - c[0], oy = my - c[1], oz = mz - c[2];
    q.open_r = float(2 * half / theta + std::sqrt(ox * ox + oy * oy + oz * oz));
    q.gx = float(c[0]);
    q.gy = float(c[1]);
    q.gz = float(c[2]);
    q.half = float(half);
    q.start = b;
    q.count = e - b;
    q.leaf = leaf ? 1 : 0;
}

// Builds the subtree of cell (c, half) holding order[b, e) into `out`, depth-first with
// local `next` links. Children of shallow cells are built by separate OpenMP tasks into
// their own vectors and spliced back in octant order.
void grow(Octree& T, std::vector<Node>& out, int b, int e, const double c[3], double half, int depth) {
    const int me = int(out.size());
    out.emplace_back();
    double M = 0, sx = 0, sy = 0, sz = 0;
    const bool leaf = (e - b) <= kLeafMax || depth >= kDepthMax;
    if (leaf) {
        for (int i = b; i < e; ++i) {
            const int j = T.order[i];
            const double m = T.mass[j];
            M += m;
            sx += m * T.pos[3 * j];
            sy += m * T.pos[3 * j + 1];
            sz += m * T.pos[3 * j + 2];
        }
    } else {
        int bounds[9];
        split8(T, b, e, c, bounds);
        const double hc = 0.5 * half;
        double cc[8][3];
        for (int o = 0; o < 8; ++o) {
            cc[o][0] = c[0] + ((o & 1) ? hc : -hc);
            cc[o][1] = c[1] + ((o & 2) ? hc : -hc);
            cc[o][2] = c[2] + ((o & 4) ? hc : -hc);
        }
        if (depth < kTaskDepth && (e - b) > 4096) {
            std::vector<Node> sub[8];
            for (int o = 0; o < 8; ++o) {
                if (bounds[o] == bounds[o + 1]) continue;
#pragma omp task shared(T, sub, bounds, cc) firstprivate(o, hc, depth)
                grow(T, sub[o], bounds[o], bounds[o + 1], cc[o], hc, depth + 1);
            }
#pragma omp taskwait
            for (int o = 0; o < 8; ++o) {
                if (sub[o].empty()) continue;
                const int base = int(out.size());
                for (Node q : sub[o]) {
                    q.next += base;
                    out.push_back(q);
                }
                const Node& ch = out[base];
                M += ch.m;
                sx += double(ch.m) * ch.cx;
                sy += double(ch.m) * ch.cy;
                sz += double(ch.m) * ch.cz;
            }
        } else {
            for (int o = 0; o < 8; ++o) {
                if (bounds[o] == bounds[o + 1]) continue;
                const int ch_id = int(out.size());
                grow(T, out, bounds[o], bounds[o + 1], cc[o], hc, depth + 1);
                const Node& ch = out[ch_id];
                M += ch.m;
                sx += double(ch.m) * ch.cx;
                sy += double(ch.m) * ch.cy;
                sz += double(ch.m) * ch.cz;
            }
        }
    }
    set_node(out[me], M, sx, sy, sz, c, half, b, e, leaf, T.theta);
    out[me].next = int(out.size());
}

void build(Octree& T, int n, const double* pos, const double* mass, double theta) {
    T.n = n;
    T.pos = pos;
    T.mass = mass;
    T.theta = float(theta);
    T.order.resize(n);
    T.scratch.resize(n);
    T.oct.resize(n);

    // root cube (cpp/nbody.cpp:210-219)
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    double lx = lo[0], ly = lo[1], lz = lo[2], hx = hi[0], hy = hi[1], hz = hi[2];
#pragma omp parallel for reduction(min : lx, ly, lz) reduction(max : hx, hy, hz)
    for (int i = 0; i < n; ++i) {
        T.order[i] = i;
        lx = std::min(lx, pos[3 * i]);
        hx = std::max(hx, pos[3 * i]);
        ly = std::min(ly, pos[3 * i + 1]);
        hy = std::max(hy, pos[3 * i + 1]);
        lz = std::min(lz, pos[3 * i + 2]);
        hz = std::max(hz, pos[3 * i + 2]);
    }
    const double c[3] = {0.5 * (lx + hx), 0.5 * (ly + hy), 0.5 * (lz + hz)};
    const double half = 0.5 * std::max({hx - lx, hy - ly, hz - lz}) * 1.0001 + 1e-12;

    T.nodes.clear();
    T.nodes.reserve(size_t(2 * n / kLeafMax + 1024));
#pragma omp parallel
#pragma omp single
    grow(T, T.nodes, 0, n, c, half, 0);

    // walk groups: the shallowest nodes with at most kGroupMax particles, or leaves
    // (cpp/nbody.cpp:235-243)
    T.groups.clear();
    const int nn = int(T.nodes.size());
    int k = 0;
    while (k < nn) {
        const Node& q = T.nodes[k];
        if (q.count <= kGroupMax || q.leaf) {
            T.groups.push_back(k);
            k = q.next;
        } else {
            ++k;
        }
    }

    // tree-order single-precision copy and build-time positions (cpp/nbody.cpp:245-255)
    T.fx.resize(n);
    T.fy.resize(n);
    T.fz.resize(n);
    T.fm.resize(n);
    T.pos_at_build.assign(pos, pos + 3 * size_t(n));
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const int j = T.order[i];
        T.fx[i] = float(pos[3 * j]);
        T.fy[i] = float(pos[3 * j + 1]);
        T.fz[i] = float(pos[3 * j + 2]);
        T.fm[i] = float(mass[j]);
    }
}

// Same cells, new moments; opening radii grow with the largest displacement since the
// build (cpp/nbody.cpp:262-305).
void refit(Octree& T, const double* pos, const double* mass) {
    const int n = T.n;
    T.pos = pos;
    T.mass = mass;
    T.pdisp.resize(n);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const int j = T.order[i];
        T.fx[i] = float(pos[3 * j]);
        T.fy[i] = float(pos[3 * j + 1]);
        T.fz[i] = float(pos[3 * j + 2]);
        T.fm[i] = float(mass[j]);
        const double dx = pos[3 * j] - T.pos_at_build[3 * j];
        const double dy = pos[3 * j + 1] - T.pos_at_build[3 * j + 1];
        const double dz = pos[3 * j + 2] - T.pos_at_build[3 * j + 2];
        T.pdisp[i] = mass[j] > 0 ? float(std::sqrt(dx * dx + dy * dy + dz * dz)) : 0.0f;
    }
    const int nn = int(T.nodes.size());
    T.ndisp.resize(nn);
    for (int k = nn - 1; k >= 0; --k) {  // children always follow their parent
        Node& q = T.nodes[k];
        double M = 0, sx = 0, sy = 0, sz = 0;
        float dmax = 0;
        if (q.leaf) {
            for (int i = q.start; i < q.start + q.count; ++i) {
                const double m = T.fm[i];
                M += m;
                sx += m * T.fx[i];
                sy += m * T.fy[i];
                sz += m * T.fz[i];
                dmax = std::max(dmax, T.pdisp[i]);
            }
        } else {
            for (int ch = k + 1; ch < q.next; ch = T.nodes[ch].next) {
                const Node& cq = T.nodes[ch];
                M += cq.m;
                sx += double(cq.m) * cq.cx;
                sy += double(cq.m) * cq.cy;
                sz += double(cq.m) * cq.cz;
                dmax = std::max(dmax, T.ndisp[ch]);
            }
        }
        T.ndisp[k] = dmax;
        const double inv = M > 0 ? 1.0 / M : 0.0;
        q.cx = float(sx * inv);
        q.cy = float(sy * inv);
        q.cz = float(sz * inv);
        q.m = float(M);
        const double ox = sx * inv - q.gx, oy = sy * inv - q.gy, oz = sz * inv - q.gz;
        q.open_r = float(2 * (q.half + dmax) / T.theta + std::sqrt(ox * ox + oy * oy + oz * oz));
    }
}

// Walk of one sphere: the interaction list of accepted nodes and opened-leaf particles.
template <class Append>
void walk_list(const Octree& T, float bx, float by, float bz, float br, Append&& append) {
    const Node* nd = T.nodes.data();
    const int nn = int(T.nodes.size());
    for (int k = 0; k < nn;) {
        const Node& q = nd[k];
        const float dx = q.cx - bx, dy = q.cy - by, dz = q.cz - bz;
        const float t = q.open_r + br;
        if (dx * dx + dy * dy + dz * dz > t * t) {
            append(q.cx, q.cy, q.cz, q.m);
            k = q.next;
        } else if (q.leaf) {
            for (int j = q.start; j < q.start + q.count; ++j) append(T.fx[j], T.fy[j], T.fz[j], T.fm[j]);
            k = q.next;
        } else {
            ++k;
        }
    }
}

// Walk items of <= chunk active particles (the library's GF_OPT_WALK_CHUNK; no reference
// counterpart): a group's active particles in tree order are cut into items, each walked
// with the bounding sphere (float32 box centre, radius padded by 1e-6) of its own particles.
// Codes 65..96: runs of consecutive sibling groups (the same parent node) cut greedily into
// items of <= 2 (code - 64) active particles (an item takes its first group whatever its
// count), each walked with the sphere of its active particles; items without one are skipped.
int g_walk_chunk = 0;
constexpr int kChunkMax = 64;

// [first, end) tree positions of the merged-by-active-count items of an active set.
std::vector<std::pair<int, int>> merged_active_items(const Octree& T, const uint8_t* active, int cap) {
    const Node* nd = T.nodes.data();
    const int nn = int(T.nodes.size());
    std::vector<int> par(nn, -1);
    for (int k = 0; k < nn; ++k) {
        if (nd[k].leaf) continue;
        const int end = nd[k].next < 0 ? nn : nd[k].next;
        for (int c = k + 1; c < end && c >= 0; c = nd[c].next) par[c] = k;
    }
    std::vector<std::pair<int, int>> items;
    const int ng = int(T.groups.size());
    for (int g = 0; g < ng;) {
        int e = g + 1;  // the run of groups with g's parent
        while (e < ng && par[T.groups[e]] == par[T.groups[g]]) ++e;
        int start = g, w = 0;
        auto close = [&](int from, int to, int weight) {
            if (weight > 0) items.emplace_back(nd[T.groups[from]].start, nd[T.groups[to - 1]].start +
                                                                              nd[T.groups[to - 1]].count);
        };
        for (int l = g; l < e; ++l) {
            const Node& G = nd[T.groups[l]];
            int c = 0;
            for (int i = G.start; i < G.start + G.count; ++i) c += active[T.order[i]] ? 1 : 0;
            if (l > start && w + c <= cap) {
                w += c;
                continue;
            }
            if (l > start) {
                close(start, l, w);
                start = l;
            }
            w = c;
        }
        close(start, e, w);
        g = e;
    }
    return items;
}

// Group walk + list evaluation (cpp/nbody.cpp:323-411).
void accel(Octree& T, double* acc, double eps, const uint8_t* active) {
    const float eps2 = float(eps * eps);
    const Node* nd = T.nodes.data();
    const int ng = int(T.groups.size());
    const float* px = T.fx.data();
    const float* py = T.fy.data();
    const float* pz = T.fz.data();
    const float* pm = T.fm.data();
    const bool merged = active && g_walk_chunk > kChunkMax;
    const std::vector<std::pair<int, int>> items =
        merged ? merged_active_items(T, active, 2 * (g_walk_chunk - kChunkMax)) : std::vector<std::pair<int, int>>();
    const int nitems = int(items.size());
#pragma omp parallel
    {
        std::vector<float> lx(8192), ly(8192), lz(8192), lm(8192);
        int len = 0;
        auto append = [&](float a, float b, float c, float d) {
            if (len == int(lx.size())) {
                const size_t s = 2 * lx.size();
                lx.resize(s);
                ly.resize(s);
                lz.resize(s);
                lm.resize(s);
            }
            lx[len] = a;
            ly[len] = b;
            lz[len] = c;
            lm[len] = d;
            ++len;
        };
        auto eval = [&](int p) {
            const float x = px[p], y = py[p], z = pz[p];
            float sx = 0, sy = 0, sz = 0;
#pragma omp simd reduction(+ : sx, sy, sz)
            for (int j = 0; j < len; ++j) {
                const float ex = lx[j] - x, ey = ly[j] - y, ez = lz[j] - z;
                const float r2 = ex * ex + ey * ey + ez * ez + eps2;
                const float inv = 1.0f / std::sqrt(r2);
                const float f = lm[j] * inv * inv * inv;
                sx += f * ex;
                sy += f * ey;
                sz += f * ez;
            }
            const int k = T.order[p];
            acc[3 * k] = sx;
            acc[3 * k + 1] = sy;
            acc[3 * k + 2] = sz;
        };
        if (merged) {
#pragma omp for schedule(dynamic, 4)
            for (int it = 0; it < nitems; ++it) {
                const int b = items[it].first, e = items[it].second;
                float x0 = 1e30f, y0 = 1e30f, z0 = 1e30f, x1 = -1e30f, y1 = -1e30f, z1 = -1e30f;
                for (int i = b; i < e; ++i) {
                    if (!active[T.order[i]]) continue;
                    x0 = std::min(x0, px[i]); x1 = std::max(x1, px[i]);
                    y0 = std::min(y0, py[i]); y1 = std::max(y1, py[i]);
                    z0 = std::min(z0, pz[i]); z1 = std::max(z1, pz[i]);
                }
                const float bx = 0.5f * (x0 + x1), by = 0.5f * (y0 + y1), bz = 0.5f * (z0 + z1);
                float br2 = 0;
                for (int i = b; i < e; ++i) {
                    if (!active[T.order[i]]) continue;
                    const float dx = px[i] - bx, dy = py[i] - by, dz = pz[i] - bz;
                    br2 = std::max(br2, dx * dx + dy * dy + dz * dz);
                }
                len = 0;
                walk_list(T, bx, by, bz, std::sqrt(br2) * (1.f + 1e-6f), append);
                for (int i = b; i < e; ++i)
                    if (active[T.order[i]]) eval(i);
            }
        } else {
#pragma omp for schedule(dynamic, 4)
        for (int g = 0; g < ng; ++g) {
            const Node& G = nd[T.groups[g]];
            const int b = G.start, e = G.start + G.count;
            if (active && g_walk_chunk > 0) {
                std::vector<int> act;
                for (int i = b; i < e; ++i)
                    if (active[T.order[i]]) act.push_back(i);
                for (size_t c0 = 0; c0 < act.size(); c0 += size_t(g_walk_chunk)) {
                    const size_t c1 = std::min(act.size(), c0 + size_t(g_walk_chunk));
                    float x0 = 1e30f, y0 = 1e30f, z0 = 1e30f, x1 = -1e30f, y1 = -1e30f, z1 = -1e30f;
                    for (size_t a = c0; a < c1; ++a) {
                        const int i = act[a];
                        x0 = std::min(x0, px[i]); x1 = std::max(x1, px[i]);
                        y0 = std::min(y0, py[i]); y1 = std::max(y1, py[i]);
                        z0 = std::min(z0, pz[i]); z1 = std::max(z1, pz[i]);
                    }
                    const float bx = 0.5f * (x0 + x1), by = 0.5f * (y0 + y1), bz = 0.5f * (z0 + z1);
                    float br2 = 0;
                    for (size_t a = c0; a < c1; ++a) {
                        const int i = act[a];
                        const float dx = px[i] - bx, dy = py[i] - by, dz = pz[i] - bz;
                        br2 = std::max(br2, dx * dx + dy * dy + dz * dz);
                    }
                    len = 0;
                    walk_list(T, bx, by, bz, std::sqrt(br2) * (1.f + 1e-6f), append);
                    for (size_t a = c0; a < c1; ++a) eval(act[a]);
                }
                continue;
            }
            if (active) {
                bool any = false;
                for (int i = b; i < e && !any; ++i) any = active[T.order[i]] != 0;
                if (!any) continue;
            }
            float x0 = 1e30f, y0 = 1e30f, z0 = 1e30f, x1 = -1e30f, y1 = -1e30f, z1 = -1e30f;
            for (int i = b; i < e; ++i) {
                if (pm[i] <= 0) continue;
                x0 = std::min(x0, px[i]);
                x1 = std::max(x1, px[i]);
                y0 = std::min(y0, py[i]);
                y1 = std::max(y1, py[i]);
                z0 = std::min(z0, pz[i]);
                z1 = std::max(z1, pz[i]);
            }
            const float bx = 0.5f * (x0 + x1), by = 0.5f * (y0 + y1), bz = 0.5f * (z0 + z1);
            float br2 = 0;
            for (int i = b; i < e; ++i) {
                if (pm[i] <= 0) continue;
                const float dx = px[i] - bx, dy = py[i] - by, dz = pz[i] - bz;
                br2 = std::max(br2, dx * dx + dy * dy + dz * dz);
            }
            if (x0 > x1) continue;
            const float br = std::sqrt(br2);

            len = 0;
            walk_list(T, bx, by, bz, br, append);
            for (int p = b; p < e; ++p) {
                if (active && !active[T.order[p]]) continue;
                eval(p);
            }
        }
        }  // groups
    }
}

// ---- SPH (galaxy_formation/sph.py) ------------------------------------------------------

constexpr double kPi = 3.14159265358979323846;

// Cubic-spline M4 kernel, support 2h (sph.py:31-40).
inline double w_m4(double r, double h) {
    const double q = r / h;
    const double s = 1.0 / (kPi * h * h * h);
    if (q < 1.0) return s * (1 - 1.5 * q * q + 0.75 * q * q * q);
    if (q < 2.0) {
        const double t = 2 - q;
        return s * 0.25 * t * t * t;
    }
    return 0.0;
}

// (1/r) dW/dr (sph.py:43-54).
inline double dw_m4(double r, double h) {
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
    return g / std::max(r, 1e-30);
}

}  // namespace

extern "C" {

int orc_num_threads(void) { return omp_get_max_threads(); }

void orc_set_threads(int t) {
    if (t > 0) omp_set_num_threads(t);
}

void orc_set_walk_chunk(int c) { g_walk_chunk = c > 0 ? c : 0; }  // codes as GF_OPT_WALK_CHUNK

// Mirrors nbody_accel_active (cpp/nbody.cpp:422-425): a process-global tree, rebuilt when
// asked or when n changes, refitted otherwise.
void orc_accel_active(int n, const double* pos, const double* mass, double* acc, double theta,
                      double eps, const uint8_t* active, int rebuild) {
    Octree& T = g_oct;
    if (rebuild || T.n != n || T.nodes.empty())
        build(T, n, pos, mass, theta);
    else
        refit(T, pos, mass);
    accel(T, acc, eps, active);
}

// Mirrors nbody_accel_direct (cpp/nbody.cpp:428-441).
void orc_accel_direct(int n, const double* pos, const double* mass, double* acc, double eps) {
    const double eps2 = eps * eps;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double ax = 0, ay = 0, az = 0;
        for (int j = 0; j < n; ++j) {
            const double dx = pos[3 * j] - pos[3 * i], dy = pos[3 * j + 1] - pos[3 * i + 1],
                         dz = pos[3 * j + 2] - pos[3 * i + 2];
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            const double f = mass[j] / (r2 * std::sqrt(r2));
            ax += f * dx;
            ay += f * dy;
            az += f * dz;
        }
        acc[3 * i] = ax;
        acc[3 * i + 1] = ay;
        acc[3 * i + 2] = az;
    }
}

// Direct sum for a subset of targets (same arithmetic), used for error reports at sizes
// where the full O(N^2) sum is too slow.
void orc_accel_direct_targets(int n, const double* pos, const double* mass, int nt,
                              const int64_t* targets, double* acc, double eps) {
    const double eps2 = eps * eps;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nt; ++t) {
        const int64_t i = targets[t];
        double ax = 0, ay = 0, az = 0;
        for (int j = 0; j < n; ++j) {
            const double dx = pos[3 * j] - pos[3 * i], dy = pos[3 * j + 1] - pos[3 * i + 1],
                         dz = pos[3 * j + 2] - pos[3 * i + 2];
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            const double f = mass[j] / (r2 * std::sqrt(r2));
            ax += f * dx;
            ay += f * dy;
            az += f * dz;
        }
        acc[3 * t] = ax;
        acc[3 * t + 1] = ay;
        acc[3 * t + 2] = az;
    }
}

// Tree inspection for structural parity tests.
int orc_tree_num_nodes(void) { return int(g_oct.nodes.size()); }
int orc_tree_num_groups(void) { return int(g_oct.groups.size()); }

// Copies the last tree out. ints: (nn, 4) start, count, next, leaf; floats: (nn, 9)
// cx, cy, cz, m, open_r, gx, gy, gz, half; order: (n,); groups: (ng,).
void orc_tree_export(int32_t* ints, float* floats, int32_t* order, int32_t* groups) {
    const Octree& T = g_oct;
    const int nn = int(T.nodes.size());
    for (int k = 0; k < nn; ++k) {
        const Node& q = T.nodes[k];
        ints[4 * k] = q.start;
        ints[4 * k + 1] = q.count;
        ints[4 * k + 2] = q.next;
        ints[4 * k + 3] = q.leaf;
        const float f[9] = {q.cx, q.cy, q.cz, q.m, q.open_r, q.gx, q.gy, q.gz, q.half};
        std::memcpy(floats + 9 * size_t(k), f, sizeof f);
    }
    std::memcpy(order, T.order.data(), sizeof(int32_t) * size_t(T.n));
    std::memcpy(groups, T.groups.data(), sizeof(int32_t) * T.groups.size());
}

double orc_sph_kernel(double r, double h) { return w_m4(r, h); }
double orc_sph_kernel_grad(double r, double h) { return dw_m4(r, h); }

// Density, pressure + viscosity acceleration, du/dt and Courant step (sph.py:57-106).
// nb: (n, k) local neighbour indices, the particle itself included.
void orc_sph_forces(int n, int k, const double* pos, const double* vel, const double* mass,
                    const int64_t* nb, const double* h, const double* u, double gamma,
                    double alpha, double beta, double* rho, double* acc, double* dudt,
                    double* dt_i) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double s = 0.0;
        for (int jj = 0; jj < k; ++jj) {
            const int64_t j = nb[size_t(i) * k + jj];
            const double dx = pos[3 * i] - pos[3 * j], dy = pos[3 * i + 1] - pos[3 * j + 1],
                         dz = pos[3 * i + 2] - pos[3 * j + 2];
            s += mass[j] * w_m4(std::sqrt(dx * dx + dy * dy + dz * dz), h[i]);
        }
        rho[i] = s;
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const double Pi = (gamma - 1) * rho[i] * u[i];
        const double ci = std::sqrt(gamma * (gamma - 1) * u[i]);
        const double pri = Pi / (rho[i] * rho[i]);
        double ax = 0, ay = 0, az = 0, du = 0, mu_max = 0;
        for (int jj = 0; jj < k; ++jj) {
            const int64_t j = nb[size_t(i) * k + jj];
            if (j == i) continue;
            const double dx = pos[3 * i] - pos[3 * j], dy = pos[3 * i + 1] - pos[3 * j + 1],
                         dz = pos[3 * i + 2] - pos[3 * j + 2];
            const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
            const double gi = dw_m4(r, h[i]);
            const double gj = dw_m4(r, h[j]);
            const double Pj = (gamma - 1) * rho[j] * u[j];
            const double cj = std::sqrt(gamma * (gamma - 1) * u[j]);
            const double vr = (vel[3 * i] - vel[3 * j]) * dx + (vel[3 * i + 1] - vel[3 * j + 1]) * dy +
                              (vel[3 * i + 2] - vel[3 * j + 2]) * dz;
            double visc = 0.0;
            if (vr < 0) {
                const double hb = 0.5 * (h[i] + h[j]);
                const double mu = hb * vr / (r * r + 0.01 * hb * hb);
                mu_max = std::max(mu_max, -mu);
                visc = (-alpha * 0.5 * (ci + cj) * mu + beta * mu * mu) / (0.5 * (rho[i] + rho[j]));
            }
            const double gb = 0.5 * (gi + gj);
            const double f = pri * gi + Pj / (rho[j] * rho[j]) * gj + visc * gb;
            ax -= mass[j] * f * dx;
            ay -= mass[j] * f * dy;
            az -= mass[j] * f * dz;
            du += mass[j] * (pri * gi + 0.5 * visc * gb) * vr;
        }
        acc[3 * i] = ax;
        acc[3 * i + 1] = ay;
        acc[3 * i + 2] = az;
        dudt[i] = du;
        dt_i[i] = 0.3 * h[i] / (ci + 1.2 * (alpha * ci + beta * mu_max) + 1e-30);
    }
}

// k nearest among each particle's candidates (sph.py:109-135). cand: (n, m) local indices,
// -1 = none. Returns 1 when every particle had at least k candidates, else 0 (rows of
// particles without enough candidates are left untouched, as in the reference).
int orc_knn_from_candidates(int n, int m, const double* pos, const int64_t* cand, int k,
                            int64_t* nb, double* dist) {
    int ok = 1;
#pragma omp parallel
    {
        std::vector<double> d2(m);
        std::vector<int> idx(m);
#pragma omp for schedule(static) reduction(&& : ok)
        for (int i = 0; i < n; ++i) {
            int cnt = 0;
            for (int jj = 0; jj < m; ++jj) {
                const int64_t j = cand[size_t(i) * m + jj];
                if (j < 0) {
                    d2[jj] = INFINITY;
                    continue;
                }
                const double dx = pos[3 * i] - pos[3 * j], dy = pos[3 * i + 1] - pos[3 * j + 1],
                             dz = pos[3 * i + 2] - pos[3 * j + 2];
                d2[jj] = dx * dx + dy * dy + dz * dz;
                ++cnt;
            }
            if (cnt < k) {
                ok = 0;
                continue;
            }
            std::iota(idx.begin(), idx.end(), 0);
            std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return d2[a] < d2[b]; });
            for (int jj = 0; jj < k; ++jj) {
                nb[size_t(i) * k + jj] = cand[size_t(i) * m + idx[jj]];
                dist[size_t(i) * k + jj] = std::sqrt(d2[idx[jj]]);
            }
        }
    }
    return ok;
}

// Exact k nearest neighbours of every point among all points (self included, distance
// ascending, ties by index), brute force O(n^2): the oracle for the neighbour search.
void orc_knn_brute(int n, const double* pos, int k, double* dist, int64_t* nb) {
#pragma omp parallel
    {
        std::vector<std::pair<double, int>> d2(n);
#pragma omp for schedule(dynamic, 16)
        for (int i = 0; i < n; ++i) {
            for (int j = 0; j < n; ++j) {
                const double dx = pos[3 * i] - pos[3 * j], dy = pos[3 * i + 1] - pos[3 * j + 1],
                             dz = pos[3 * i + 2] - pos[3 * j + 2];
                d2[j] = {dx * dx + dy * dy + dz * dz, j};
            }
            const int kk = std::min(k, n);
            std::partial_sort(d2.begin(), d2.begin() + kk, d2.end());
            for (int jj = 0; jj < kk; ++jj) {
                dist[size_t(i) * k + jj] = std::sqrt(d2[jj].first);
                nb[size_t(i) * k + jj] = d2[jj].second;
            }
        }
    }
}

// Orthographic projection with a bilinear deposit of four weights per particle into
// img (ngroups, H, W), as cpp/nbody.cpp:445-469; serial, so the float sums of a pixel come
// in particle order.
void orc_render(int n, const double* pos, const uint8_t* group, int ngroups, const double* rot,
                const double* center, double scale, int W, int H, float* img) {
    const size_t plane = size_t(W) * H;
    for (size_t t = 0; t < size_t(ngroups) * plane; ++t) img[t] = 0.0f;
    for (int i = 0; i < n; ++i) {
        const double x = pos[3 * size_t(i)] - center[0];
        const double y = pos[3 * size_t(i) + 1] - center[1];
        const double z = pos[3 * size_t(i) + 2] - center[2];
        const double sx = rot[0] * x + rot[1] * y + rot[2] * z;
        const double sy = rot[3] * x + rot[4] * y + rot[5] * z;
        const double u = 0.5 * W + scale * sx - 0.5, v = 0.5 * H - scale * sy - 0.5;
        if (!(u >= 0 && v >= 0 && u < W - 1 && v < H - 1)) continue;
        const int iu = int(u), iv = int(v);
        const float fu = float(u - iu), fv = float(v - iv);
        float* p = img + size_t(group[i]) * plane + size_t(iv) * W + iu;
        p[0] += (1 - fu) * (1 - fv);
        p[1] += fu * (1 - fv);
        p[W] += (1 - fu) * fv;
        p[W + 1] += fu * fv;
    }
}

// 8-bit RGB from the group images (cpp/nbody.cpp:474-503): per group a log-compressed
// brightness plus a bilinearly upsampled glow, weighted by the group colour, then the soft
// saturation 255 (1 - exp(-exposure s)), rounded.
void orc_tonemap(int W, int H, int ngroups, const float* img, const float* glow, int gw, int gh,
                 const float* colors, float inv_ref, float K, float exposure, uint8_t* out) {
    const size_t plane = size_t(W) * H, gplane = size_t(gw) * gh;
    const float norm = 1.0f / std::log1p(K);
    const float ax = float(gw) / W, ay = float(gh) / H;
    for (int y = 0; y < H; ++y) {
        const float gyf = std::min(std::max((y + 0.5f) * ay - 0.5f, 0.0f), gh - 1.001f);
        const int gy = int(gyf);
        const float fy = gyf - gy;
        for (int x = 0; x < W; ++x) {
            const float gxf = std::min(std::max((x + 0.5f) * ax - 0.5f, 0.0f), gw - 1.001f);
            const int gx = int(gxf);
            const float fx = gxf - gx;
            float c[3] = {0, 0, 0};
            for (int g = 0; g < ngroups; ++g) {
                const float* q = glow + g * gplane + size_t(gy) * gw + gx;
                const float glow_v = (1 - fy) * ((1 - fx) * q[0] + fx * q[1]) + fy * ((1 - fx) * q[gw] + fx * q[gw + 1]);
                const float l = std::log1p(K * inv_ref * img[g * plane + size_t(y) * W + x]) * norm + glow_v;
                for (int a = 0; a < 3; ++a) c[a] += l * colors[3 * g + a];
            }
            for (int a = 0; a < 3; ++a)
                out[3 * (size_t(y) * W + x) + a] = uint8_t(255.0f * (1 - std::exp(-exposure * c[a])) + 0.5f);
        }
    }
}

}  // extern "C"
