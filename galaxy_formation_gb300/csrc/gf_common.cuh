// gf_common.cuh — shared definitions of the GB300 force library (libgfgpu.so).
//
// Error model: internal host code throws gf::Error; every extern "C" entry point catches it
// and turns it into a status word readable through gf_last_status()/gf_last_error().
// Kernels never trap: they OR a bit into a device status word (ctx.d_status) and return.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/gfgpu.h"

namespace gf {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define GF_CUDA(call)                                                  \
    do {                                                               \
        cudaError_t gf_e_ = (call);                                    \
        if (gf_e_ != cudaSuccess) gf::cuda_fail(gf_e_, #call, __FILE__, __LINE__); \
    } while (0)

#define GF_CHECK_LAUNCH()               \
    do {                                \
        GF_CUDA(cudaGetLastError());    \
        ++gf::ctx().launches;           \
    } while (0)

// Bumped whenever any DevBuf (re)allocates: a captured CUDA graph that bakes buffer
// addresses is valid only while this stays unchanged.
extern unsigned long long g_alloc_generation;
// Set while a CUDA graph is being captured: a buffer that would have to grow then is an error
// (an allocation inside a capture fails, and the captured addresses must stay valid).
extern bool g_no_alloc;

// A grow-only device allocation.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    template <class T>
    T* get(size_t count) {
        const size_t need = count * sizeof(T) + 256;
        if (need > bytes) {
            if (g_no_alloc) throw Error(GF_ERR_CAPACITY, "a device buffer would grow inside a captured step");
            if (p) GF_CUDA(cudaFree(p));
            p = nullptr;
            bytes = 0;
            GF_CUDA(cudaMalloc(&p, need));
            bytes = need;
            ++g_alloc_generation;
        }
        return static_cast<T*>(p);
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
};

constexpr int kWarp = 32;

__host__ __device__ inline int div_up(long long a, long long b) { return int((a + b - 1) / b); }

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ int warp_incl_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ int warp_sum(int v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One round of a warp's tree walk over a shared-memory stack of child ranges (entry =
// first << 4 | count, count 1..8, top at sp - 1): takes whole ranges from the top while they fit
// in 32 * NPL node slots and the head of the next one (the rest of that range stays on the
// stack). Slot s = lane + 32 i gets node[i] (-1 when empty); returns the number of nodes taken.
// The node of a slot is found by a binary search over the ranges' inclusive sums (shuffles
// only, no shared-memory staging), so the slots past the first 32 cost nothing in rounds that
// fill fewer. The caller synchronises the warp before the stack is read again.
template <int NPL>
__device__ __forceinline__ int pop_round(int* stack, int& sp, int (&node)[NPL]) {
    constexpr int kRound = 32 * NPL;
    const int lane = threadIdx.x & 31;
    const int kk = min(sp, 32);
    int e = 0, c = 0;
    if (lane < kk) {
        e = stack[sp - 1 - lane];
        c = e & 15;
    }
    const int incl = warp_incl_scan(c);
    const int excl = incl - c;
    const unsigned fullm = __ballot_sync(0xffffffffu, lane < kk && incl <= kRound);
    const int nfull = __popc(fullm);
    int nnodes = __shfl_sync(0xffffffffu, incl, kk - 1);
    if (nfull < kk) {  // range `nfull` is split: its tail stays on the stack
        nnodes = kRound;
        if (lane == nfull) {
            const int take = kRound - excl;
            stack[sp - 1 - lane] = (((e >> 4) + take) << 4) | (c - take);
        }
    }
    sp -= nfull;
    const int incl2 = min(incl, kRound);
    const int first = e >> 4;
#pragma unroll
    for (int i = 0; i < NPL; ++i) {
        node[i] = -1;
        if (32 * i < nnodes) {  // warp-uniform
            const int slot = lane + 32 * i;
            int src = 0;  // ranges ending at or before the slot
#pragma unroll
            for (int step = 16; step; step >>= 1) {
                const int v = __shfl_sync(0xffffffffu, incl2, src + step - 1);
                if (v <= slot) src += step;
            }
            const int f = __shfl_sync(0xffffffffu, first, src);
            const int x = __shfl_sync(0xffffffffu, excl, src);
            if (slot < nnodes) node[i] = f + (slot - x);
        }
    }
    return nnodes;
}

// Kahan-compensated float32 sum.
struct KahanF {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float v) {
        const float y = v - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

// In-place ascending bitonic sort of P (power of two <= 128) keys in shared memory by the
// calling warp; ties broken by the integer tag. Non-negative float64 distances are sorted by
// their bit patterns as unsigned 64-bit integers (the same order, including +inf): integer
// compares avoid the float64 pipe, which is narrow on this GPU.
template <class K>
__device__ inline void warp_bitonic(K* key, int* tag, int P) {
    const int lane = threadIdx.x & 31;
    for (int size = 2; size <= P; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = lane; t < P / 2; t += 32) {
                const int a = ((t & ~(stride - 1)) << 1) | (t & (stride - 1));
                const int b = a + stride;
                const bool up = (a & size) == 0;
                const K ka = key[a], kb = key[b];
                const int ta = tag[a], tb = tag[b];
                const bool gt = ka > kb || (ka == kb && ta > tb);
                if (gt == up) {
                    key[a] = kb;
                    key[b] = ka;
                    tag[a] = tb;
                    tag[b] = ta;
                }
            }
            __syncwarp();
        }
    }
}

// Ascending bitonic sort of P (power of two <= 128) 64-bit keys in shared memory by the
// calling warp (keys are unique when they carry an index in their low bits). (A register
// version, keys exchanged by shuffles, removed the shared-memory bank conflicts but slowed the
// neighbour search: more instructions and register spills in an issue-bound kernel.)
__device__ inline void warp_sort_u64(unsigned long long* key, int P) {
    const int lane = threadIdx.x & 31;
    for (int size = 2; size <= P; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = lane; t < P / 2; t += 32) {
                const int a = ((t & ~(stride - 1)) << 1) | (t & (stride - 1));
                const int b = a + stride;
                const bool up = (a & size) == 0;
                const unsigned long long ka = key[a], kb = key[b];
                if ((ka > kb) == up) {
                    key[a] = kb;
                    key[b] = ka;
                }
            }
            __syncwarp();
        }
    }
}

// atomicAdd with acquire-release semantics at GPU scope (bottom-up tree passes: the last
// arriving child sees its siblings' records without separate fences)
__device__ __forceinline__ int atom_add_acq_rel(int* p, int v) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

__device__ __forceinline__ void raise_status(uint32_t* st, uint32_t bit) {
    if (st) atomicOr(st, bit);
}

// Scratch of exclusive_scan / radix_sort_pairs. Work queued on different streams at the same
// time needs different scratch (null = the context's, for the library's main stream).
struct ScanScratch {
    DevBuf scan_tmp, sort_tmp;
};

// Device-wide exclusive scan of int32 (n may be 0). `total` (device) receives the sum.
void exclusive_scan(const int* in, int* out, int n, int* total, cudaStream_t s, ScanScratch* sc = nullptr);

// Sizes the scratch of exclusive_scan / radix_sort_pairs for inputs of up to n elements.
void reserve_scan_sort(int n, ScanScratch* sc = nullptr);

// Stable LSD radix sort of (key, value) pairs on bits [bit_lo, bit_hi) of the keys.
// Results end in keys/vals (the alternate buffers are scratch of the same size).
void radix_sort_pairs(uint64_t* keys, int* vals, uint64_t* keys_alt, int* vals_alt, int n,
                      int bit_lo, int bit_hi, cudaStream_t s, ScanScratch* sc = nullptr);

// A subset of particles to process: idx[0 .. *count) (device memory, count read on the
// device so the launch stays valid inside a captured graph); idx == null means all n.
struct Subset {
    const int* idx = nullptr;
    const int* count = nullptr;
};

// Item t of a launch over n slots: false when past the subset; `base` maps t -> particle
// when processing everything (e.g. a visiting order; null = identity).
__device__ __forceinline__ bool subset_item(const Subset& S, int t, int n, const int* base, int& i) {
    if (S.idx) {
        if (t >= *S.count) return false;
        i = S.idx[t];
        return true;
    }
    if (t >= n) return false;
    i = base ? base[t] : t;
    return true;
}

// A CUDA event for host-side timing on a stream.
struct Event {
    cudaEvent_t e = nullptr;
    Event() { GF_CUDA(cudaEventCreate(&e)); }
    ~Event() {
        if (e) cudaEventDestroy(e);
    }
    Event(const Event&) = delete;
    Event& operator=(const Event&) = delete;
    void record(cudaStream_t s) { GF_CUDA(cudaEventRecord(e, s)); }
    float since(const Event& a) const {  // ms from a to this (both recorded and complete)
        float ms = 0.f;
        GF_CUDA(cudaEventElapsedTime(&ms, a.e, e));
        return ms;
    }
};

// Timed stages (CUDA events recorded on the launching stream while profiling is on).
enum Stage {
    kStTreeBuild = 0,  // whole gravity tree build (bbox .. walk layout)
    kStTreeRefit,      // refit
    kStWalk,           // the walk kernel (k_walk_mono) alone
    kStGroupPrep,      // work list of active groups
    kStKnn,            // neighbour-search kernel (k_knn) alone
    kStKnnTree,        // octree of the gas for the neighbour search
    kStSphDensity,     // density kernel alone
    kStSphForce,       // force kernel alone
    kStVerlet,         // Verlet reselection
    kStForce,          // one whole force evaluation
    kStTreeSort,       // radix sort of the gravity tree's Morton keys
    kStTreeEmit,       // node emission of the gravity tree (k_emit)
    kStTreeMoments,    // moments pass of the gravity tree build
    kStCount
};

struct Profiler {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> recs[kStCount];
    cudaEvent_t take();
    void clear();
};

// Records the start/stop events of a stage around a scope (no-op when profiling is off).
struct ProfScope {
    int stage;
    cudaStream_t s;
    bool on;
    ProfScope(int st, cudaStream_t st_s);
    ~ProfScope();
};

// Per-process state shared by every entry point.
struct Context {
    bool ready = false;
    int device = -1;
    int sms = 0;
    cudaStream_t stream = nullptr;
    uint32_t* d_status = nullptr;   // device status word (kernels OR bits into it)
    uint32_t* h_status = nullptr;   // pinned host mirror
    int last_status = 0;
    std::string last_error;
    DevBuf scan_tmp, sort_tmp;      // scratch of the scan / radix sort
    long long launches = 0;         // kernels launched since load
    Profiler prof;
};

Context& ctx();
void ensure_ready();
// Measured float32 FFMA throughput of this GPU (TFLOP/s, FMA = 2 flops), best of 5.
double fp32_peak_tflops();
// Adds the device status word to the host status and clears it (synchronises `s`).
int collect_status(cudaStream_t s);

}  // namespace gf
