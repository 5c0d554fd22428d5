// gf_core.cu — library context, status handling, device-wide scan and radix sort.
//
// Radix sort: stable LSD sort of (uint64 key, int32 value) pairs, 8-bit digits, one sweep
// per digit (the single-pass scheme of Adinets & Merrill, "Onesweep", 2022):
//   histogram  one launch reads the keys once and counts the digits of every pass,
//   pass       one launch per digit: each block takes the next tile by ticket, ranks its keys
//              stably (__match_any_sync per warp, warps in key order), publishes its digit
//              counts, adds up the counts of the tiles before it by decoupled look-back (a
//              tile's flag says whether its value is its own count or the inclusive prefix;
//              waits are bounded, GF_ERR_TIMEOUT past the bound) and scatters each key to
//              (keys of smaller digits) + (its digit in earlier tiles) + its rank.
// Tiles are 2048 keys (256 threads x 8). Traffic per pass: 12 B read + 12 B write per pair,
// plus 8 B per pair once for the histogram.
#include <cstdarg>
#include <algorithm>
#include <cstring>

#include "gf_common.cuh"

namespace gf {

static Context g_ctx;
unsigned long long g_alloc_generation = 0;
bool g_no_alloc = false;

Context& ctx() { return g_ctx; }

void cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
    char buf[512];
    snprintf(buf, sizeof buf, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    throw Error(GF_ERR_CUDA, buf);
}

void ensure_ready() {
    Context& c = g_ctx;
    if (c.ready) return;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        throw Error(GF_ERR_NO_DEVICE, "no CUDA device");
    }
    GF_CUDA(cudaGetDevice(&c.device));
    GF_CUDA(cudaDeviceGetAttribute(&c.sms, cudaDevAttrMultiProcessorCount, c.device));
    GF_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    GF_CUDA(cudaMalloc(&c.d_status, sizeof(uint32_t)));
    GF_CUDA(cudaMemset(c.d_status, 0, sizeof(uint32_t)));
    GF_CUDA(cudaMallocHost(&c.h_status, sizeof(uint32_t)));
    *c.h_status = 0;
    c.ready = true;
}

cudaEvent_t Profiler::take() {
    if (!pool.empty()) {
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    GF_CUDA(cudaEventCreate(&e));
    return e;
}

void Profiler::clear() {
    for (auto& v : recs) {
        for (auto& pr : v) {
            pool.push_back(pr.first);
            pool.push_back(pr.second);
        }
        v.clear();
    }
}

// a stage id outside [0, kStCount) records nothing
ProfScope::ProfScope(int st, cudaStream_t st_s)
    : stage(st), s(st_s), on(g_ctx.prof.on && st >= 0 && st < kStCount) {
    if (!on) return;
    Profiler& P = g_ctx.prof;
    cudaEvent_t a = P.take(), b = P.take();
    P.recs[stage].push_back({a, b});
    GF_CUDA(cudaEventRecord(a, s));
}

ProfScope::~ProfScope() {
    if (!on) return;
    cudaEventRecord(g_ctx.prof.recs[stage].back().second, s);
}

int collect_status(cudaStream_t s) {
    Context& c = g_ctx;
    GF_CUDA(cudaMemcpyAsync(c.h_status, c.d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    GF_CUDA(cudaMemsetAsync(c.d_status, 0, sizeof(uint32_t), s));
    GF_CUDA(cudaStreamSynchronize(s));
    const int st = int(*c.h_status);
    if (st) {
        c.last_status |= st;
        if (c.last_error.empty()) {
            char buf[128];
            snprintf(buf, sizeof buf, "device status 0x%x", st);
            c.last_error = buf;
        }
    }
    return st;
}

// ---------------------------------------------------------------------------------------
// exclusive scan (int32): tile sums -> scan of tile sums -> per-tile scan + offset (up to
// kScanDirectTiles tiles the last two steps are one launch)

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int block_excl_scan(int v, int* s_warp, int* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    int incl = warp_incl_scan(v);
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int w = lane < nw ? s_warp[lane] : 0;
        int wi = warp_incl_scan(w);
        if (lane < nw) s_warp[lane] = wi - w;
        if (lane == nw - 1) s_warp[32] = wi;
    }
    __syncthreads();
    const int r = incl - v + s_warp[warp];
    if (total) *total = s_warp[32];
    __syncthreads();
    return r;
}

__global__ void k_scan_tile_sums(const int* __restrict__ in, int n, int* __restrict__ sums) {
    __shared__ int s_warp[33];
    const int base = blockIdx.x * kScanTile;
    int acc = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int i = base + k * kScanThreads + threadIdx.x;
        if (i < n) acc += in[i];
    }
    int tot;
    block_excl_scan(acc, s_warp, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// single block: exclusive scan of `cnt` tile sums in place, total to *total
__global__ void k_scan_sums(int* sums, int cnt, int* total) {
    __shared__ int s_warp[33];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < cnt; base += blockDim.x * kScanItems) {
        int v[kScanItems];
        int acc = 0;
        const int b0 = base + threadIdx.x * kScanItems;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            v[k] = (b0 + k < cnt) ? sums[b0 + k] : 0;
            acc += v[k];
        }
        int tot;
        int ex = block_excl_scan(acc, s_warp, &tot) + carry;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            if (b0 + k < cnt) sums[b0 + k] = ex;
            ex += v[k];
        }
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void k_scan_tiles(const int* __restrict__ in, int* __restrict__ out, int n,
                             const int* __restrict__ offs) {
    __shared__ int s_warp[33];
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    int acc = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        acc += v[k];
    }
    int ex = block_excl_scan(acc, s_warp, nullptr) + offs[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = ex;
        ex += v[k];
    }
}

// Second launch of the two-launch scan: each block adds up the tile sums before its own tile
// (at most kScanDirectTiles of them: a few KB of L2 reads per block) and scans its tile; the
// last block writes the total.
constexpr int kScanDirectTiles = 2048;

__global__ void k_scan_tiles_direct(const int* __restrict__ in, int* __restrict__ out, int n,
                                    const int* __restrict__ sums, int* __restrict__ total) {
    __shared__ int s_warp[33];
    int before = 0;
    for (int t = threadIdx.x; t < int(blockIdx.x); t += kScanThreads) before += sums[t];
    int prefix;
    block_excl_scan(before, s_warp, &prefix);
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    int acc = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        acc += v[k];
    }
    int tile_total;
    int ex = block_excl_scan(acc, s_warp, &tile_total) + prefix;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = ex;
        ex += v[k];
    }
    if (total && threadIdx.x == 0 && blockIdx.x == gridDim.x - 1) *total = prefix + tile_total;
}

void exclusive_scan(const int* in, int* out, int n, int* total, cudaStream_t s, ScanScratch* sc) {
    if (n <= 0) {
        if (total) GF_CUDA(cudaMemsetAsync(total, 0, sizeof(int), s));
        return;
    }
    const int tiles = div_up(n, kScanTile);
    int* sums = (sc ? sc->scan_tmp : g_ctx.scan_tmp).get<int>(size_t(tiles) + 1);
    k_scan_tile_sums<<<tiles, kScanThreads, 0, s>>>(in, n, sums);
    GF_CHECK_LAUNCH();
    if (tiles <= kScanDirectTiles) {
        k_scan_tiles_direct<<<tiles, kScanThreads, 0, s>>>(in, out, n, sums, total);
        GF_CHECK_LAUNCH();
        return;
    }
    k_scan_sums<<<1, 1024, 0, s>>>(sums, tiles, total);
    GF_CHECK_LAUNCH();
    k_scan_tiles<<<tiles, kScanThreads, 0, s>>>(in, out, n, sums);
    GF_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------------------
// radix sort

constexpr int kRsThreads = 256;
constexpr int kRsWarps = kRsThreads / 32;
// --- one sweep per digit --------------------------------------------------------------------

constexpr int kOsItems = 8;                   // keys per thread
constexpr int kOsWarpItems = 32 * kOsItems;   // consecutive keys per warp
constexpr int kOsTile = kRsThreads * kOsItems;
constexpr int kOsMaxPasses = 8;
constexpr unsigned kOsAgg = 1u << 30;         // look-back flags: the tile's own count,
constexpr unsigned kOsInc = 2u << 30;         // or the inclusive prefix up to the tile
constexpr unsigned kOsValue = (1u << 30) - 1;
constexpr long kOsSpinMax = 1l << 20;         // bounded waits (a waited-on tile is always running)
constexpr int kOsWindow = 16;                 // look-back statuses loaded at a time

__device__ __forceinline__ unsigned ld_relaxed(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(unsigned* p, unsigned v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Digit counts of every pass: hist[p * 256 + d] (hist zeroed by the caller).
__global__ void __launch_bounds__(kRsThreads) k_os_hist(const uint64_t* __restrict__ keys, int n, int bit_lo,
                                                        int npass, int* __restrict__ hist) {
    __shared__ int h[kOsMaxPasses * 256];
    for (int i = threadIdx.x; i < npass * 256; i += kRsThreads) h[i] = 0;
    __syncthreads();
    for (int i = blockIdx.x * kRsThreads + threadIdx.x; i < n; i += gridDim.x * kRsThreads) {
        const uint64_t k = keys[i];
        for (int p = 0; p < npass; ++p) atomicAdd(&h[p * 256 + int((k >> (bit_lo + 8 * p)) & 255u)], 1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < npass * 256; i += kRsThreads)
        if (h[i]) atomicAdd(&hist[i], h[i]);
}

// One pass: tiles in ticket order; status[tile * 256 + d] holds the flag and value of digit d.
__global__ void __launch_bounds__(kRsThreads) k_os_pass(
    const uint64_t* __restrict__ kin, const int* __restrict__ vin, uint64_t* __restrict__ kout,
    int* __restrict__ vout, int n, int shift, const int* __restrict__ tot, unsigned* __restrict__ status,
    int* __restrict__ ticket, uint32_t* __restrict__ err) {
    __shared__ int s_cnt[kRsWarps][256];
    __shared__ int s_base[256];
    __shared__ int s_warp[33];
    __shared__ int s_tile;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1);
    for (int w = 0; w < kRsWarps; ++w) s_cnt[w][threadIdx.x] = 0;
    // keys of smaller digits (the pass's digit totals, scanned)
    const int gbase = block_excl_scan(tot[threadIdx.x], s_warp, nullptr);  // synchronises
    const int tile = s_tile;
    const int base = tile * kOsTile + warp * kOsWarpItems;
    uint64_t k[kOsItems];
    int v[kOsItems];
    int rank[kOsItems];
    const unsigned lt = lanemask_lt();
#pragma unroll
    for (int s = 0; s < kOsItems; ++s) {
        const int i = base + s * 32 + lane;
        const bool ok = i < n;
        k[s] = ok ? kin[i] : 0ull;
        v[s] = ok ? vin[i] : 0;
    }
#pragma unroll
    for (int s = 0; s < kOsItems; ++s) {
        const int i = base + s * 32 + lane;
        const bool ok = i < n;
        const unsigned d = ok ? unsigned((k[s] >> shift) & 255u) : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int before = ok ? s_cnt[warp][d] : 0;
        rank[s] = before + __popc(peers & lt);
        __syncwarp();
        if (ok && lane == __ffs(peers) - 1) s_cnt[warp][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // thread d: the tile's count of digit d, and the exclusive prefix over warps
    const int d = threadIdx.x;
    int run = 0;
    for (int w = 0; w < kRsWarps; ++w) {
        const int c = s_cnt[w][d];
        s_cnt[w][d] = run;
        run += c;
    }
    unsigned* my = status + size_t(tile) * 256 + d;
    int excl = 0;
    if (tile == 0) {
        st_relaxed(my, kOsInc | unsigned(run));
    } else {
        st_relaxed(my, kOsAgg | unsigned(run));
        // look back over the tiles before this one until an inclusive prefix, kOsWindow
        // statuses loaded at a time (a tile before 0 counts as an inclusive 0); a tile not
        // ready yet is polled again (bounded)
        int j = tile - 1;
        long polls = 0;
        for (;;) {
            unsigned w[kOsWindow];
#pragma unroll
            for (int u = 0; u < kOsWindow; ++u) w[u] = j - u >= 0 ? ld_relaxed(status + size_t(j - u) * 256 + d) : kOsInc;
            int u = 0;
            bool done = false;
#pragma unroll
            for (int t = 0; t < kOsWindow; ++t) {
                if (done || u < t) continue;  // stopped at an inclusive or a tile not ready
                if ((w[t] & ~kOsValue) == 0u) continue;
                excl += int(w[t] & kOsValue);
                if (w[t] & kOsInc) done = true;
                u = t + 1;
            }
            if (done) break;
            j -= u;
            if (u == 0 && ++polls >= kOsSpinMax) {  // gave up: flag it and stop (output invalid)
                raise_status(err, GF_ERR_TIMEOUT);
                break;
            }
        }
        st_relaxed(my, kOsInc | unsigned(excl + run));
    }
    s_base[d] = gbase + excl;
    __syncthreads();
#pragma unroll
    for (int s = 0; s < kOsItems; ++s) {
        const int i = base + s * 32 + lane;
        if (i < n) {
            const unsigned dg = unsigned((k[s] >> shift) & 255u);
            const int pos = s_base[dg] + s_cnt[warp][dg] + rank[s];
            kout[pos] = k[s];
            vout[pos] = v[s];
        }
    }
}

// Scratch of a one-sweep sort of n pairs: digit totals [8][256], tickets [8], tile status
// [8][tiles][256].
size_t os_scratch_ints(int n) {
    const size_t tiles = size_t(div_up(std::max(n, 1), kOsTile));
    return size_t(kOsMaxPasses) * 256 + 64 + size_t(kOsMaxPasses) * tiles * 256;
}

void reserve_scan_sort(int n, ScanScratch* sc) {
    DevBuf& sort_tmp = sc ? sc->sort_tmp : g_ctx.sort_tmp;
    DevBuf& scan_tmp = sc ? sc->scan_tmp : g_ctx.scan_tmp;
    sort_tmp.get<int>(os_scratch_ints(n));
    scan_tmp.get<int>(size_t(div_up(std::max(n, 1), kScanTile)) + 1);
}

void radix_sort_pairs(uint64_t* keys, int* vals, uint64_t* keys_alt, int* vals_alt, int n,
                      int bit_lo, int bit_hi, cudaStream_t s, ScanScratch* sc) {
    if (n <= 1) return;
    if (n > int(kOsValue)) throw Error(GF_ERR_CAPACITY, "radix sort of more than 2^30 - 1 keys");
    const int npass = div_up(bit_hi - bit_lo, 8);
    if (npass < 1 || npass > kOsMaxPasses) throw Error(GF_ERR_ARG, "radix sort bit range");
    const int tiles = div_up(n, kOsTile);
    int* hist = (sc ? sc->sort_tmp : g_ctx.sort_tmp).get<int>(os_scratch_ints(n));
    int* tickets = hist + kOsMaxPasses * 256;
    unsigned* status = reinterpret_cast<unsigned*>(tickets + 64);
    const size_t zero = size_t(kOsMaxPasses) * 256 + 64 + size_t(npass) * tiles * 256;
    GF_CUDA(cudaMemsetAsync(hist, 0, sizeof(int) * zero, s));
    const int hblocks = std::min(div_up(n, kRsThreads * 8), 2 * g_ctx.sms);
    k_os_hist<<<hblocks, kRsThreads, 0, s>>>(keys, n, bit_lo, npass, hist);
    GF_CHECK_LAUNCH();
    uint64_t *ka = keys, *kb = keys_alt;
    int *va = vals, *vb = vals_alt;
    for (int p = 0; p < npass; ++p) {
        k_os_pass<<<tiles, kRsThreads, 0, s>>>(ka, va, kb, vb, n, bit_lo + 8 * p, hist + 256 * p,
                                               status + size_t(p) * tiles * 256, tickets + p, g_ctx.d_status);
        GF_CHECK_LAUNCH();
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    if (npass & 1) {
        GF_CUDA(cudaMemcpyAsync(keys, ka, sizeof(uint64_t) * n, cudaMemcpyDeviceToDevice, s));
        GF_CUDA(cudaMemcpyAsync(vals, va, sizeof(int) * n, cudaMemcpyDeviceToDevice, s));
    }
}

// ---------------------------------------------------------------------------------------
// FP32 CUDA-core calibration: 8 independent FFMA chains per thread, all SMs busy.

__global__ void k_ffma_peak(float* out, int iters, float a, float b) {
    float x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-3f + k;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fmaf(x[k], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    if (s == 12345.678f) out[0] = s;  // keeps the chains alive
}

double fp32_peak_tflops() {
    Context& c = g_ctx;
    float* out = c.scan_tmp.get<float>(1);
    const int blocks = c.sms * 8, threads = 256, iters = 4096;
    cudaEvent_t e0, e1;
    GF_CUDA(cudaEventCreate(&e0));
    GF_CUDA(cudaEventCreate(&e1));
    k_ffma_peak<<<blocks, threads, 0, c.stream>>>(out, iters, 0.9999f, 1e-4f);  // warm-up
    GF_CHECK_LAUNCH();
    double best = 0;
    for (int rep = 0; rep < 5; ++rep) {
        GF_CUDA(cudaEventRecord(e0, c.stream));
        k_ffma_peak<<<blocks, threads, 0, c.stream>>>(out, iters, 0.9999f, 1e-4f);
        GF_CHECK_LAUNCH();
        GF_CUDA(cudaEventRecord(e1, c.stream));
        GF_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        GF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        const double flops = 2.0 * 8 * double(iters) * blocks * threads;
        best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return best;
}

}  // namespace gf
