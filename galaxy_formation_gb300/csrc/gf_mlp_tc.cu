// gf_mlp_tc.cu — inference of the smoothing-length MLP with its layer-2 contraction on the
// 5th-generation tensor cores (tcgen05, sm_103a).
//
// One CTA of 128 threads per tile of 128 samples (thread t = sample row t):
//   1. layer 1 (4 -> 64, float32 from the bfloat16 weights) per thread; the ReLU activations
//      are rounded to bfloat16 and stored as row t of the A tile (128 x 64) in shared memory;
//   2. one thread issues D[128 x 64] = A x W2^T as four tcgen05.mma (K = 16 each, bfloat16
//      inputs, float32 accumulation in tensor memory) and commits them to an mbarrier;
//   3. after the (bounded) wait, warp w reads TMEM lanes 32w .. 32w + 31 (its 32 rows, all
//      64 columns) with tcgen05.ld and finishes layer 2 (+ b2, ReLU) and layer 3 per row.
// W2 (bfloat16, row j = output unit j, K-major) is staged once per CTA. Operands use the
// canonical K-major layout without swizzle: 8-row x 16-byte core matrices, core matrix
// (row group g, k group c) at byte offset (8 g + c) * 128, so the leading-dimension (K)
// stride between core matrices is 128 bytes and the stride between row groups 1024 bytes.
//
// Every wait is bounded: a CTA whose MMA does not complete raises GF_ERR_TIMEOUT in the status
// word, waits once more (bounded) for the MMA in flight, frees its tensor memory and stops.
#include <cuda_bf16.h>

#include <algorithm>

#include "gf_mlp.cuh"

namespace gf {

namespace {

constexpr int H = kMlpHidden;
constexpr int kTcM = 128, kTcN = 64;
constexpr int kTcThreads = 128;
constexpr int kTmemCols = 64;  // float32 accumulator: 64 columns of 128 lanes
constexpr long kSpinMax = 1l << 20;
// dynamic shared memory per CTA: at most 7 CTAs fit on an SM, so their tensor memory
// (7 x 64 of the 512 columns) never has to wait for an allocation
constexpr size_t kTcSmemBytes = 32 * 1024;

// instruction descriptor (kind::f16): D float32 (bits 4-5 = 1), A and B bfloat16 (bits 7-9 and
// 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(kTcN >> 3) << 17) |
                            (uint32_t(kTcM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ int cm_offset(int r, int k) {  // bytes, K = 64 (8 k groups)
    return ((((r >> 3) << 3) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1);
}

// shared-memory matrix descriptor: start address, leading / stride byte offsets (all >> 4),
// descriptor version 1 (bits 46-47), base offset 0, no swizzle (bits 61-63 = 0)
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return uint64_t((addr >> 4) & 0x3FFFu) | (uint64_t((lbo >> 4) & 0x3FFFu) << 16) |
           (uint64_t((sbo >> 4) & 0x3FFFu) << 32) | (uint64_t(1) << 46);
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(phase)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t phase) {
    for (long it = 0; it < kSpinMax; ++it)
        if (mbar_try_wait(bar, phase)) return true;
    return false;
}

struct TcSmem {
    uint8_t a[kTcM * H * 2];  // A tile, bfloat16, canonical layout (16 KB)
    uint8_t b[kTcN * H * 2];  // W2, bfloat16, canonical layout (8 KB)
    float w1[H * 4], b1[H], b2[H], w3[H], b3;
    unsigned long long bar;
    uint32_t tmem;
    int fail;
};

__global__ void __launch_bounds__(kTcThreads) k_mlp_forward_tc(int n, const float* __restrict__ X, MlpNorm nm,
                                                               const __nv_bfloat16* __restrict__ P,
                                                               float* __restrict__ Y, uint32_t* status) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    // operands on a 1024-byte boundary (the launch adds 1024 bytes of slack)
    const uint32_t mis = smem_u32(smem_raw) & 1023u;
    TcSmem& S = *reinterpret_cast<TcSmem*>(smem_raw + ((1024u - mis) & 1023u));
    const int t = threadIdx.x, warp = t >> 5;
    for (int i = t; i < H * H; i += kTcThreads) {
        const int j = i / H, k = i % H;
        *reinterpret_cast<__nv_bfloat16*>(S.b + cm_offset(j, k)) = P[kOffW2 + i];
    }
    for (int i = t; i < H * 4; i += kTcThreads) S.w1[i] = __bfloat162float(P[kOffW1 + i]);
    for (int i = t; i < H; i += kTcThreads) {
        S.b1[i] = __bfloat162float(P[kOffB1 + i]);
        S.b2[i] = __bfloat162float(P[kOffB2 + i]);
        S.w3[i] = __bfloat162float(P[kOffW3 + i]);
    }
    const uint32_t bar = smem_u32(&S.bar);
    if (t == 0) {
        S.b3 = __bfloat162float(P[kOffB3]);
        S.fail = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(&S.tmem)), "r"(kTmemCols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // W2 visible to the tensor cores
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = S.tmem;
    const uint32_t a_addr = smem_u32(S.a), b_addr = smem_u32(S.b);
    uint32_t phase = 0;

    for (int tile = blockIdx.x; tile * kTcM < n; tile += gridDim.x) {
        const int i = tile * kTcM + t;
        // layer 1 for row t, bfloat16 activations into the A tile
        float xn[4] = {0.f, 0.f, 0.f, 0.f};
        if (i < n)
#pragma unroll
            for (int q = 0; q < 4; ++q) xn[q] = (X[4 * size_t(i) + q] - nm.mean[q]) * nm.inv_std[q];
#pragma unroll 8
        for (int k = 0; k < H; k += 2) {
            float v[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                float z = S.b1[k + u];
#pragma unroll
                for (int q = 0; q < 4; ++q) z = fmaf(S.w1[(k + u) * 4 + q], xn[q], z);
                v[u] = i < n ? fmaxf(z, 0.f) : 0.f;
            }
            *reinterpret_cast<__nv_bfloat162*>(S.a + cm_offset(t, k)) = __floats2bfloat162_rn(v[0], v[1]);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        if (t == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int s = 0; s < H / 16; ++s) {
                const uint64_t ad = smem_desc(a_addr + s * 256, 128, 1024);
                const uint64_t bd = smem_desc(b_addr + s * 256, 128, 1024);
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                    ::"r"(tmem), "l"(ad), "l"(bd), "r"(kIdesc), "r"(s) : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         ::"r"(bar) : "memory");
        }
        const bool done = mbar_wait_bounded(bar, phase);
        if (__syncthreads_or(!done)) {
            if (t == 0) {
                S.fail = 1;
                if (status) atomicOr(status, uint32_t(GF_ERR_TIMEOUT));
            }
            mbar_wait_bounded(bar, phase);  // let an MMA in flight finish before the memory goes
            break;
        }
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // rows 32 warp .. 32 warp + 31: lane t & 31 of the warp holds row t
        float y = S.b3;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            uint32_t r[32];
            const uint32_t taddr = tmem + (uint32_t(32 * warp) << 16) + uint32_t(32 * half);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, "
                "[%32];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                  "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                  "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                : "r"(taddr)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                const int j = 32 * half + c;
                y = fmaf(S.w3[j], fmaxf(__uint_as_float(r[c]) + S.b2[j], 0.f), y);
            }
        }
        if (i < n) Y[i] = y * nm.t_std + nm.t_mean;
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();  // A tile and accumulator free for the next tile
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

}  // namespace

// Launches the tensor-core forward; the dynamic shared memory is the 1024-aligned TcSmem.
void mlp_forward_tc(int n, const float* X, const MlpNorm& nm, const __nv_bfloat16* P, float* Y, cudaStream_t s) {
    if (n <= 0) return;
    static_assert(sizeof(TcSmem) + 1024 <= kTcSmemBytes, "shared memory of the tensor-core MLP");
    const size_t sm = kTcSmemBytes;
    static bool attr = false;
    if (!attr) {
        GF_CUDA(cudaFuncSetAttribute(k_mlp_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm)));
        attr = true;
    }
    const int tiles = div_up(n, kTcM);
    const int grid = std::min(tiles, 4 * ctx().sms);
    k_mlp_forward_tc<<<grid, kTcThreads, sm, s>>>(n, X, nm, P, Y, ctx().d_status);
    GF_CHECK_LAUNCH();
}

}  // namespace gf
