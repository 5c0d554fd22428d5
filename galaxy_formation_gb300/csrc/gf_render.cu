// gf_render.cu — particle splat and tone map (cpp/nbody.cpp:443-503) as CUDA kernels.
// No graphics API: images are plain device buffers.
//   splat:   one thread per particle, orthographic projection, bilinear deposit with
//            float atomics (cpp/nbody.cpp:445-469);
//   tonemap: one thread per pixel: log compression + bilinear glow + soft saturation to
//            8-bit RGB (cpp/nbody.cpp:474-503).
#include "gf_sph.cuh"

namespace gf {

namespace {

__global__ void k_splat(int n, const double* __restrict__ pos, const uint8_t* __restrict__ group, int ngroups,
                        const double* __restrict__ rot, const double* __restrict__ center, double scale,
                        int W, int H, float* __restrict__ img, uint32_t* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (group[i] >= ngroups) {  // no image plane for this group: skipped, reported
        raise_status(status, GF_ERR_ARG);
        return;
    }
    const size_t plane = size_t(W) * H;
    const double x = pos[3 * size_t(i)] - center[0], y = pos[3 * size_t(i) + 1] - center[1],
                 z = pos[3 * size_t(i) + 2] - center[2];
    const double u = 0.5 * W + scale * (rot[0] * x + rot[1] * y + rot[2] * z) - 0.5;
    const double v = 0.5 * H - scale * (rot[3] * x + rot[4] * y + rot[5] * z) - 0.5;
    if (!(u >= 0 && v >= 0 && u < W - 1 && v < H - 1)) return;
    const int iu = int(u), iv = int(v);
    const float fu = float(u - iu), fv = float(v - iv);
    float* p = img + group[i] * plane + size_t(iv) * W + iu;
    atomicAdd(p, (1 - fu) * (1 - fv));
    atomicAdd(p + 1, fu * (1 - fv));
    atomicAdd(p + W, (1 - fu) * fv);
    atomicAdd(p + W + 1, fu * fv);
}

__global__ void k_tonemap(int W, int H, int ngroups, const float* __restrict__ img,
                          const float* __restrict__ glow, int gw, int gh, const float* __restrict__ colors,
                          float inv_ref, float K, float exposure, uint8_t* __restrict__ out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= W || y >= H) return;
    const size_t plane = size_t(W) * H, gplane = size_t(gw) * gh;
    const float inv_logK = 1.0f / log1pf(K);
    const float sx = float(gw) / W, sy = float(gh) / H;
    const float gyf = fminf(fmaxf((y + 0.5f) * sy - 0.5f, 0.0f), gh - 1.001f);
    const int gy = int(gyf);
    const float fy = gyf - gy;
    const float gxf = fminf(fmaxf((x + 0.5f) * sx - 0.5f, 0.0f), gw - 1.001f);
    const int gx = int(gxf);
    const float fx = gxf - gx;
    float r = 0, g = 0, b = 0;
    for (int k = 0; k < ngroups; ++k) {
        float l = log1pf(K * inv_ref * img[k * plane + size_t(y) * W + x]) * inv_logK;
        const float* q = glow + k * gplane + size_t(gy) * gw + gx;
        l += (1 - fy) * ((1 - fx) * q[0] + fx * q[1]) + fy * ((1 - fx) * q[gw] + fx * q[gw + 1]);
        r += l * colors[3 * k];
        g += l * colors[3 * k + 1];
        b += l * colors[3 * k + 2];
    }
    uint8_t* o = out + 3 * (size_t(y) * W + x);
    o[0] = uint8_t(255.0f * (1 - expf(-exposure * r)) + 0.5f);
    o[1] = uint8_t(255.0f * (1 - expf(-exposure * g)) + 0.5f);
    o[2] = uint8_t(255.0f * (1 - expf(-exposure * b)) + 0.5f);
}

}  // namespace

void render_splat(int n, const double* pos, const uint8_t* group, int ngroups, const double* rot,
                  const double* center, double scale, int W, int H, float* img, cudaStream_t s) {
    GF_CUDA(cudaMemsetAsync(img, 0, sizeof(float) * size_t(ngroups) * W * H, s));
    if (n <= 0) return;
    k_splat<<<div_up(n, 256), 256, 0, s>>>(n, pos, group, ngroups, rot, center, scale, W, H, img, ctx().d_status);
    GF_CHECK_LAUNCH();
}

void render_tonemap(int W, int H, int ngroups, const float* img, const float* glow, int gw, int gh,
                    const float* colors, float inv_ref, float K, float exposure, uint8_t* out,
                    cudaStream_t s) {
    if (W <= 0 || H <= 0) return;
    k_tonemap<<<dim3(div_up(W, 128), H), 128, 0, s>>>(W, H, ngroups, img, glow, gw, gh, colors, inv_ref,
                                                      K, exposure, out);
    GF_CHECK_LAUNCH();
}

}  // namespace gf
