// mb_render.cu — headless sphere-impostor renderer into a device image.
//
// The reference draws every sphere as an instanced impostor whose fragment
// shader (src/custom_materials/physics_ball/deferred_physics_ball.wgsl:26-107,
// with src/custom_materials/sdf.wgsl) intersects the view ray with the sphere
// (radius grown near the floor by `temporary_solution`, 28-33), then
// ray-marches 16 steps on the smooth maximum (K = 0.08) of the sphere's and the
// floor plane's signed distances so that spheres melt into the floor, and takes
// the normal from the gradient of that smooth maximum.  Here the same per-pixel
// arithmetic runs for an orthographic camera looking straight down (-y) at an
// x/z window, in two kernels:
//   1. k_splat: one thread per sphere rasterises the sphere's disc; each covered
//      pixel keeps the highest surface point (64-bit atomicMax of height bits and
//      sphere index, so ties resolve to the larger index);
//   2. k_shade: one thread per pixel runs the shader's march and normal for its
//      winning sphere and writes RGBA8 (base colour 255,191,0 lit by one
//      directional light; the reference's PBR lighting belongs to Bevy's
//      renderer) and the surface height (0 and a floor colour where no sphere
//      is visible or the march leaves the sphere).

#include <cuda_runtime.h>

#include "mb_internal.h"

namespace mb {
namespace {

constexpr float kK = 0.08f;             // smooth-max blend (deferred_physics_ball.wgsl:63)
constexpr uint64_t kEmpty = 0ull;       // no sphere: height bits 0 with index 0 loses to any hit above 0

struct View {
    float x0, z0, sx, sz;  // pixel (u, v) centre = (x0 + (u + 0.5) sx, z0 + (v + 0.5) sz)
    uint32_t w, h;
};

// temporary_solution (deferred_physics_ball.wgsl:28-33)
__device__ __forceinline__ float4 grown(float4 s) {
    const float x = fminf(fmaxf(s.y / s.w, 0.0f), 1.0f);
    const float y = 0.26f * (x - 1.0f) * (x - 1.0f) + 1.0f;
    return make_float4(s.x, s.y, s.z, s.w * y);
}

__global__ void __launch_bounds__(256)
    k_splat(const float4* __restrict__ pos, uint32_t n, View V, unsigned long long* __restrict__ zbuf) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 s = grown(__ldg(pos + i));
    if (!(s.w > 0.0f)) return;
    // pixels whose centre lies within the disc of radius s.w around (s.x, s.z)
    const float u0 = ceilf((s.x - s.w - V.x0) / V.sx - 0.5f), u1 = floorf((s.x + s.w - V.x0) / V.sx - 0.5f);
    const float v0 = ceilf((s.z - s.w - V.z0) / V.sz - 0.5f), v1 = floorf((s.z + s.w - V.z0) / V.sz - 0.5f);
    if (!(u1 >= 0.0f && v1 >= 0.0f && u0 < (float)V.w && v0 < (float)V.h)) return;
    const int ua = (int)fmaxf(u0, 0.0f), ub = (int)fminf(u1, (float)V.w - 1.0f);
    const int va = (int)fmaxf(v0, 0.0f), vb = (int)fminf(v1, (float)V.h - 1.0f);
    const float r2 = s.w * s.w;
    for (int v = va; v <= vb; ++v) {
        const float dz = V.z0 + ((float)v + 0.5f) * V.sz - s.z;
        for (int u = ua; u <= ub; ++u) {
            const float dx = V.x0 + ((float)u + 0.5f) * V.sx - s.x;
            const float c2 = r2 - (dx * dx + dz * dz);
            if (c2 < 0.0f) continue;
            float top = s.y + sqrtf(c2);
            top = top > 0.0f ? top : 0.0f;  // heights below the floor count as +0 (bits 0)
            const unsigned long long key =
                ((unsigned long long)__float_as_uint(top) << 32) | (unsigned long long)(i + 1u);
            atomicMax(zbuf + (size_t)v * V.w + u, key);
        }
    }
}

__device__ __forceinline__ float len3(float x, float y, float z) { return sqrtf(x * x + y * y + z * z); }

// smooth_max / gradient weights (sdf.wgsl:11-27)
__device__ __forceinline__ float smooth_max(float a, float b, float k) {
    const float ki = 1.0f / k;
    return k * log2f(exp2f(a * ki) + exp2f(b * ki));
}

__global__ void __launch_bounds__(256)
    k_shade(const float4* __restrict__ pos, View V, const unsigned long long* __restrict__ zbuf,
            uint32_t* __restrict__ rgba, float* __restrict__ height) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= V.w * V.h) return;
    const uint32_t u = p % V.w, v = p / V.w;
    const unsigned long long key = zbuf[p];
    const uint32_t floor_rgba = 0xFF4D4D4Du;  // grey floor, opaque
    if (key == kEmpty) {
        rgba[p] = floor_rgba;
        height[p] = 0.0f;
        return;
    }
    const uint32_t idx = (uint32_t)(key & 0xFFFFFFFFull) - 1u;
    const float4 s = grown(__ldg(pos + idx));
    // ray towards the eye (straight up); the fragment sits on the sphere's top surface
    float hx = V.x0 + ((float)u + 0.5f) * V.sx, hz = V.z0 + ((float)v + 0.5f) * V.sz;
    float hy = __uint_as_float((uint32_t)(key >> 32));
    // normal_sphere at the hit (sdf.wgsl:107-109)
    float nx = hx - s.x, ny = hy - s.y, nz = hz - s.z;
    const float nl = len3(nx, ny, nz);
    nx /= nl;
    ny /= nl;
    nz /= nl;
    // march on smooth_max(sphere, plane) (deferred_physics_ball.wgsl:80-92); plane
    // (0, -1, 0, 0): sdf = -y; the step moves against the ray, i.e. down
    float sd_sphere = 0.0f, sd_plane = -hy;
    bool hit = false;
    for (int it = 0; it < 16; ++it) {
        const float d = smooth_max(sd_sphere, sd_plane, kK);
        hy -= d;
        if (d < 0.001f) {
            hit = true;
            break;
        }
        sd_sphere = len3(hx - s.x, hy - s.y, hz - s.z) - s.w;
        sd_plane = -hy;
    }
    if (!hit) {
        rgba[p] = floor_rgba;
        height[p] = 0.0f;
        return;
    }
    // gradient_smooth_max(sd_sphere, sd_plane, K, n_sphere, (0, -1, 0)) (sdf.wgsl:20-27)
    const float hh = (sd_plane - sd_sphere) / kK;
    const float pa = 1.0f / (1.0f + exp2f(hh)), pb = 1.0f / (1.0f + exp2f(-hh));
    float gx = pa * nx, gy = pa * ny - pb, gz = pa * nz;
    const float gl = len3(gx, gy, gz);
    if (gl > 0.0f) {
        gx /= gl;
        gy /= gl;
        gz /= gl;
    }
    // one directional light from above: ambient 0.25 + diffuse 0.75
    const float lx = 0.3713907f, ly = 0.9284767f, lz = 0.0f;  // normalize(0.4, 1, 0)
    const float lit = 0.25f + 0.75f * fmaxf(gx * lx + gy * ly + gz * lz, 0.0f);
    const uint32_t r = (uint32_t)fminf(255.0f * lit + 0.5f, 255.0f);
    const uint32_t g = (uint32_t)fminf(191.0f * lit + 0.5f, 255.0f);
    rgba[p] = 0xFF000000u | (r) | (g << 8);  // blue 0
    height[p] = hy;
}

}  // namespace

cudaError_t render_topdown(const float4* pos, uint32_t n, uint32_t w, uint32_t h, float x0, float z0, float x1,
                           float z1, unsigned long long* zbuf, uint32_t* rgba, float* height, cudaStream_t st) {
    if (!w || !h) return cudaSuccess;
    View V{x0, z0, (x1 - x0) / (float)w, (z1 - z0) / (float)h, w, h};
    cudaError_t e = cudaMemsetAsync(zbuf, 0, sizeof(unsigned long long) * w * h, st);
    if (e) return e;
    if (n) {
        k_splat<<<(n + 255u) / 256u, 256, 0, st>>>(pos, n, V, zbuf);
        if ((e = cudaGetLastError())) return e;
    }
    k_shade<<<(w * h + 255u) / 256u, 256, 0, st>>>(pos, V, zbuf, rgba, height);
    return cudaGetLastError();
}

}  // namespace mb
