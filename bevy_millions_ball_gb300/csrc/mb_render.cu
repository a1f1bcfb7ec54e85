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

#include <cmath>

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

// ---------------------------------------------------------------- perspective view
// The reference's own camera (src/main.rs:65-79: Camera3d at (0, 64, 64) looking
// at the origin, Bevy's default perspective with a 45-degree vertical field of
// view, clear colour sRGB (248, 151, 184)) or any eye and target, +y up.  Per
// pixel the nearest sphere along the pixel's ray (64-bit atomicMin of distance
// bits and sphere index) is marched and its normal taken exactly as in the
// top-down view, with the ray of the pixel instead of a vertical one; the march
// steps along the ray away from the eye (the shader's world_position_hit -=
// sdf * ray_direction, ray_direction pointing at the eye).  Lighting stands in
// for Bevy's PBR pass: the reference's directional light (src/main.rs:83-89,
// rotation Euler ZYX (0, -0.15 pi, -0.15 pi), shining along its -z), a GGX
// specular lobe with the material's perceptual roughness 0.435 and a dielectric
// F0 of 0.04, an ambient term, sRGB encoding.  The box interior (the
// reference's background cube, src/main.rs:104-114) shows where no sphere
// does: the far side of the box along the ray, base colour (0.8, 0.7, 0.6).
struct Cam {
    float ex, ey, ez;  // eye
    float gx, gy, gz;  // target
    float th, ta;      // tan(fov / 2), and times width / height
    float lx, ly, lz;  // unit vector towards the light
    float hs, top;     // the box: |x|, |z| <= hs, 0 <= y <= top
    uint32_t w, h;
};
struct Basis {
    float fx, fy, fz, rx, ry, rz, ux, uy, uz;
};
// forward = normalize(target - eye), right = normalize(cross(forward, +y)),
// up = cross(right, forward)
__device__ __forceinline__ Basis basis(const Cam& C) {
    Basis B;
    float fx = C.gx - C.ex, fy = C.gy - C.ey, fz = C.gz - C.ez;
    float l = len3(fx, fy, fz);
    B.fx = fx / l;
    B.fy = fy / l;
    B.fz = fz / l;
    float rx = -B.fz, rz = B.fx;  // cross(f, (0, 1, 0)) = (-fz, 0, fx)
    l = sqrtf(rx * rx + rz * rz);
    B.rx = rx / l;
    B.ry = 0.0f;
    B.rz = rz / l;
    B.ux = B.ry * B.fz - B.rz * B.fy;
    B.uy = B.rz * B.fx - B.rx * B.fz;
    B.uz = B.rx * B.fy - B.ry * B.fx;
    return B;
}
__device__ __forceinline__ void pixel_ray(const Cam& C, const Basis& B, uint32_t u, uint32_t v, float& dx,
                                          float& dy, float& dz) {
    const float sx = (2.0f * ((float)u + 0.5f) / (float)C.w - 1.0f) * C.ta;
    const float sy = (1.0f - 2.0f * ((float)v + 0.5f) / (float)C.h) * C.th;
    const float x = B.fx + sx * B.rx + sy * B.ux, y = B.fy + sx * B.ry + sy * B.uy, z = B.fz + sx * B.rz + sy * B.uz;
    const float l = len3(x, y, z);
    dx = x / l;
    dy = y / l;
    dz = z / l;
}
// distance along the unit ray (e, d) to the sphere's near surface; <= 0 or NaN: none
__device__ __forceinline__ float ray_sphere(const Cam& C, float dx, float dy, float dz, float4 s) {
    const float ox = C.ex - s.x, oy = C.ey - s.y, oz = C.ez - s.z;
    const float b = ox * dx + oy * dy + oz * dz;
    const float c = (ox * ox + oy * oy + oz * oz) - s.w * s.w;
    const float disc = b * b - c;
    if (!(disc >= 0.0f)) return -1.0f;
    return -b - sqrtf(disc);
}
constexpr unsigned long long kFar = ~0ull;

__global__ void __launch_bounds__(256)
    k_splat_view(const float4* __restrict__ pos, uint32_t n, Cam C, unsigned long long* __restrict__ zbuf) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 s = grown(__ldg(pos + i));
    if (!(s.w > 0.0f)) return;
    const Basis B = basis(C);
    const float px = s.x - C.ex, py = s.y - C.ey, pz = s.z - C.ez;
    const float cx = px * B.rx + py * B.ry + pz * B.rz, cy = px * B.ux + py * B.uy + pz * B.uz,
                cz = px * B.fx + py * B.fy + pz * B.fz;
    if (!(cz - s.w > 1e-3f)) return;  // the sphere must lie wholly in front of the eye
    // screen box of the view-space cube around the sphere (x / z over its corners),
    // one pixel wider on every side
    const float zn = cz - s.w, zf = cz + s.w;
    const float xl = cx - s.w, xh = cx + s.w, yl = cy - s.w, yh = cy + s.w;
    const float sxl = xl / (xl >= 0.0f ? zf : zn), sxh = xh / (xh >= 0.0f ? zn : zf);
    const float syl = yl / (yl >= 0.0f ? zf : zn), syh = yh / (yh >= 0.0f ? zn : zf);
    const float ua = (sxl / C.ta + 1.0f) * 0.5f * (float)C.w - 1.5f, ub = (sxh / C.ta + 1.0f) * 0.5f * (float)C.w + 0.5f;
    const float va = (1.0f - syh / C.th) * 0.5f * (float)C.h - 1.5f, vb = (1.0f - syl / C.th) * 0.5f * (float)C.h + 0.5f;
    if (!(ub >= 0.0f && vb >= 0.0f && ua < (float)C.w && va < (float)C.h)) return;
    const int u0 = (int)fmaxf(ceilf(ua), 0.0f), u1 = (int)fminf(floorf(ub), (float)C.w - 1.0f);
    const int v0 = (int)fmaxf(ceilf(va), 0.0f), v1 = (int)fminf(floorf(vb), (float)C.h - 1.0f);
    for (int v = v0; v <= v1; ++v) {
        for (int u = u0; u <= u1; ++u) {
            float dx, dy, dz;
            pixel_ray(C, B, (uint32_t)u, (uint32_t)v, dx, dy, dz);
            const float t = ray_sphere(C, dx, dy, dz, s);
            if (!(t > 0.0f)) continue;
            const unsigned long long key = ((unsigned long long)__float_as_uint(t) << 32) | (unsigned long long)(i + 1u);
            atomicMin(zbuf + (size_t)v * C.w + u, key);
        }
    }
}

__device__ __forceinline__ float srgb8(float x) {  // linear [0, 1] -> sRGB, 0..255
    x = fminf(fmaxf(x, 0.0f), 1.0f);
    const float e = x <= 0.0031308f ? 12.92f * x : 1.055f * powf(x, 1.0f / 2.4f) - 0.055f;
    return fminf(255.0f * e + 0.5f, 255.0f);
}
__device__ __forceinline__ uint32_t rgba8(float r, float g, float b) {
    return 0xFF000000u | (uint32_t)srgb8(r) | ((uint32_t)srgb8(g) << 8) | ((uint32_t)srgb8(b) << 16);
}
constexpr float kAmbient = 0.2f, kAlpha = 0.435f * 0.435f, kF0 = 0.04f, kPi = 3.14159265f;

__global__ void __launch_bounds__(256)
    k_shade_view(const float4* __restrict__ pos, Cam C, const unsigned long long* __restrict__ zbuf,
                 uint32_t* __restrict__ rgba, float* __restrict__ depth) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= C.w * C.h) return;
    const uint32_t u = p % C.w, v = p / C.w;
    const Basis B = basis(C);
    float dx, dy, dz;
    pixel_ray(C, B, u, v, dx, dy, dz);
    const unsigned long long key = zbuf[p];
    if (key != kFar) {
        const float4 s = grown(__ldg(pos + ((uint32_t)(key & 0xFFFFFFFFull) - 1u)));
        const float t = __uint_as_float((uint32_t)(key >> 32));
        float hx = C.ex + t * dx, hy = C.ey + t * dy, hz = C.ez + t * dz;
        float nx = hx - s.x, ny = hy - s.y, nz = hz - s.z;  // normal_sphere (sdf.wgsl:107-109)
        const float nl = len3(nx, ny, nz);
        nx /= nl;
        ny /= nl;
        nz /= nl;
        float sd_sphere = 0.0f, sd_plane = -hy, walked = 0.0f;
        bool hit = false;
        for (int it = 0; it < 16; ++it) {  // deferred_physics_ball.wgsl:80-92
            const float d = smooth_max(sd_sphere, sd_plane, kK);
            hx += d * dx;
            hy += d * dy;
            hz += d * dz;
            walked += d;
            if (d < 0.001f) {
                hit = true;
                break;
            }
            sd_sphere = len3(hx - s.x, hy - s.y, hz - s.z) - s.w;
            sd_plane = -hy;
        }
        if (hit) {
            const float hh = (sd_plane - sd_sphere) / kK;  // gradient_smooth_max (sdf.wgsl:20-27)
            const float pa = 1.0f / (1.0f + exp2f(hh)), pb = 1.0f / (1.0f + exp2f(-hh));
            float gx = pa * nx, gy = pa * ny - pb, gz = pa * nz;
            const float gl = len3(gx, gy, gz);
            if (gl > 0.0f) {
                gx /= gl;
                gy /= gl;
                gz /= gl;
            }
            // GGX lobe (Trowbridge-Reitz distribution, height-correlated Smith
            // visibility, Schlick Fresnel) and Lambert diffuse for one light
            const float vx = -dx, vy = -dy, vz = -dz;
            const float nl_ = fmaxf(gx * C.lx + gy * C.ly + gz * C.lz, 0.0f);
            const float nv = fmaxf(gx * vx + gy * vy + gz * vz, 1e-4f);
            float ax = vx + C.lx, ay = vy + C.ly, az = vz + C.lz;
            const float al = len3(ax, ay, az);
            float spec = 0.0f;
            if (al > 0.0f && nl_ > 0.0f) {
                ax /= al;
                ay /= al;
                az /= al;
                const float nh = fmaxf(gx * ax + gy * ay + gz * az, 0.0f), vh = fmaxf(vx * ax + vy * ay + vz * az, 0.0f);
                const float a2 = kAlpha * kAlpha, dd = nh * nh * (a2 - 1.0f) + 1.0f;
                const float D = a2 / (kPi * dd * dd);
                const float vis = 0.5f / (nl_ * sqrtf(nv * nv * (1.0f - a2) + a2) + nv * sqrtf(nl_ * nl_ * (1.0f - a2) + a2));
                const float m = 1.0f - vh, m2 = m * m;
                const float F = kF0 + (1.0f - kF0) * (m2 * m2 * m);
                spec = D * vis * F * nl_;
            }
            const float lit = kAmbient + nl_;
            rgba[p] = rgba8(1.0f * lit + spec, (191.0f / 255.0f) * lit + spec, spec);
            if (depth) depth[p] = t + walked;
            return;
        }
    }
    // the far side of the box along the ray (the background cube seen from outside
    // or inside), else the clear colour
    float tn = 0.0f, tf = 3.0e38f;
    int axis = -1;
    const float lo[3] = {-C.hs, 0.0f, -C.hs}, hi[3] = {C.hs, C.top, C.hs}, e[3] = {C.ex, C.ey, C.ez},
                d[3] = {dx, dy, dz};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (d[k] != 0.0f) {
            float t0 = (lo[k] - e[k]) / d[k], t1 = (hi[k] - e[k]) / d[k];
            if (t0 > t1) {
                const float x = t0;
                t0 = t1;
                t1 = x;
            }
            tn = fmaxf(tn, t0);
            if (t1 < tf) {
                tf = t1;
                axis = k;
            }
        } else if (e[k] < lo[k] || e[k] > hi[k]) {
            tn = 3.0e38f;
        }
    }
    if (axis >= 0 && tf > tn) {
        // inward normal of the exit face: against the ray along that axis
        const float bx = axis == 0 ? (dx > 0.0f ? -1.0f : 1.0f) : 0.0f;
        const float by = axis == 1 ? (dy > 0.0f ? -1.0f : 1.0f) : 0.0f;
        const float bz = axis == 2 ? (dz > 0.0f ? -1.0f : 1.0f) : 0.0f;
        const float lit = kAmbient + fmaxf(bx * C.lx + by * C.ly + bz * C.lz, 0.0f);
        rgba[p] = rgba8(0.8f * lit, 0.7f * lit, 0.6f * lit);
        if (depth) depth[p] = tf;
        return;
    }
    rgba[p] = 0xFF000000u | 248u | (151u << 8) | (184u << 16);
    if (depth) depth[p] = 0.0f;
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

namespace mb {
void reference_view(float eye[3], float target[3], float* fov_degrees, float to_light[3]) {
    eye[0] = 0.0f;
    eye[1] = 64.0f;
    eye[2] = 64.0f;
    target[0] = target[1] = target[2] = 0.0f;
    *fov_degrees = 45.0f;
    const double pi = 3.14159265358979323846, b = -0.15 * pi, c = -0.15 * pi;
    // R_y(b) R_x(c) (0, 0, -1): the direction the light travels
    const double x = -std::cos(c) * std::sin(b), y = std::sin(c), z = -std::cos(c) * std::cos(b);
    to_light[0] = (float)-x;
    to_light[1] = (float)-y;
    to_light[2] = (float)-z;
}

cudaError_t render_view(const float4* pos, uint32_t n, uint32_t w, uint32_t h, const float eye[3],
                        const float target[3], float tan_half_fov, const float to_light[3], float half_map_size,
                        float map_top, unsigned long long* zbuf, uint32_t* rgba, float* depth, cudaStream_t st) {
    if (!w || !h) return cudaSuccess;
    Cam C{eye[0], eye[1], eye[2], target[0], target[1], target[2], tan_half_fov,
          tan_half_fov * ((float)w / (float)h), to_light[0], to_light[1], to_light[2], half_map_size, map_top, w, h};
    cudaError_t e = cudaMemsetAsync(zbuf, 0xFF, sizeof(unsigned long long) * w * h, st);
    if (e) return e;
    if (n) {
        k_splat_view<<<(n + 255u) / 256u, 256, 0, st>>>(pos, n, C, zbuf);
        if ((e = cudaGetLastError())) return e;
    }
    k_shade_view<<<(w * h + 255u) / 256u, 256, 0, st>>>(pos, C, zbuf, rgba, depth);
    return cudaGetLastError();
}
}  // namespace mb
