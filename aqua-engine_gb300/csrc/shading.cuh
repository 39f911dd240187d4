// shading.cuh — device helpers shared by the wavefront kernels and the
// batched persistent kernel: camera rays (`Perspective`,
// scenes/cbox.json:516-543), per-path random numbers, bilinear sRGB textures
// (`Image` colours, scenes/room.json:6) and light selection.
#pragma once

#include "device.cuh"

namespace aq {

__device__ __forceinline__ v3 f3(float4 a) { return mk(a.x, a.y, a.z); }

// Shirley-Chiu concentric square-to-disk mapping.
__device__ __forceinline__ void concentric(float u, float v, float& x, float& y) {
    float a = 2.0f * u - 1.0f, b = 2.0f * v - 1.0f;
    if (a == 0.0f && b == 0.0f) { x = y = 0.0f; return; }
    float r, phi;
    if (fabsf(a) > fabsf(b)) { r = a; phi = (kPi / 4.0f) * (b / a); }
    else { r = b; phi = (kPi / 2.0f) - (kPi / 4.0f) * (a / b); }
    x = r * cosf(phi);
    y = r * sinf(phi);
}

__device__ __forceinline__ void camera_ray(const DevCamera& c, uint32_t pixel, float u0, float u1, float u2,
                                           float u3, v3& o, v3& d) {
    uint32_t px = pixel % (uint32_t)c.width, py = pixel / (uint32_t)c.width;
    float sx = (2.0f * (((float)px + u0) / (float)c.width) - 1.0f) * c.tan_half * c.aspect;
    float sy = (1.0f - 2.0f * (((float)py + u1) / (float)c.height)) * c.tan_half;
    v3 dc = mk(sx, sy, -1.0f), oc = mk(0, 0, 0);
    if (c.lens_radius > 0.0f) {
        float lx, ly;
        concentric(u2, u3, lx, ly);
        oc = mk(lx * c.lens_radius, ly * c.lens_radius, 0.0f);
        dc = dc * c.focal - oc;
    }
    v3 R = mk(c.right[0], c.right[1], c.right[2]), U = mk(c.up[0], c.up[1], c.up[2]),
       B = mk(c.back[0], c.back[1], c.back[2]);
    o = mk(c.pos[0], c.pos[1], c.pos[2]) + R * oc.x + U * oc.y + B * oc.z;
    d = normalize(R * dc.x + U * dc.y + B * dc.z);
}

__device__ __forceinline__ float draw(uint64_t& st, uint64_t inc) { return u01(pcg32_next(st, inc)); }

__device__ __forceinline__ float srgb_lut_lookup(const float* lut, uint32_t c) { return lut[c & 255u]; }

__device__ __forceinline__ v3 texel(const DevScene& S, const DevTexture& T, int x, int y, const float* lut) {
    x %= T.w; if (x < 0) x += T.w;
    y %= T.h; if (y < 0) y += T.h;
    uint32_t p = ldg_(S.texels + T.offset + (size_t)y * (size_t)T.w + (size_t)x);
    return mk(srgb_lut_lookup(lut, p), srgb_lut_lookup(lut, p >> 8), srgb_lut_lookup(lut, p >> 16));
}

// Bilinear lookup with wrap addressing; texels are decoded to linear first.
__device__ __forceinline__ v3 tex_bilinear(const DevScene& S, int ti, float u, float v, const float* lut) {
    DevTexture T = S.texs[ti];
    float x = u * (float)T.w - 0.5f, y = v * (float)T.h - 0.5f;
    float fx = floorf(x), fy = floorf(y);
    float ax = x - fx, ay = y - fy;
    int ix = (int)fx, iy = (int)fy;
    v3 c00 = texel(S, T, ix, iy, lut), c10 = texel(S, T, ix + 1, iy, lut);
    v3 c01 = texel(S, T, ix, iy + 1, lut), c11 = texel(S, T, ix + 1, iy + 1, lut);
    v3 a = c00 + (c10 - c00) * ax, b = c01 + (c11 - c01) * ax;
    return a + (b - a) * ay;
}

// Shading normal at hit (tri, u, v): the interpolated vertex normal, turned
// to the side of ng (which faces wo), when wo lies above it; otherwise ng.
// Flat scenes (no normals) return ng itself.
__device__ __forceinline__ v3 shading_normal(const DevScene& S, int32_t tri, float u, float v, v3 ng, v3 wo) {
    if (!S.nrm) return ng;
    const float4* np = S.nrm + 3 * (size_t)tri;
    float4 a = ldg_(np), b = ldg_(np + 1), c = ldg_(np + 2);
    v3 n = f3(a) * (1.0f - u - v) + f3(b) * u + f3(c) * v;
    float l2 = dot(n, n);
    if (!(l2 > 0.0f)) return ng;
    n = n * (1.0f / sqrtf(l2));
    if (dot(n, ng) < 0.0f) n = -n;
    return dot(n, wo) > 0.0f ? n : ng;
}

__device__ __forceinline__ int pick_light(const DevScene& S, float u) {
    int lo = 0, hi = S.n_lights - 1;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (u < S.lights[mid].le.w) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}


// sRGB decode table (IEC 61966-2-1), filled per block in shared memory.
__device__ __forceinline__ void fill_srgb_lut(float* lut) {
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        float c = (float)i / 255.0f;
        lut[i] = c <= 0.04045f ? c / 12.92f : powf((c + 0.055f) / 1.055f, 2.4f);
    }
}

}  // namespace aq
