// aq_math.h — arithmetic of the light-transport path, usable from host and
// device code: vectors, the PCG32 stream, the watertight ray/triangle test, the
// robust slab test, the Lambert + GGX BSDF, light sampling and the camera.
//
// The reference (`arukas`, src/lib.rs) ships no code; the semantics follow its
// data: `Principled` parameters (scenes/cbox.json:3-62), `Perspective` camera
// (scenes/cbox.json:516-543), `Point` lights (scenes/cbox.json:544-561) and the
// quad area light of CornellBox-Original.mtl:80-87 / .obj:160-167.
//
// Functions whose results must be bit-identical between the device and the
// FP32 CPU traversal (ray/box, ray/triangle) spell every rounding step with
// the *_rn helpers below so that no fused multiply-add is formed.
#pragma once

#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define AQ_HD __host__ __device__ __forceinline__
#define AQ_DEV __device__ __forceinline__
#else
#define AQ_HD inline
#define AQ_DEV inline
#endif

namespace aq {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.318309886183790671538f;

// ------------------------------------------------------------------ rounding
// Single rounding per operation, no contraction. Host builds use
// -ffp-contract=off; device builds call the _rn intrinsics.
AQ_HD float mul_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
AQ_HD float add_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
AQ_HD float sub_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
AQ_HD float div_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}
AQ_HD float rcp_rn(float a) {
#if defined(__CUDA_ARCH__)
    return __frcp_rn(a);
#else
    return 1.0f / a;
#endif
}
AQ_HD double dmul_rn(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
AQ_HD double dsub_rn(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
AQ_HD float fminf_(float a, float b) { return a < b ? a : b; }
AQ_HD float fmaxf_(float a, float b) { return a > b ? a : b; }
// Min/max of the slab test: one FMNMX on the device. The inputs are never
// NaN (inverse directions are finite), so the result equals the
// compare-select form except possibly for the sign of a zero, which no
// comparison downstream can see.
AQ_HD float smin(float a, float b) {
#if defined(__CUDA_ARCH__)
    return fminf(a, b);
#else
    return a < b ? a : b;
#endif
}
AQ_HD float smax(float a, float b) {
#if defined(__CUDA_ARCH__)
    return fmaxf(a, b);
#else
    return a > b ? a : b;
#endif
}

// ------------------------------------------------------------------ vectors
struct v3 {
    float x, y, z;
};
AQ_HD v3 mk(float x, float y, float z) { return v3{x, y, z}; }
AQ_HD v3 operator+(v3 a, v3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
AQ_HD v3 operator-(v3 a, v3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
AQ_HD v3 operator-(v3 a) { return {-a.x, -a.y, -a.z}; }
AQ_HD v3 operator*(v3 a, v3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
AQ_HD v3 operator*(v3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
AQ_HD v3 operator*(float s, v3 a) { return {a.x * s, a.y * s, a.z * s}; }
AQ_HD v3 operator/(v3 a, float s) { float r = 1.0f / s; return {a.x * r, a.y * r, a.z * r}; }
AQ_HD float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
AQ_HD v3 cross(v3 a, v3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
AQ_HD float length(v3 a) { return sqrtf(dot(a, a)); }
AQ_HD v3 normalize(v3 a) { return a * (1.0f / sqrtf(dot(a, a))); }
AQ_HD float maxc(v3 a) { return fmaxf_(a.x, fmaxf_(a.y, a.z)); }
AQ_HD float lum(v3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }
AQ_HD float comp(v3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
AQ_HD v3 lerp(v3 a, v3 b, float t) { return a + (b - a) * t; }

// ------------------------------------------------------------------ PCG32
// PCG-XSH-RR 64/32 (O'Neill 2014, "PCG: A Family of Simple Fast
// Space-Efficient Statistically Good Algorithms for Random Number
// Generation"), pcg32_srandom_r seeding. One stream per pixel: inc = 2*pixel+1.
constexpr uint64_t kPcgMult = 6364136223846793005ULL;

AQ_HD uint32_t pcg32_next(uint64_t& state, uint64_t inc) {
    uint64_t old = state;
    state = old * kPcgMult + inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((0u - rot) & 31u));
}
AQ_HD uint64_t pcg32_seed(uint64_t initstate, uint64_t initseq, uint64_t& inc) {
    uint64_t state = 0;
    inc = (initseq << 1u) | 1u;
    pcg32_next(state, inc);
    state += initstate;
    pcg32_next(state, inc);
    return state;
}
// SplitMix64 finaliser (Steele, Lea, Flood 2014) to decorrelate sample starts.
AQ_HD uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
// Start of sample `sample` of pixel `pixel`: stream = pixel, state from
// (seed, sample). Every path owns its own position in its pixel's stream.
AQ_HD uint64_t path_rng_state(uint64_t seed, uint32_t pixel, uint32_t sample) {
    uint64_t inc;
    return pcg32_seed(splitmix64(seed ^ (0xD1B54A32D192ED03ULL * ((uint64_t)sample + 1ULL))),
                      (uint64_t)pixel, inc);
}
AQ_HD uint64_t pixel_inc(uint32_t pixel) { return ((uint64_t)pixel << 1u) | 1u; }
// Uniform float in [0,1): top 24 bits, exactly representable.
AQ_HD float u01(uint32_t r) { return (float)(r >> 8) * (1.0f / 16777216.0f); }

// Random numbers a path draws: per camera sample and per bounce, always the
// same count whatever branch is taken, so a divergence stays within one path.
constexpr int kCameraDims = 4;  // pixel jitter x/y, lens u/v
constexpr int kBounceDims = 8;  // light pick, light u/v, lobe, dir u/v, RR, spare

// ------------------------------------------------------------------ ray/box
// Slab test in the form (b - o) * invd (Ize 2013, "Robust BVH Ray Traversal",
// JCGT 2(2)). The far distance is scaled by 1 + 1e-5, well above Ize's
// 1 + 2*gamma(3) (3.6e-7): a box the exact ray touches is never rejected,
// and a box is not culled by a triangle hit that ties with one inside it to
// within the rounding of the triangle test either, so the closest hit, ties
// broken by the smaller scene index, does not depend on the visit order.
constexpr float kSlabFarScale = 1.00001f;

struct RayPre {
    v3 o, invd;
    float tmin, tmax;
};
AQ_HD float safe_inv(float d) {
    float ad = d < 0.0f ? -d : d;
    float dd = ad < 1e-20f ? (d < 0.0f ? -1e-20f : 1e-20f) : d;
    return rcp_rn(dd);
}
// Returns entry distance, or +inf when the box is missed within [tmin, tfar].
AQ_HD float slab_entry(float lox, float hix, float loy, float hiy, float loz, float hiz,
                       const RayPre& r, float tfar_limit) {
    float tx0 = mul_rn(sub_rn(lox, r.o.x), r.invd.x);
    float tx1 = mul_rn(sub_rn(hix, r.o.x), r.invd.x);
    float ty0 = mul_rn(sub_rn(loy, r.o.y), r.invd.y);
    float ty1 = mul_rn(sub_rn(hiy, r.o.y), r.invd.y);
    float tz0 = mul_rn(sub_rn(loz, r.o.z), r.invd.z);
    float tz1 = mul_rn(sub_rn(hiz, r.o.z), r.invd.z);
    float tn = smax(smax(smin(tx0, tx1), smin(ty0, ty1)), smax(smin(tz0, tz1), r.tmin));
    float tf = smin(smin(smax(tx0, tx1), smax(ty0, ty1)), smin(smax(tz0, tz1), tfar_limit));
    tf = mul_rn(tf, kSlabFarScale);
    return tn <= tf ? tn : INFINITY;
}

// ------------------------------------------------------------------ ray/triangle
// Watertight ray/triangle intersection (Woop, Benthin, Wald 2013, JCGT 2(1)).
// Per-ray shear constants, then per triangle: translate, shear, edge functions
// (with the paper's double-precision fallback when an edge function is 0),
// determinant and scaled distance.
struct RayShear {
    v3 o;
    int kx, ky, kz;
    float Sx, Sy, Sz;
};
AQ_HD RayShear make_shear(v3 o, v3 d) {
    RayShear s;
    s.o = o;
    float ax = d.x < 0 ? -d.x : d.x, ay = d.y < 0 ? -d.y : d.y, az = d.z < 0 ? -d.z : d.z;
    int kz = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (comp(d, kz) < 0.0f) { int t = kx; kx = ky; ky = t; }
    s.kx = kx; s.ky = ky; s.kz = kz;
    float dz = comp(d, kz);
    s.Sx = div_rn(comp(d, kx), dz);
    s.Sy = div_rn(comp(d, ky), dz);
    s.Sz = rcp_rn(dz);
    return s;
}

struct TriHit {
    float t, u, v;  // u: weight of v1, v: weight of v2
    bool hit;
};
AQ_HD TriHit intersect_tri(const RayShear& s, v3 v0, v3 v1, v3 v2, float tmin, float tmax) {
    TriHit h;
    h.hit = false; h.t = 0.0f; h.u = 0.0f; h.v = 0.0f;
    v3 A = mk(sub_rn(v0.x, s.o.x), sub_rn(v0.y, s.o.y), sub_rn(v0.z, s.o.z));
    v3 B = mk(sub_rn(v1.x, s.o.x), sub_rn(v1.y, s.o.y), sub_rn(v1.z, s.o.z));
    v3 C = mk(sub_rn(v2.x, s.o.x), sub_rn(v2.y, s.o.y), sub_rn(v2.z, s.o.z));
    float Akz = comp(A, s.kz), Bkz = comp(B, s.kz), Ckz = comp(C, s.kz);
    float Ax = sub_rn(comp(A, s.kx), mul_rn(s.Sx, Akz));
    float Ay = sub_rn(comp(A, s.ky), mul_rn(s.Sy, Akz));
    float Bx = sub_rn(comp(B, s.kx), mul_rn(s.Sx, Bkz));
    float By = sub_rn(comp(B, s.ky), mul_rn(s.Sy, Bkz));
    float Cx = sub_rn(comp(C, s.kx), mul_rn(s.Sx, Ckz));
    float Cy = sub_rn(comp(C, s.ky), mul_rn(s.Sy, Ckz));
    float U = sub_rn(mul_rn(Cx, By), mul_rn(Cy, Bx));
    float V = sub_rn(mul_rn(Ax, Cy), mul_rn(Ay, Cx));
    float W = sub_rn(mul_rn(Bx, Ay), mul_rn(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)dsub_rn(dmul_rn((double)Cx, (double)By), dmul_rn((double)Cy, (double)Bx));
        V = (float)dsub_rn(dmul_rn((double)Ax, (double)Cy), dmul_rn((double)Ay, (double)Cx));
        W = (float)dsub_rn(dmul_rn((double)Bx, (double)Ay), dmul_rn((double)By, (double)Ax));
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return h;
    float det = add_rn(add_rn(U, V), W);
    if (det == 0.0f) return h;
    float Az = mul_rn(s.Sz, Akz), Bz = mul_rn(s.Sz, Bkz), Cz = mul_rn(s.Sz, Ckz);
    float T = add_rn(add_rn(mul_rn(U, Az), mul_rn(V, Bz)), mul_rn(W, Cz));
    float rcp = rcp_rn(det);
    float t = mul_rn(T, rcp);
    if (!(t > tmin && t < tmax)) return h;
    h.t = t;
    h.u = mul_rn(V, rcp);
    h.v = mul_rn(W, rcp);
    h.hit = true;
    return h;
}

// ------------------------------------------------------------------ frames
// Orthonormal basis from a unit normal (Duff et al. 2017, "Building an
// Orthonormal Basis, Revisited", JCGT 6(1)).
AQ_HD void onb(v3 n, v3& t, v3& b) {
    float sign = n.z >= 0.0f ? 1.0f : -1.0f;
    float a = -1.0f / (sign + n.z);
    float bb = n.x * n.y * a;
    t = mk(1.0f + sign * n.x * n.x * a, sign * bb, -sign * n.x);
    b = mk(bb, sign + n.y * n.y * a, -n.y);
}

// Self-intersection avoidance by integer ULP offset along the normal
// (Waechter & Binder 2019, "A Fast and Robust Method for Avoiding
// Self-Intersection", Ray Tracing Gems ch. 6).
AQ_HD float int_as_float_(int32_t i) {
#if defined(__CUDA_ARCH__)
    return __int_as_float(i);
#else
    union { int32_t i; float f; } u; u.i = i; return u.f;
#endif
}
AQ_HD int32_t float_as_int_(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_int(f);
#else
    union { int32_t i; float f; } u; u.f = f; return u.i;
#endif
}
AQ_HD v3 offset_ray(v3 p, v3 n) {
    const float origin = 1.0f / 32.0f, float_scale = 1.0f / 65536.0f, int_scale = 256.0f;
    int32_t ix = (int32_t)(int_scale * n.x), iy = (int32_t)(int_scale * n.y), iz = (int32_t)(int_scale * n.z);
    v3 pi = mk(int_as_float_(float_as_int_(p.x) + (p.x < 0 ? -ix : ix)),
               int_as_float_(float_as_int_(p.y) + (p.y < 0 ? -iy : iy)),
               int_as_float_(float_as_int_(p.z) + (p.z < 0 ? -iz : iz)));
    return mk(fabsf(p.x) < origin ? p.x + float_scale * n.x : pi.x,
              fabsf(p.y) < origin ? p.y + float_scale * n.y : pi.y,
              fabsf(p.z) < origin ? p.z + float_scale * n.z : pi.z);
}

// ------------------------------------------------------------------ BSDF
// `Principled` (scenes/cbox.json:3-62). The base model is Lambert + GGX:
// f = (1-m) C/pi + D G2 F / (4 cos_o cos_i), with
//   D   GGX / Trowbridge-Reitz (Walter et al. 2007, EGSR),
//   G2  height-correlated Smith, 1 / (1 + L(wo) + L(wi)),
//   F   Schlick, F0 = lerp(0.08*specular, C, m),
//   alpha = max(roughness^2, 1e-3).
// When F0 = 0 (specular 0 and metallic 0) there is no GGX lobe at all: the
// surface is Lambertian. Sampling picks the GGX lobe with probability p_s and
// then samples visible normals (Heitz 2018, "Sampling the GGX Distribution
// of Visible Normals", JCGT 7(4)); otherwise cosine-weighted. The pdf is the
// mixture pdf.
//
// The full model (the `*_full` functions, used by scenes whose materials set
// specular_tint, sheen, clearcoat or transmission) adds, with t =
// transmission and C_t = C / lum(C):
//   diffuse and sheen weighted by (1-m)(1-t); sheen = sheen *
//     lerp(1, C_t, sheen_tint) * (1 - |wi.h|)^5 (Burley 2012);
//   the Schlick lobe weighted by 1 - (1-m)t, its dielectric F0 tinted:
//     0.08 * specular * lerp(1, C_t, specular_tint);
//   a rough dielectric lobe weighted by (1-m)t (Walter et al. 2007): exact
//     dielectric Fresnel F at the microfacet, reflection F D G2 / (4 cos cos)
//     (white), refraction C (1-F) D G2 |wi.h||wo.h| / (|cos_i| cos_o (wo.h +
//     eta wi.h)^2), eta = n(wi side) / n(wo side) = ior entering the front
//     face, 1/ior leaving it; sampled by visible normals, then reflection
//     with probability F;
//   clearcoat: 0.25 clearcoat D_GTR1 F_Schlick(0.04) G1(wo) G1(wi) /
//     (4 cos cos), GTR1 alpha = clearcoat_roughness^2, G1 with alpha 0.25
//     (Burley 2012, sampled by its closed-form inverse).
// With those four parameters 0 every full-model expression reduces to the
// base model's arithmetic exactly (additions of 0, products with 1).
struct Bsdf {
    v3 color;
    float metallic, alpha, specular;
    v3 F0;
    float p_spec;
    bool has_spec;
    // full model only
    float wdiff, wspec, wglass;  // (1-m)(1-t), 1-(1-m)t, (1-m)t
    v3 sheen;                    // wdiff * sheen * lerp(1, C_t, sheen_tint)
    float eta;                   // n(other side) / n(wo side)
    float cc, cc_a2;             // 0.25 clearcoat, GTR1 alpha^2
    float p_glass, p_cc;         // lobe-selection probabilities
};
AQ_HD Bsdf make_bsdf(v3 color, float metallic, float roughness, float specular) {
    Bsdf b;
    b.color = color;
    b.metallic = metallic;
    b.alpha = fmaxf_(roughness * roughness, 1e-3f);
    b.specular = specular;
    v3 f0d = mk(0.08f * specular, 0.08f * specular, 0.08f * specular);
    b.F0 = lerp(f0d, color, metallic);
    b.has_spec = (b.F0.x + b.F0.y + b.F0.z) > 0.0f;
    float ws = lum(b.F0);
    float wd = (1.0f - metallic) * lum(color);
    float ps = (ws + wd) > 0.0f ? ws / (ws + wd) : 0.5f;
    if (ws > 0.0f && wd > 0.0f) ps = fminf_(fmaxf_(ps, 0.1f), 0.9f);
    b.p_spec = b.has_spec ? ps : 0.0f;
    b.wdiff = 1.0f - metallic; b.wspec = 1.0f; b.wglass = 0.0f;
    b.sheen = mk(0, 0, 0);
    b.eta = 1.0f; b.cc = 0.0f; b.cc_a2 = 0.0f; b.p_glass = 0.0f; b.p_cc = 0.0f;
    return b;
}
// front: wo lies on the side the triangle's winding normal points to.
AQ_HD Bsdf make_bsdf_full(v3 color, float metallic, float roughness, float specular, float spec_tint, float sheen,
                          float sheen_tint, float clearcoat, float cc_rough, float tr, float ior_in, bool front) {
    Bsdf b;
    b.color = color;
    b.metallic = metallic;
    b.alpha = fmaxf_(roughness * roughness, 1e-3f);
    b.specular = specular;
    const float lc = lum(color);
    const v3 one = mk(1.0f, 1.0f, 1.0f);
    const v3 tint = lc > 0.0f ? color * (1.0f / lc) : one;
    v3 f0d = lerp(one, tint, spec_tint) * (0.08f * specular);
    b.F0 = lerp(f0d, color, metallic);
    b.wdiff = (1.0f - metallic) * (1.0f - tr);
    b.wglass = (1.0f - metallic) * tr;
    b.wspec = 1.0f - b.wglass;
    b.has_spec = (b.F0.x + b.F0.y + b.F0.z) > 0.0f && b.wspec > 0.0f;
    b.sheen = lerp(one, tint, sheen_tint) * (b.wdiff * sheen);
    const float ior = fmaxf_(ior_in, 1.001f);
    b.eta = front ? ior : 1.0f / ior;
    b.cc = 0.25f * clearcoat;
    const float ca = fminf_(fmaxf_(cc_rough * cc_rough, 1e-3f), 0.999f);
    b.cc_a2 = ca * ca;
    float ws = b.has_spec ? lum(b.F0) * b.wspec : 0.0f;
    float wd = b.wdiff * lc + lum(b.sheen);
    float ps = (ws + wd) > 0.0f ? ws / (ws + wd) : 0.5f;
    if (ws > 0.0f && wd > 0.0f) ps = fminf_(fmaxf_(ps, 0.1f), 0.9f);
    b.p_spec = b.has_spec ? ps : 0.0f;
    const float tot = wd + ws + b.wglass + b.cc;
    b.p_glass = b.wglass > 0.0f ? b.wglass / tot : 0.0f;
    b.p_cc = b.cc > 0.0f ? b.cc / tot : 0.0f;
    return b;
}
AQ_HD float ggx_D(float a2, float cos_h) {
    float c2 = cos_h * cos_h;
    float d = c2 * (a2 - 1.0f) + 1.0f;
    return a2 / (kPi * d * d);
}
AQ_HD float ggx_Lambda(float a2, float cos_t) {
    float c2 = cos_t * cos_t;
    float t2 = fmaxf_(1.0f - c2, 0.0f) / c2;
    return 0.5f * (-1.0f + sqrtf(1.0f + a2 * t2));
}
AQ_HD v3 schlick(v3 F0, float c) {
    float m = fminf_(fmaxf_(1.0f - c, 0.0f), 1.0f);
    float m5 = (m * m) * (m * m) * m;
    return F0 + (mk(1.0f, 1.0f, 1.0f) - F0) * m5;
}
AQ_HD float pow5_(float x) { return (x * x) * (x * x) * x; }
// GTR1 (Berry) distribution of the clearcoat lobe (Burley 2012, appendix B).
AQ_HD float gtr1_D(float a2, float cos_h) {
    return (a2 - 1.0f) / (kPi * logf(a2) * (1.0f + (a2 - 1.0f) * cos_h * cos_h));
}
// Unpolarised dielectric Fresnel reflectance; cos_i >= 0 on the incident
// side, eta = n(transmitted side) / n(incident side).
AQ_HD float fresnel_dielectric(float cos_i, float eta) {
    float s2 = (1.0f - cos_i * cos_i) / (eta * eta);
    if (s2 >= 1.0f) return 1.0f;
    float ct = sqrtf(1.0f - s2);
    float rs = (cos_i - eta * ct) / (cos_i + eta * ct);
    float rp = (eta * cos_i - ct) / (eta * cos_i + ct);
    return 0.5f * (rs * rs + rp * rp);
}
// wo, wi in the local frame (z = normal). Returns f (not times cos).
AQ_HD v3 bsdf_eval(const Bsdf& b, v3 wo, v3 wi) {
    if (wo.z <= 0.0f || wi.z <= 0.0f) return mk(0, 0, 0);
    v3 f = b.color * ((1.0f - b.metallic) * kInvPi);
    if (!b.has_spec) return f;
    v3 h = wo + wi;
    float hl = length(h);
    if (hl > 0.0f) {
        h = h * (1.0f / hl);
        float a2 = b.alpha * b.alpha;
        float D = ggx_D(a2, h.z);
        float G2 = 1.0f / (1.0f + ggx_Lambda(a2, wo.z) + ggx_Lambda(a2, wi.z));
        v3 F = schlick(b.F0, dot(wi, h));
        f = f + F * (D * G2 / (4.0f * wo.z * wi.z));
    }
    return f;
}
AQ_HD float bsdf_pdf(const Bsdf& b, v3 wo, v3 wi) {
    if (wo.z <= 0.0f || wi.z <= 0.0f) return 0.0f;
    float pd = wi.z * kInvPi;
    float ps = 0.0f;
    if (b.p_spec > 0.0f) {
        v3 h = wo + wi;
        float hl = length(h);
        if (hl > 0.0f) {
            h = h * (1.0f / hl);
            float a2 = b.alpha * b.alpha;
            float G1 = 1.0f / (1.0f + ggx_Lambda(a2, wo.z));
            ps = G1 * ggx_D(a2, h.z) / (4.0f * wo.z);
        }
    }
    return (1.0f - b.p_spec) * pd + b.p_spec * ps;
}
// GGX visible-normal sample for wo (Heitz 2018).
AQ_HD v3 ggx_vndf(float a, v3 wo, float u1, float u2) {
    v3 Vh = normalize(mk(a * wo.x, a * wo.y, wo.z));
    float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
    v3 T1 = lensq > 0.0f ? mk(-Vh.y, Vh.x, 0.0f) * (1.0f / sqrtf(lensq)) : mk(1.0f, 0.0f, 0.0f);
    v3 T2 = cross(Vh, T1);
    float r = sqrtf(u1);
    float phi = 2.0f * kPi * u2;
    float t1 = r * cosf(phi), t2 = r * sinf(phi);
    float s = 0.5f * (1.0f + Vh.z);
    t2 = (1.0f - s) * sqrtf(fmaxf_(1.0f - t1 * t1, 0.0f)) + s * t2;
    v3 Nh = T1 * t1 + T2 * t2 + Vh * sqrtf(fmaxf_(0.0f, 1.0f - t1 * t1 - t2 * t2));
    return normalize(mk(a * Nh.x, a * Nh.y, fmaxf_(0.0f, Nh.z)));
}
// Returns the sampled local direction; wi.z <= 0 means "no valid sample".
AQ_HD v3 bsdf_sample(const Bsdf& b, v3 wo, float ulobe, float u1, float u2) {
    if (ulobe < b.p_spec) {
        v3 Ne = ggx_vndf(b.alpha, wo, u1, u2);
        float d = dot(wo, Ne);
        return Ne * (2.0f * d) - wo;
    }
    float r = sqrtf(u1);
    float phi = 2.0f * kPi * u2;
    return mk(r * cosf(phi), r * sinf(phi), sqrtf(fmaxf_(0.0f, 1.0f - u1)));
}

// Half vector of refraction between wo (this side) and wi (the other side,
// index ratio eta), oriented to +z.
AQ_HD v3 refraction_half(v3 wo, v3 wi, float eta) {
    v3 h = normalize(wo + wi * eta);
    return h.z < 0.0f ? -h : h;
}
AQ_HD v3 bsdf_eval_full(const Bsdf& b, v3 wo, v3 wi) {
    if (wo.z <= 0.0f || wi.z == 0.0f) return mk(0, 0, 0);
    const float a2 = b.alpha * b.alpha;
    if (wi.z < 0.0f) {
        if (!(b.wglass > 0.0f)) return mk(0, 0, 0);
        v3 h = refraction_half(wo, wi, b.eta);
        float co = dot(wo, h), ci = dot(wi, h);
        if (!(co > 0.0f && ci < 0.0f)) return mk(0, 0, 0);
        float F = fresnel_dielectric(co, b.eta);
        float den = co + b.eta * ci;
        float G2 = 1.0f / (1.0f + ggx_Lambda(a2, wo.z) + ggx_Lambda(a2, wi.z));
        float v = b.wglass * (1.0f - F) * ggx_D(a2, h.z) * G2 * (-ci) * co / (-wi.z * wo.z * den * den);
        return b.color * v;
    }
    v3 f = b.color * (b.wdiff * kInvPi);
    v3 h = wo + wi;
    float hl = length(h);
    if (!(hl > 0.0f)) return f;
    h = h * (1.0f / hl);
    const float wih = dot(wi, h);
    f = f + b.sheen * pow5_(fminf_(fmaxf_(1.0f - wih, 0.0f), 1.0f));
    const float den = 4.0f * wo.z * wi.z;
    if (b.has_spec || b.wglass > 0.0f) {
        float D = ggx_D(a2, h.z);
        float G2 = 1.0f / (1.0f + ggx_Lambda(a2, wo.z) + ggx_Lambda(a2, wi.z));
        if (b.has_spec) {
            v3 F = schlick(b.F0, wih);
            f = f + F * (D * G2 / den * b.wspec);
        }
        if (b.wglass > 0.0f) {
            float F = fresnel_dielectric(dot(wo, h), b.eta);
            float v = b.wglass * F * D * G2 / den;
            f = f + mk(v, v, v);
        }
    }
    if (b.cc > 0.0f) {
        const float ga2 = 0.0625f;  // alpha 0.25
        float G = 1.0f / ((1.0f + ggx_Lambda(ga2, wo.z)) * (1.0f + ggx_Lambda(ga2, wi.z)));
        float m = fminf_(fmaxf_(1.0f - wih, 0.0f), 1.0f);
        float Fc = 0.04f + 0.96f * pow5_(m);
        float v = b.cc * gtr1_D(b.cc_a2, h.z) * Fc * G / den;
        f = f + mk(v, v, v);
    }
    return f;
}
AQ_HD float bsdf_pdf_full(const Bsdf& b, v3 wo, v3 wi) {
    if (wo.z <= 0.0f || wi.z == 0.0f) return 0.0f;
    const float a2 = b.alpha * b.alpha;
    const float G1 = 1.0f / (1.0f + ggx_Lambda(a2, wo.z));
    if (wi.z < 0.0f) {
        if (!(b.p_glass > 0.0f)) return 0.0f;
        v3 h = refraction_half(wo, wi, b.eta);
        float co = dot(wo, h), ci = dot(wi, h);
        if (!(co > 0.0f && ci < 0.0f)) return 0.0f;
        float F = fresnel_dielectric(co, b.eta);
        float den = co + b.eta * ci;
        return b.p_glass * (1.0f - F) * G1 * ggx_D(a2, h.z) * co / wo.z * (b.eta * b.eta * (-ci) / (den * den));
    }
    float pd = wi.z * kInvPi;
    float ps = 0.0f, pg = 0.0f, pc = 0.0f;
    v3 h = wo + wi;
    float hl = length(h);
    if (hl > 0.0f) {
        h = h * (1.0f / hl);
        float pv = G1 * ggx_D(a2, h.z) / (4.0f * wo.z);
        if (b.p_spec > 0.0f) ps = pv;
        if (b.p_glass > 0.0f) pg = fresnel_dielectric(dot(wo, h), b.eta) * pv;
        if (b.p_cc > 0.0f) pc = gtr1_D(b.cc_a2, h.z) * h.z / (4.0f * dot(wo, h));
    }
    float base = (1.0f - b.p_spec) * pd + b.p_spec * ps;
    return (1.0f - b.p_glass - b.p_cc) * base + b.p_glass * pg + b.p_cc * pc;
}
// Returns the sampled local direction: wi.z > 0 reflection, wi.z < 0
// refraction (glass lobe only), wi = 0 no sample. A reflection that lands
// below the surface or a refraction that lands above it is no sample, so
// that the pdf of every direction returned is bsdf_pdf_full's.
AQ_HD v3 bsdf_sample_full(const Bsdf& b, v3 wo, float ulobe, float u1, float u2) {
    const v3 none = mk(0.0f, 0.0f, 0.0f);
    if (ulobe < b.p_glass) {
        v3 h = ggx_vndf(b.alpha, wo, u1, u2);
        float co = dot(wo, h);
        float F = fresnel_dielectric(co, b.eta);
        if (ulobe < b.p_glass * F) {
            v3 r = h * (2.0f * co) - wo;
            return r.z > 0.0f ? r : none;
        }
        float ie = 1.0f / b.eta;
        float s2 = ie * ie * fmaxf_(0.0f, 1.0f - co * co);
        float ct = sqrtf(fmaxf_(0.0f, 1.0f - s2));
        v3 t = h * (ie * co - ct) - wo * ie;
        return t.z < 0.0f ? t : none;
    }
    ulobe -= b.p_glass;
    if (ulobe < b.p_cc) {
        float c2 = (1.0f - powf(b.cc_a2, 1.0f - u1)) / (1.0f - b.cc_a2);
        float ch = sqrtf(fminf_(fmaxf_(c2, 0.0f), 1.0f));
        float sh = sqrtf(fmaxf_(0.0f, 1.0f - ch * ch));
        float phi = 2.0f * kPi * u2;
        v3 h = mk(sh * cosf(phi), sh * sinf(phi), ch);
        float d = dot(wo, h);
        if (d < 0.0f) { h = -h; d = -d; }
        v3 r = h * (2.0f * d) - wo;
        return r.z > 0.0f ? r : none;
    }
    ulobe -= b.p_cc;
    const float rest = 1.0f - b.p_glass - b.p_cc;
    v3 r = bsdf_sample(b, wo, rest > 0.0f ? ulobe / rest : 1.0f, u1, u2);
    return r.z > 0.0f ? r : none;
}

// The base or the full model, chosen at compile time by the kernels.
template <bool FULL>
AQ_HD v3 bsdf_eval_t(const Bsdf& b, v3 wo, v3 wi) { return FULL ? bsdf_eval_full(b, wo, wi) : bsdf_eval(b, wo, wi); }
template <bool FULL>
AQ_HD float bsdf_pdf_t(const Bsdf& b, v3 wo, v3 wi) { return FULL ? bsdf_pdf_full(b, wo, wi) : bsdf_pdf(b, wo, wi); }
template <bool FULL>
AQ_HD v3 bsdf_sample_t(const Bsdf& b, v3 wo, float ul, float u1, float u2) {
    return FULL ? bsdf_sample_full(b, wo, ul, u1, u2) : bsdf_sample(b, wo, ul, u1, u2);
}

AQ_HD float power_heuristic(float a, float b) {
    float a2 = a * a, b2 = b * b;
    return (a2 + b2) > 0.0f ? a2 / (a2 + b2) : 0.0f;
}

// sRGB transfer (IEC 61966-2-1) decode, used for `Srgb` colours
// (cbox.json:5 Srgb 0.8677 -> 0.725 = CornellBox-Original.mtl:37 Kd).
inline double srgb_to_linear(double c) {
    return c <= 0.04045 ? c / 12.92 : pow((c + 0.055) / 1.055, 2.4);
}

}  // namespace aq
