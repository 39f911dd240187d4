// oracle.cpp — CPU oracle (test infrastructure; see oracle.h). Parity
// unpinned: the reference ships no implementation to compare against.
//
// Built with -ffp-contract=off so that every float expression rounds once
// per operation, which the bit-exact traversal comparison relies on.
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <thread>
#include <utility>
#include <vector>

namespace {

// ------------------------------------------------------------------ vectors
template <class T>
struct V3 {
    T x, y, z;
};
template <class T> V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> T dot3(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> V3<T> cross3(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> T len3(V3<T> a) { return std::sqrt(dot3(a, a)); }
template <class T> V3<T> unit(V3<T> a) { return a * (T(1) / std::sqrt(dot3(a, a))); }
template <class T> T max3(V3<T> a) { return std::max(a.x, std::max(a.y, a.z)); }
template <class T> T at(V3<T> a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
template <class T> T luminance(V3<T> c) { return T(0.2126) * c.x + T(0.7152) * c.y + T(0.0722) * c.z; }

inline float mn(float a, float b) { return a < b ? a : b; }
inline float mx(float a, float b) { return a > b ? a : b; }

// ------------------------------------------------------------------ PCG32
struct Pcg {
    uint64_t state, inc;
    uint32_t next() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((0u - rot) & 31u));
    }
    void seed(uint64_t initstate, uint64_t initseq) {
        state = 0;
        inc = (initseq << 1u) | 1u;
        next();
        state += initstate;
        next();
    }
    double uniform() { return (double)(next() >> 8) * (1.0 / 16777216.0); }
};
uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
// Sample `sample` of pixel `pixel`: PCG32 stream `pixel`, start derived
// from (seed, sample).
Pcg path_rng(uint64_t seed, uint32_t pixel, uint32_t sample) {
    Pcg r;
    r.seed(mix64(seed ^ (0xD1B54A32D192ED03ULL * ((uint64_t)sample + 1ULL))), (uint64_t)pixel);
    return r;
}

// ------------------------------------------------------------------ scene view
struct Tri {
    V3<float> a, b, c;
};
Tri tri_at(const orc_scene* s, int32_t i) {
    const float* v = s->verts + 9 * (size_t)i;
    return {{v[0], v[1], v[2]}, {v[3], v[4], v[5]}, {v[6], v[7], v[8]}};
}

// ------------------------------------------------------------------ FP32 watertight
struct ShearF {
    V3<float> o;
    int kx, ky, kz;
    float Sx, Sy, Sz;
};
ShearF shear_f(V3<float> o, V3<float> d) {
    ShearF s;
    s.o = o;
    float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    s.kz = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
    s.kx = (s.kz + 1) % 3;
    s.ky = (s.kx + 1) % 3;
    if (at(d, s.kz) < 0.0f) std::swap(s.kx, s.ky);
    s.Sx = at(d, s.kx) / at(d, s.kz);
    s.Sy = at(d, s.ky) / at(d, s.kz);
    s.Sz = 1.0f / at(d, s.kz);
    return s;
}
// Returns true and (t, u, v) when tmin < t < tmax.
bool hit_f(const ShearF& s, const Tri& tr, float tmin, float tmax, float& t, float& u, float& v) {
    V3<float> A = tr.a - s.o, B = tr.b - s.o, Cc = tr.c - s.o;
    float Az_ = at(A, s.kz), Bz_ = at(B, s.kz), Cz_ = at(Cc, s.kz);
    float Ax = at(A, s.kx) - s.Sx * Az_, Ay = at(A, s.ky) - s.Sy * Az_;
    float Bx = at(B, s.kx) - s.Sx * Bz_, By = at(B, s.ky) - s.Sy * Bz_;
    float Cx = at(Cc, s.kx) - s.Sx * Cz_, Cy = at(Cc, s.ky) - s.Sy * Cz_;
    float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = (U + V) + W;
    if (det == 0.0f) return false;
    float T = ((U * (s.Sz * Az_)) + (V * (s.Sz * Bz_))) + (W * (s.Sz * Cz_));
    float r = 1.0f / det;
    float tt = T * r;
    if (!(tt > tmin && tt < tmax)) return false;
    t = tt;
    u = V * r;
    v = W * r;
    return true;
}

// ------------------------------------------------------------------ FP64 watertight
bool hit_d(V3<double> o, V3<double> d, const Tri& tr, double tmin, double tmax, double& t, double& u, double& v) {
    double ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    int kz = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
    int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
    if (at(d, kz) < 0.0) std::swap(kx, ky);
    double Sx = at(d, kx) / at(d, kz), Sy = at(d, ky) / at(d, kz), Sz = 1.0 / at(d, kz);
    V3<double> a{tr.a.x, tr.a.y, tr.a.z}, b{tr.b.x, tr.b.y, tr.b.z}, c{tr.c.x, tr.c.y, tr.c.z};
    V3<double> A = a - o, B = b - o, Cc = c - o;
    double Ax = at(A, kx) - Sx * at(A, kz), Ay = at(A, ky) - Sy * at(A, kz);
    double Bx = at(B, kx) - Sx * at(B, kz), By = at(B, ky) - Sy * at(B, kz);
    double Cx = at(Cc, kx) - Sx * at(Cc, kz), Cy = at(Cc, ky) - Sy * at(Cc, kz);
    double U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if ((U < 0 || V < 0 || W < 0) && (U > 0 || V > 0 || W > 0)) return false;
    double det = U + V + W;
    if (det == 0.0) return false;
    double T = U * Sz * at(A, kz) + V * Sz * at(B, kz) + W * Sz * at(Cc, kz);
    double tt = T / det;
    if (!(tt > tmin && tt < tmax)) return false;
    t = tt;
    u = V / det;
    v = W / det;
    return true;
}

// ------------------------------------------------------------------ BVH walk
// Walks the exported BVH in the order of the device's canonical traversal
// (csrc/device.cuh, traverse): same nodes, same box tests, same counts.
inline const float* node_at(const orc_scene* s, int32_t i) { return s->nodes + 32 * (size_t)i; }

// Four-wide node (32 floats: lo.x, hi.x, lo.y, hi.y, lo.z, hi.z of the four
// child boxes, then the child links as int32). Restates the device's
// visit_wide (csrc/device.cuh): entry distances of the four boxes, the same
// five-comparator ordering network (ties keep slot order), the hit children
// but the nearest pushed farthest first; returns the nearest child, else the
// top of the stack, else kDone.
constexpr int32_t kDone = std::numeric_limits<int32_t>::min();
constexpr int kStack = 128;  // the library refuses trees needing 96 or more
template <class T, class Entry>
int32_t visit_wide(const float* w, Entry&& entry, int32_t* stack, int& sp) {
    T t[4];
    int32_t c[4];
    for (int k = 0; k < 4; ++k) {
        t[k] = entry(w[k], w[4 + k], w[8 + k], w[12 + k], w[16 + k], w[20 + k]);
        memcpy(&c[k], &w[24 + k], 4);
    }
    auto ce = [&](int a, int b) {
        if (t[b] < t[a]) {
            std::swap(t[a], t[b]);
            std::swap(c[a], c[b]);
        }
    };
    ce(0, 1); ce(2, 3); ce(0, 2); ce(1, 3); ce(1, 2);
    const T inf = std::numeric_limits<T>::infinity();
    for (int k = 3; k >= 1; --k)
        if (t[k] != inf) {
            if (sp >= kStack) abort();
            stack[sp++] = c[k];
        }
    if (t[0] != inf) return c[0];
    return sp > 0 ? stack[--sp] : kDone;
}

struct RayF {
    V3<float> o, d, invd;
    float tmin, tmax;
};
inline float inv_safe(float d) {
    float ad = std::fabs(d);
    float dd = ad < 1e-20f ? (d < 0.0f ? -1e-20f : 1e-20f) : d;
    return 1.0f / dd;
}
inline float entry_f(float lox, float hix, float loy, float hiy, float loz, float hiz, const RayF& r, float tlim) {
    float tx0 = (lox - r.o.x) * r.invd.x, tx1 = (hix - r.o.x) * r.invd.x;
    float ty0 = (loy - r.o.y) * r.invd.y, ty1 = (hiy - r.o.y) * r.invd.y;
    float tz0 = (loz - r.o.z) * r.invd.z, tz1 = (hiz - r.o.z) * r.invd.z;
    float tn = mx(mx(mn(tx0, tx1), mn(ty0, ty1)), mx(mn(tz0, tz1), r.tmin));
    float tf = mn(mn(mx(tx0, tx1), mx(ty0, ty1)), mn(mx(tz0, tz1), tlim));
    tf = tf * 1.00001f;  // conservative far scale, 1e-5 relative
    return tn <= tf ? tn : std::numeric_limits<float>::infinity();
}

// A quantized node (bvh.h: origin + 8-bit offsets, plane = fmaf(q, 2^(e -
// 127), origin)) decoded into the 32-float layout the walk reads; empty
// slots (link ~0) get +inf boxes, which every ray misses, as the device
// skips them.
const float* decode_qnode(const orc_scene* s, int32_t i, float* w) {
    const float* q = s->qnodes + 16 * (size_t)i;
    uint32_t ex, bytes[6];
    memcpy(&ex, &q[3], 4);
    memcpy(bytes, &q[8], 24);
    int32_t link[4];
    memcpy(link, &q[4], 16);
    for (int a = 0; a < 3; ++a) {
        uint32_t sb = ((ex >> (8 * a)) & 0xffu) << 23;
        float sc;
        memcpy(&sc, &sb, 4);
        for (int k = 0; k < 4; ++k) {
            const float ql = (float)((bytes[2 * a] >> (8 * k)) & 0xffu);
            const float qh = (float)((bytes[2 * a + 1] >> (8 * k)) & 0xffu);
            const bool empty = link[k] == ~0;
            w[8 * a + k] = empty ? std::numeric_limits<float>::infinity() : std::fmaf(ql, sc, q[a]);
            w[8 * a + 4 + k] = empty ? std::numeric_limits<float>::infinity() : std::fmaf(qh, sc, q[a]);
        }
    }
    memcpy(&w[24], link, 16);
    return w;
}

struct HitF {
    float t, u, v;
    int32_t leaf_idx, id;
    uint32_t nodes, tris;
};
HitF trace_f(const orc_scene* s, V3<float> o, V3<float> d, float tmin, float tmax, bool any) {
    RayF r{o, d, {inv_safe(d.x), inv_safe(d.y), inv_safe(d.z)}, tmin, tmax};
    ShearF sh = shear_f(o, d);
    HitF h{tmax, 0, 0, -1, 0x7fffffff, 0, 0};
    int32_t stack[kStack];
    int sp = 0;
    int32_t node = 0;
    auto entry = [&](float lx, float hx, float ly, float hy, float lz, float hz) {
        return entry_f(lx, hx, ly, hy, lz, hz, r, h.t);
    };
    float qbuf[32];
    while (true) {
        while (node >= 0) {
            h.nodes++;
            node = visit_wide<float>(s->qnodes ? decode_qnode(s, node, qbuf) : node_at(s, node), entry, stack, sp);
        }
        if (node == kDone) return h;
        int32_t code = ~node;
        int32_t first = code >> 3, cnt = code & 7;
        for (int k = 0; k < cnt; ++k) {
            int32_t id = s->tri_order[first + k];
            float t, u, v;
            h.tris++;
            if (hit_f(sh, tri_at(s, id), tmin, tmax, t, u, v)) {
                if (any) { h.t = t; h.leaf_idx = first + k; h.id = id; return h; }
                if (t < h.t || (t == h.t && id < h.id)) { h.t = t; h.u = u; h.v = v; h.leaf_idx = first + k; h.id = id; }
            }
        }
        if (sp == 0) return h;
        node = stack[--sp];
    }
}

// FP64 walk of the same tree (boxes are float, exact in double).
struct HitD {
    double t, u, v;
    int32_t id;
};
HitD trace_d(const orc_scene* s, V3<double> o, V3<double> d, double tmin, double tmax, bool any) {
    V3<double> invd{1.0 / (std::fabs(d.x) < 1e-300 ? 1e-300 : d.x), 1.0 / (std::fabs(d.y) < 1e-300 ? 1e-300 : d.y),
                    1.0 / (std::fabs(d.z) < 1e-300 ? 1e-300 : d.z)};
    HitD h{tmax, 0, 0, -1};
    int32_t stack[kStack];
    int sp = 0;
    int32_t node = 0;
    auto entry = [&](double lx, double hx, double ly, double hy, double lz, double hz) {
        double tx0 = (lx - o.x) * invd.x, tx1 = (hx - o.x) * invd.x;
        double ty0 = (ly - o.y) * invd.y, ty1 = (hy - o.y) * invd.y;
        double tz0 = (lz - o.z) * invd.z, tz1 = (hz - o.z) * invd.z;
        double tn = std::max(std::max(std::min(tx0, tx1), std::min(ty0, ty1)), std::max(std::min(tz0, tz1), tmin));
        double tf = std::min(std::min(std::max(tx0, tx1), std::max(ty0, ty1)), std::min(std::max(tz0, tz1), h.t));
        tf *= 1.0 + 1e-12;
        return tn <= tf ? tn : std::numeric_limits<double>::infinity();
    };
    while (true) {
        while (node >= 0) node = visit_wide<double>(node_at(s, node), entry, stack, sp);
        if (node == kDone) return h;
        int32_t code = ~node;
        int32_t first = code >> 3, cnt = code & 7;
        for (int k = 0; k < cnt; ++k) {
            int32_t id = s->tri_order[first + k];
            double t, u, v;
            if (hit_d(o, d, tri_at(s, id), tmin, tmax, t, u, v)) {
                if (any) { h.t = t; h.id = id; return h; }
                if (t < h.t || (t == h.t && id < h.id)) { h.t = t; h.u = u; h.v = v; h.id = id; }
            }
        }
        if (sp == 0) return h;
        node = stack[--sp];
    }
}

template <class F>
void parallel_for(int64_t n, int threads, F&& f) {
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    threads = (int)std::min<int64_t>(threads, std::max<int64_t>(n, 1));
    std::atomic<int64_t> next{0};
    const int64_t chunk = 64;
    auto work = [&]() {
        while (true) {
            int64_t b = next.fetch_add(chunk);
            if (b >= n) break;
            int64_t e = std::min(n, b + chunk);
            for (int64_t i = b; i < e; ++i) f(i);
        }
    };
    std::vector<std::thread> th;
    for (int i = 1; i < threads; ++i) th.emplace_back(work);
    work();
    for (auto& t : th) t.join();
}

// ------------------------------------------------------------------ BSDF
// The `Principled` model (scenes/cbox.json:3-62), restated from its
// published lobes (see oracle.h): Lambert diffuse and sheen (Burley 2012),
// GGX / Trowbridge-Reitz specular with height-correlated Smith masking and
// Schlick Fresnel (Walter et al. 2007), visible-normal sampling (Heitz 2018),
// a rough dielectric reflection/refraction lobe with exact Fresnel (Walter
// et al. 2007) and a GTR1 clearcoat (Burley 2012). With specular_tint,
// sheen, clearcoat and transmission all 0 the terms reduce to Lambert + GGX.
template <class T>
struct Mat {
    V3<T> color, F0, sheen;
    T metallic, alpha, p_spec;
    bool has_spec;
    T wdiff, wspec, wglass, eta, cc, cc_a2, p_glass, p_cc;
};
template <class T> T lum3(V3<T> c) { return T(0.2126) * c.x + T(0.7152) * c.y + T(0.0722) * c.z; }
template <class T> V3<T> mix3(V3<T> a, V3<T> b, T t) { return a + (b - a) * t; }
template <class T>
Mat<T> make_mat(V3<T> color, T metallic, T roughness, T specular, T spec_tint, T sheen, T sheen_tint, T clearcoat,
                T cc_rough, T tr, T ior, bool front) {
    Mat<T> m;
    m.color = color;
    m.metallic = metallic;
    m.alpha = std::max(roughness * roughness, T(1e-3));
    const T lc = lum3(color);
    const V3<T> one{1, 1, 1};
    const V3<T> tint = lc > T(0) ? color * (T(1) / lc) : one;
    V3<T> f0d = mix3(one, tint, spec_tint) * (T(0.08) * specular);
    m.F0 = mix3(f0d, color, metallic);
    m.wdiff = (T(1) - metallic) * (T(1) - tr);
    m.wglass = (T(1) - metallic) * tr;
    m.wspec = T(1) - m.wglass;
    m.has_spec = (m.F0.x + m.F0.y + m.F0.z) > T(0) && m.wspec > T(0);
    m.sheen = mix3(one, tint, sheen_tint) * (m.wdiff * sheen);
    T e = std::max(ior, T(1.001));
    m.eta = front ? e : T(1) / e;
    m.cc = T(0.25) * clearcoat;
    T ca = std::min(std::max(cc_rough * cc_rough, T(1e-3)), T(0.999));
    m.cc_a2 = ca * ca;
    T ws = m.has_spec ? lum3(m.F0) * m.wspec : T(0);
    T wd = m.wdiff * lc + lum3(m.sheen);
    T ps = (ws + wd) > T(0) ? ws / (ws + wd) : T(0.5);
    if (ws > T(0) && wd > T(0)) ps = std::min(std::max(ps, T(0.1)), T(0.9));
    m.p_spec = m.has_spec ? ps : T(0);
    T tot = wd + ws + m.wglass + m.cc;
    m.p_glass = m.wglass > T(0) ? m.wglass / tot : T(0);
    m.p_cc = m.cc > T(0) ? m.cc / tot : T(0);
    return m;
}
template <class T> T D_ggx(T a2, T c) {
    T d = c * c * (a2 - T(1)) + T(1);
    return a2 / (T(M_PI) * d * d);
}
template <class T> T Lambda(T a2, T c) {
    T t2 = std::max(T(1) - c * c, T(0)) / (c * c);
    return T(0.5) * (-T(1) + std::sqrt(T(1) + a2 * t2));
}
template <class T> T D_gtr1(T a2, T c) { return (a2 - T(1)) / (T(M_PI) * std::log(a2) * (T(1) + (a2 - T(1)) * c * c)); }
template <class T> T pow5(T x) { return (x * x) * (x * x) * x; }
// Unpolarised Fresnel reflectance of a dielectric interface: cos_i >= 0 on
// the incident side, eta = n(transmitted) / n(incident).
template <class T> T fresnel_diel(T ci, T eta) {
    T s2 = (T(1) - ci * ci) / (eta * eta);
    if (s2 >= T(1)) return T(1);
    T ct = std::sqrt(T(1) - s2);
    T rs = (ci - eta * ct) / (ci + eta * ct), rp = (eta * ci - ct) / (eta * ci + ct);
    return T(0.5) * (rs * rs + rp * rp);
}
template <class T> V3<T> refr_half(V3<T> wo, V3<T> wi, T eta) {
    V3<T> h = unit(wo + wi * eta);
    return h.z < T(0) ? -h : h;
}
template <class T> V3<T> eval(const Mat<T>& m, V3<T> wo, V3<T> wi) {
    if (wo.z <= T(0) || wi.z == T(0)) return {0, 0, 0};
    const T a2 = m.alpha * m.alpha;
    if (wi.z < T(0)) {
        if (!(m.wglass > T(0))) return {0, 0, 0};
        V3<T> h = refr_half(wo, wi, m.eta);
        T co = dot3(wo, h), ci = dot3(wi, h);
        if (!(co > T(0) && ci < T(0))) return {0, 0, 0};
        T F = fresnel_diel(co, m.eta), den = co + m.eta * ci;
        T G2 = T(1) / (T(1) + Lambda(a2, wo.z) + Lambda(a2, wi.z));
        return m.color * (m.wglass * (T(1) - F) * D_ggx(a2, h.z) * G2 * (-ci) * co / (-wi.z * wo.z * den * den));
    }
    V3<T> f = m.color * (m.wdiff / T(M_PI));
    V3<T> h = wo + wi;
    T hl = len3(h);
    if (!(hl > T(0))) return f;
    h = h * (T(1) / hl);
    const T wih = dot3(wi, h);
    const T c = std::min(std::max(T(1) - wih, T(0)), T(1));
    f = f + m.sheen * pow5(c);
    const T den = T(4) * wo.z * wi.z;
    if (m.has_spec || m.wglass > T(0)) {
        T D = D_ggx(a2, h.z);
        T G2 = T(1) / (T(1) + Lambda(a2, wo.z) + Lambda(a2, wi.z));
        if (m.has_spec) {
            T c5 = pow5(c);
            V3<T> F{m.F0.x + (T(1) - m.F0.x) * c5, m.F0.y + (T(1) - m.F0.y) * c5, m.F0.z + (T(1) - m.F0.z) * c5};
            f = f + F * (D * G2 / den * m.wspec);
        }
        if (m.wglass > T(0)) {
            T v = m.wglass * fresnel_diel(dot3(wo, h), m.eta) * D * G2 / den;
            f = f + V3<T>{v, v, v};
        }
    }
    if (m.cc > T(0)) {
        const T ga2 = T(0.0625);
        T G = T(1) / ((T(1) + Lambda(ga2, wo.z)) * (T(1) + Lambda(ga2, wi.z)));
        T v = m.cc * D_gtr1(m.cc_a2, h.z) * (T(0.04) + T(0.96) * pow5(c)) * G / den;
        f = f + V3<T>{v, v, v};
    }
    return f;
}
template <class T> T pdf(const Mat<T>& m, V3<T> wo, V3<T> wi) {
    if (wo.z <= T(0) || wi.z == T(0)) return T(0);
    const T a2 = m.alpha * m.alpha;
    const T G1 = T(1) / (T(1) + Lambda(a2, wo.z));
    if (wi.z < T(0)) {
        if (!(m.p_glass > T(0))) return T(0);
        V3<T> h = refr_half(wo, wi, m.eta);
        T co = dot3(wo, h), ci = dot3(wi, h);
        if (!(co > T(0) && ci < T(0))) return T(0);
        T F = fresnel_diel(co, m.eta), den = co + m.eta * ci;
        return m.p_glass * (T(1) - F) * G1 * D_ggx(a2, h.z) * co / wo.z * (m.eta * m.eta * (-ci) / (den * den));
    }
    T pd = wi.z / T(M_PI), ps = T(0), pg = T(0), pc = T(0);
    V3<T> h = wo + wi;
    T hl = len3(h);
    if (hl > T(0)) {
        h = h * (T(1) / hl);
        T pv = G1 * D_ggx(a2, h.z) / (T(4) * wo.z);
        if (m.p_spec > T(0)) ps = pv;
        if (m.p_glass > T(0)) pg = fresnel_diel(dot3(wo, h), m.eta) * pv;
        if (m.p_cc > T(0)) pc = D_gtr1(m.cc_a2, h.z) * h.z / (T(4) * dot3(wo, h));
    }
    T base = (T(1) - m.p_spec) * pd + m.p_spec * ps;
    return (T(1) - m.p_glass - m.p_cc) * base + m.p_glass * pg + m.p_cc * pc;
}
template <class T> V3<T> vndf(T a, V3<T> wo, T u1, T u2) {
    V3<T> Vh = unit(V3<T>{a * wo.x, a * wo.y, wo.z});
    T l2 = Vh.x * Vh.x + Vh.y * Vh.y;
    V3<T> T1 = l2 > T(0) ? V3<T>{-Vh.y, Vh.x, T(0)} * (T(1) / std::sqrt(l2)) : V3<T>{1, 0, 0};
    V3<T> T2 = cross3(Vh, T1);
    T r = std::sqrt(u1), phi = T(2 * M_PI) * u2;
    T t1 = r * std::cos(phi), t2 = r * std::sin(phi);
    T s = T(0.5) * (T(1) + Vh.z);
    t2 = (T(1) - s) * std::sqrt(std::max(T(1) - t1 * t1, T(0))) + s * t2;
    V3<T> Nh = T1 * t1 + T2 * t2 + Vh * std::sqrt(std::max(T(0), T(1) - t1 * t1 - t2 * t2));
    return unit(V3<T>{a * Nh.x, a * Nh.y, std::max(T(0), Nh.z)});
}
// wi.z > 0 reflection, < 0 refraction (glass lobe), 0 no sample: a
// reflection below the surface or a refraction above it is no sample, so
// every returned direction has the density pdf() reports.
template <class T> V3<T> sample(const Mat<T>& m, V3<T> wo, T ul, T u1, T u2) {
    const V3<T> none{0, 0, 0};
    if (ul < m.p_glass) {
        V3<T> h = vndf(m.alpha, wo, u1, u2);
        T co = dot3(wo, h);
        T F = fresnel_diel(co, m.eta);
        if (ul < m.p_glass * F) {
            V3<T> r = h * (T(2) * co) - wo;
            return r.z > T(0) ? r : none;
        }
        T ie = T(1) / m.eta;
        T s2 = ie * ie * std::max(T(0), T(1) - co * co);
        T ct = std::sqrt(std::max(T(0), T(1) - s2));
        V3<T> t = h * (ie * co - ct) - wo * ie;
        return t.z < T(0) ? t : none;
    }
    ul -= m.p_glass;
    if (ul < m.p_cc) {
        T c2 = (T(1) - std::pow(m.cc_a2, T(1) - u1)) / (T(1) - m.cc_a2);
        T ch = std::sqrt(std::min(std::max(c2, T(0)), T(1)));
        T sh = std::sqrt(std::max(T(0), T(1) - ch * ch));
        T phi = T(2 * M_PI) * u2;
        V3<T> h{sh * std::cos(phi), sh * std::sin(phi), ch};
        T d = dot3(wo, h);
        if (d < T(0)) { h = -h; d = -d; }
        V3<T> r = h * (T(2) * d) - wo;
        return r.z > T(0) ? r : none;
    }
    ul -= m.p_cc;
    const T rest = T(1) - m.p_glass - m.p_cc;
    ul = rest > T(0) ? ul / rest : T(1);
    V3<T> r;
    if (ul < m.p_spec) {
        V3<T> Ne = vndf(m.alpha, wo, u1, u2);
        r = Ne * (T(2) * dot3(wo, Ne)) - wo;
    } else {
        T rr = std::sqrt(u1), phi = T(2 * M_PI) * u2;
        r = {rr * std::cos(phi), rr * std::sin(phi), std::sqrt(std::max(T(0), T(1) - u1))};
    }
    return r.z > T(0) ? r : none;
}
template <class T> T power(T a, T b) {
    T a2 = a * a, b2 = b * b;
    return (a2 + b2) > T(0) ? a2 / (a2 + b2) : T(0);
}
template <class T> void basis(V3<T> n, V3<T>& t, V3<T>& b) {
    T sign = n.z >= T(0) ? T(1) : T(-1);
    T a = T(-1) / (sign + n.z);
    T bb = n.x * n.y * a;
    t = {T(1) + sign * n.x * n.x * a, sign * bb, -sign * n.x};
    b = {bb, sign + n.y * n.y * a, -n.y};
}

// Integer-ULP offset along the normal (Waechter & Binder, Ray Tracing Gems
// 2019) for float; a relative epsilon for double.
V3<float> offset(V3<float> p, V3<float> n) {
    const float origin = 1.0f / 32.0f, fs = 1.0f / 65536.0f, is = 256.0f;
    int32_t ix = (int32_t)(is * n.x), iy = (int32_t)(is * n.y), iz = (int32_t)(is * n.z);
    auto bump = [](float x, int32_t d) {
        int32_t b;
        memcpy(&b, &x, 4);
        b += x < 0 ? -d : d;
        float r;
        memcpy(&r, &b, 4);
        return r;
    };
    return {std::fabs(p.x) < origin ? p.x + fs * n.x : bump(p.x, ix),
            std::fabs(p.y) < origin ? p.y + fs * n.y : bump(p.y, iy),
            std::fabs(p.z) < origin ? p.z + fs * n.z : bump(p.z, iz)};
}
V3<double> offset(V3<double> p, V3<double> n) {
    double m = std::max(1.0, std::max(std::fabs(p.x), std::max(std::fabs(p.y), std::fabs(p.z))));
    return p + n * (2e-6 * m);
}

// ------------------------------------------------------------------ integrator
struct Lut {
    double v[256];
    Lut() {
        for (int i = 0; i < 256; ++i) v[i] = orc_srgb_to_linear((double)i / 255.0);
    }
};

template <class T>
V3<T> texture(const orc_scene* s, const Lut& lut, int ti, T u, T v) {
    int w = s->tex_w[ti], h = s->tex_h[ti];
    const uint8_t* px = s->tex_rgba[ti];
    T x = u * (T)w - T(0.5), y = v * (T)h - T(0.5);
    T fx = std::floor(x), fy = std::floor(y);
    T ax = x - fx, ay = y - fy;
    long ix = (long)fx, iy = (long)fy;
    auto tx = [&](long X, long Y) {
        X %= w; if (X < 0) X += w;
        Y %= h; if (Y < 0) Y += h;
        const uint8_t* p = px + 4 * ((size_t)Y * (size_t)w + (size_t)X);
        return V3<T>{(T)lut.v[p[0]], (T)lut.v[p[1]], (T)lut.v[p[2]]};
    };
    V3<T> c00 = tx(ix, iy), c10 = tx(ix + 1, iy), c01 = tx(ix, iy + 1), c11 = tx(ix + 1, iy + 1);
    V3<T> a = c00 + (c10 - c00) * ax, b = c01 + (c11 - c01) * ax;
    return a + (b - a) * ay;
}

struct Cam {
    double tan_half, aspect;
};

template <class T>
struct Closest {
    bool hit;
    T t, u, v;
    int32_t id;
};
template <class T>
Closest<T> closest(const orc_scene* s, V3<T> o, V3<T> d, T tmax, bool any);
template <>
Closest<float> closest<float>(const orc_scene* s, V3<float> o, V3<float> d, float tmax, bool any) {
    HitF h = trace_f(s, o, d, 0.0f, tmax, any);
    return {h.leaf_idx >= 0, h.t, h.u, h.v, h.id};
}
template <>
Closest<double> closest<double>(const orc_scene* s, V3<double> o, V3<double> d, double tmax, bool any) {
    HitD h = trace_d(s, o, d, 0.0, tmax, any);
    return {h.id >= 0, h.t, h.u, h.v, h.id};
}

// Optional constant radiance cache: paths stop at bounce query_depth and
// add throughput x cache_rgb (the device's cache query with a network whose
// output is that constant).
// query_depth -2: the path-spread rule instead of a fixed bounce (Mueller et
// al. 2021, sec. 5; the device's AQUA_NRC_QUERY_SPREAD): a0 = t1^2 / (4 pi
// cos1) at the first vertex, the spread grows by sqrt(t^2 / (pdf cos)) per
// later vertex, and the path queries at the first vertex from bounce 1 on
// where spread^2 > 0.01 a0 (cos against the shading normal).
struct CacheConst {
    int query_depth = -1;
    double rgb[3] = {0, 0, 0};
};
constexpr int kQuerySpread = -2;

template <class T>
void render_pixel(const orc_scene* s, const Lut& lut, const std::vector<double>& cdf, int32_t spp, int32_t spp_offset,
                  int32_t max_depth, int32_t rr_depth, uint64_t seed, uint32_t pixel, double sum[3], double st[3],
                  const CacheConst& cache = CacheConst()) {
    const aqua_camera& c = s->cam;
    T tan_half = (T)std::tan(0.5 * (double)c.fov_deg * M_PI / 180.0);
    T aspect = (T)c.width / (T)c.height;
    V3<T> R{(T)c.right[0], (T)c.right[1], (T)c.right[2]}, U{(T)c.up[0], (T)c.up[1], (T)c.up[2]},
        B{(T)c.back[0], (T)c.back[1], (T)c.back[2]}, P{(T)c.pos[0], (T)c.pos[1], (T)c.pos[2]};
    V3<T> env{(T)s->env[0], (T)s->env[1], (T)s->env[2]};
    const T inf = std::numeric_limits<T>::infinity();
    uint32_t px = pixel % (uint32_t)c.width, py = pixel / (uint32_t)c.width;
    for (int32_t si = 0; si < spp; ++si) {
        Pcg rng = path_rng(seed, pixel, (uint32_t)(spp_offset + si));
        T u0 = (T)rng.uniform(), u1 = (T)rng.uniform(), u2 = (T)rng.uniform(), u3 = (T)rng.uniform();
        V3<T> dc{(T(2) * (((T)px + u0) / (T)c.width) - T(1)) * tan_half * aspect,
                 (T(1) - T(2) * (((T)py + u1) / (T)c.height)) * tan_half, T(-1)};
        V3<T> oc{0, 0, 0};
        if (c.lens_radius > 0.0f) {
            T a = T(2) * u2 - T(1), b = T(2) * u3 - T(1), lx = 0, ly = 0;
            if (a != T(0) || b != T(0)) {
                T r, phi;
                if (std::fabs(a) > std::fabs(b)) { r = a; phi = T(M_PI / 4) * (b / a); }
                else { r = b; phi = T(M_PI / 2) - T(M_PI / 4) * (a / b); }
                lx = r * std::cos(phi);
                ly = r * std::sin(phi);
            }
            oc = {lx * (T)c.lens_radius, ly * (T)c.lens_radius, T(0)};
            dc = dc * (T)c.focal - oc;
        }
        V3<T> o = P + R * oc.x + U * oc.y + B * oc.z;
        V3<T> d = unit(R * dc.x + U * dc.y + B * dc.z);
        V3<T> thr{1, 1, 1};
        T pdf_b = 0;
        T spread = 0, a0 = 0;  // path-spread query mode
        for (int depth = 0;; ++depth) {
            st[1] += 1;
            Closest<T> h = closest<T>(s, o, d, inf, false);
            if (!h.hit) {
                V3<T> e = thr * env;
                sum[0] += e.x; sum[1] += e.y; sum[2] += e.z;
                break;
            }
            const float* vv = s->verts + 9 * (size_t)h.id;
            V3<T> v0{(T)vv[0], (T)vv[1], (T)vv[2]}, v1{(T)vv[3], (T)vv[4], (T)vv[5]}, v2{(T)vv[6], (T)vv[7], (T)vv[8]};
            V3<T> e1 = v1 - v0, e2 = v2 - v0;
            V3<T> p = v0 + e1 * h.u + e2 * h.v;
            V3<T> ng = unit(cross3(e1, e2));
            V3<T> wo = -d;
            int light = s->tri_light[h.id];
            if (light >= 0) {
                const aqua_light& L = s->lights[light];
                V3<T> le1{(T)L.e1[0], (T)L.e1[1], (T)L.e1[2]}, le2{(T)L.e2[0], (T)L.e2[1], (T)L.e2[2]};
                V3<T> nl = unit(cross3(le1, le2));
                T area = len3(cross3(le1, le2)) * (L.type == AQUA_LIGHT_TRIANGLE ? T(0.5) : T(1));
                T cl = dot3(nl, wo);
                if (cl > T(0)) {
                    T w = 1;
                    if (depth > 0 && pdf_b > T(0)) w = power(pdf_b, (T)L.pmf * h.t * h.t / (area * cl));
                    V3<T> e = thr * V3<T>{(T)L.radiance[0], (T)L.radiance[1], (T)L.radiance[2]} * w;
                    sum[0] += e.x; sum[1] += e.y; sum[2] += e.z;
                }
            }
            if (depth >= max_depth) break;
            if (depth == cache.query_depth) {
                for (int c2 = 0; c2 < 3; ++c2) sum[c2] += (double)at(thr, c2) * cache.rgb[c2];
                break;
            }
            const bool front = dot3(ng, wo) >= T(0);  // wo on the winding normal's side
            if (!front) ng = -ng;
            // Shading normal: the interpolated vertex normal on ng's side when
            // wo lies above it, else ng (the device's shading_normal).
            V3<T> ns = ng;
            if (s->nrm) {
                const float* nv = s->nrm + 9 * (size_t)h.id;
                T w0 = T(1) - h.u - h.v;
                V3<T> n{(T)nv[0] * w0 + (T)nv[3] * h.u + (T)nv[6] * h.v,
                        (T)nv[1] * w0 + (T)nv[4] * h.u + (T)nv[7] * h.v,
                        (T)nv[2] * w0 + (T)nv[5] * h.u + (T)nv[8] * h.v};
                T l2 = dot3(n, n);
                if (l2 > T(0)) {
                    n = n * (T(1) / std::sqrt(l2));
                    if (dot3(n, ng) < T(0)) n = -n;
                    if (dot3(n, wo) > T(0)) ns = n;
                }
            }
            if (cache.query_depth == kQuerySpread) {
                const T cv = std::max(std::fabs(dot3(ns, wo)), T(1e-6));
                if (depth == 0) a0 = h.t * h.t / (T(4) * T(M_PI) * cv);
                else spread += std::sqrt(h.t * h.t / (std::max(pdf_b, T(1e-12)) * cv));
                if (depth > 0 && spread * spread > T(0.01) * a0) {
                    for (int c2 = 0; c2 < 3; ++c2) sum[c2] += (double)at(thr, c2) * cache.rgb[c2];
                    break;
                }
            }
            const aqua_material& m = s->mats[s->tri_mat[h.id]];
            V3<T> base{(T)m.base_color[0], (T)m.base_color[1], (T)m.base_color[2]};
            if (m.base_texture >= 0) {
                const float* uv = s->uvs + 6 * (size_t)h.id;
                T w0 = T(1) - h.u - h.v;
                T tu = (T)uv[0] * w0 + (T)uv[2] * h.u + (T)uv[4] * h.v;
                T tv = (T)uv[1] * w0 + (T)uv[3] * h.u + (T)uv[5] * h.v;
                base = base * texture<T>(s, lut, m.base_texture, tu, tv);
            }
            Mat<T> M = make_mat<T>(base, (T)m.metallic, (T)m.roughness, (T)m.specular, (T)m.specular_tint,
                                   (T)m.sheen, (T)m.sheen_tint, (T)m.clearcoat, (T)m.clearcoat_roughness,
                                   (T)m.transmission, (T)m.ior, front);
            V3<T> Tt, Bt;
            basis(ns, Tt, Bt);
            V3<T> wol{dot3(wo, Tt), dot3(wo, Bt), dot3(wo, ns)};
            T u[8];
            for (int k = 0; k < 8; ++k) u[k] = (T)rng.uniform();
            if (s->n_lights > 0 && wol.z > T(0)) {
                int li = 0;
                while (li < s->n_lights - 1 && !((double)u[0] < cdf[(size_t)li])) ++li;
                const aqua_light& L = s->lights[li];
                V3<T> lp{(T)L.p0[0], (T)L.p0[1], (T)L.p0[2]};
                V3<T> le{(T)L.radiance[0], (T)L.radiance[1], (T)L.radiance[2]};
                T pmf = (T)L.pmf;
                V3<T> contrib{0, 0, 0}, wi{0, 0, 1};
                T dist = 0;
                bool below = false;  // light sample on the far side (glass lobe)
                if (L.type == AQUA_LIGHT_POINT) {
                    V3<T> dl = lp - p;
                    T d2 = dot3(dl, dl);
                    dist = std::sqrt(d2);
                    wi = dl * (T(1) / dist);
                    T cs = dot3(wi, ns), cg = dot3(wi, ng);
                    below = M.wglass > T(0) && cs < T(0) && cg < T(0);
                    if (((cs > T(0) && cg > T(0)) || below) && d2 > T(0)) {
                        V3<T> wil{dot3(wi, Tt), dot3(wi, Bt), cs};
                        contrib = thr * eval(M, wol, wil) * le * (std::fabs(cs) / (d2 * pmf));
                    }
                } else {
                    V3<T> le1{(T)L.e1[0], (T)L.e1[1], (T)L.e1[2]}, le2{(T)L.e2[0], (T)L.e2[1], (T)L.e2[2]}, xl;
                    if (L.type == AQUA_LIGHT_QUAD) xl = lp + le1 * u[1] + le2 * u[2];
                    else {
                        T su = std::sqrt(u[1]);
                        xl = lp + le1 * (su * (T(1) - u[2])) + le2 * (su * u[2]);
                    }
                    V3<T> cr = cross3(le1, le2);
                    V3<T> nl = unit(cr);
                    T area = len3(cr) * (L.type == AQUA_LIGHT_TRIANGLE ? T(0.5) : T(1));
                    V3<T> dl = xl - p;
                    T d2 = dot3(dl, dl);
                    dist = std::sqrt(d2);
                    wi = dl * (T(1) / dist);
                    T cl = -dot3(wi, nl), cs = dot3(wi, ns), cg = dot3(wi, ng);
                    below = M.wglass > T(0) && cs < T(0) && cg < T(0);
                    if (cl > T(0) && ((cs > T(0) && cg > T(0)) || below) && d2 > T(0)) {
                        V3<T> wil{dot3(wi, Tt), dot3(wi, Bt), cs};
                        T pl = pmf * d2 / (area * cl);
                        T w = power(pl, pdf(M, wol, wil));
                        contrib = thr * eval(M, wol, wil) * le * (std::fabs(cs) * w / pl);
                    }
                }
                if (contrib.x > T(0) || contrib.y > T(0) || contrib.z > T(0)) {
                    st[2] += 1;
                    Closest<T> o2 = closest<T>(s, offset(p, below ? -ng : ng), wi, dist * T(1.0 - 1e-4), true);
                    if (!o2.hit) { sum[0] += contrib.x; sum[1] += contrib.y; sum[2] += contrib.z; }
                }
            }
            V3<T> wil = sample(M, wol, u[3], u[4], u[5]);
            const bool through = wil.z < T(0);  // refracted by the glass lobe
            if (!((wil.z > T(0) || through) && wol.z > T(0))) break;
            T pb = pdf(M, wol, wil);
            if (!(pb > T(0))) break;
            thr = thr * eval(M, wol, wil) * (std::fabs(wil.z) / pb);
            if (!(max3(thr) > T(0)) || !std::isfinite(thr.x) || !std::isfinite(thr.y) || !std::isfinite(thr.z)) break;
            if (depth >= rr_depth) {
                T q = std::min(T(1), max3(thr));
                if (u[6] >= q) break;
                thr = thr * (T(1) / q);
            }
            d = unit(Tt * wil.x + Bt * wil.y + ns * wil.z);
            if (through) {
                if (!(dot3(d, ng) < T(0))) break;  // refraction must cross the surface
            } else if (s->nrm && !(dot3(d, ng) > T(0))) {
                break;  // below the geometric surface
            }
            o = offset(p, through ? -ng : ng);
            pdf_b = pb;
        }
        st[0] += 1;
    }
}

// ------------------------------------------------------------------ MLP
// bfloat16 rounding, round to nearest even (finite inputs).
double to_bf16(double v) {
    float f = (float)v;
    uint32_t b;
    memcpy(&b, &f, 4);
    b = (b + 0x7FFFu + ((b >> 16) & 1u)) & 0xFFFF0000u;
    memcpy(&f, &b, 4);
    return (double)f;
}

struct Mlp {
    std::vector<double> W[6];  // W[l] row-major [out][in]
    int outs(int l) const { return l == 5 ? 3 : 64; }
    Mlp(const float* w, bool bf) {
        for (int l = 0; l < 6; ++l) {
            int o = outs(l);
            W[l].resize((size_t)o * 64);
            for (int i = 0; i < o * 64; ++i) {
                double v = w[l * 4096 + i];
                W[l][(size_t)i] = bf ? to_bf16(v) : v;
            }
        }
    }
    // h[0] = input, h[l+1] = relu(W_l h[l]) for l < 5; y = W_5 h[5].
    void forward(const float* x, bool bf, double h[6][64], double y[3]) const {
        for (int i = 0; i < 64; ++i) h[0][i] = bf ? to_bf16(x[i]) : (double)x[i];
        for (int l = 0; l < 5; ++l)
            for (int o = 0; o < 64; ++o) {
                double z = 0.0;
                for (int i = 0; i < 64; ++i) z += W[l][(size_t)o * 64 + i] * h[l][i];
                z = z > 0.0 ? z : 0.0;
                h[l + 1][o] = bf ? to_bf16(z) : z;
            }
        for (int o = 0; o < 3; ++o) {
            double z = 0.0;
            for (int i = 0; i < 64; ++i) z += W[5][(size_t)o * 64 + i] * h[5][i];
            y[o] = z;
        }
    }
};

// Encoding of one vertex (restated from the definition in oracle.h).
void encode_row(const float* r, const float* bmin, const float* bmax, float* x) {
    double pn[3];
    for (int a = 0; a < 3; ++a) {
        double t = ((double)r[a] - bmin[a]) / ((double)bmax[a] - bmin[a]);
        pn[a] = std::min(std::max(t, 0.0), 1.0);
    }
    auto sph = [](double x0, double y0, double z0, double& u, double& v) {
        u = std::acos(std::min(std::max(z0, -1.0), 1.0)) / M_PI;
        v = (std::atan2(y0, x0) + M_PI) / (2.0 * M_PI);
        u = std::min(std::max(u, 0.0), 1.0);
        v = std::min(std::max(v, 0.0), 1.0);
    };
    // One-blob: Gaussian of width 1/k centred on bin b of k.
    auto blob = [](double v, int b, int k) {
        double d = (v - (b + 0.5) / k) * k;
        return std::exp(-0.5 * d * d);
    };
    double du, dv, nu, nv;
    sph(r[3], r[4], r[5], du, dv);
    sph(r[6], r[7], r[8], nu, nv);
    double rough = std::min(std::max((double)r[9], 0.0), 1.0);
    for (int c = 0; c < 64; ++c) {
        double v;
        if (c < 48) {  // position: 8 octaves of sin/cos per axis
            int axis = c / 16, f = (c % 16) / 2;
            double a = pn[axis] * (double)(1 << f) * M_PI;
            v = (c & 1) ? std::cos(a) : std::sin(a);
        } else if (c < 54) {  // direction: 3 bins per coordinate
            int k = c - 48;
            v = blob(k < 3 ? du : dv, k % 3, 3);
        } else if (c < 58) {  // normal: 2 bins per coordinate
            int k = c - 54;
            v = blob(k < 2 ? nu : nv, k % 2, 2);
        } else if (c == 58) {
            v = rough;
        } else if (c < 62) {
            v = r[10 + (c - 59)];
        } else if (c == 62) {
            v = 0.2126 * r[13] + 0.7152 * r[14] + 0.0722 * r[15];
        } else {
            v = 1.0;
        }
        x[c] = (float)v;
    }
}

}  // namespace

extern "C" {

void orc_mlp_forward(const float* w, const float* x, int64_t n, int emulate_bf16, float* out) {
    Mlp net(w, emulate_bf16 != 0);
    parallel_for(n, 0, [&](int64_t r) {
        double h[6][64], y[3];
        net.forward(x + 64 * r, emulate_bf16 != 0, h, y);
        for (int c = 0; c < 3; ++c) out[3 * r + c] = (float)y[c];
    });
}

void orc_mlp_forward_f64(const float* w, const float* x, int64_t n, int emulate_bf16, double* out) {
    Mlp net(w, emulate_bf16 != 0);
    parallel_for(n, 0, [&](int64_t r) {
        double h[6][64], y[3];
        net.forward(x + 64 * r, emulate_bf16 != 0, h, y);
        for (int c = 0; c < 3; ++c) out[3 * r + c] = y[c];
    });
}

void orc_mlp_grad(const float* w, const float* x, const float* target, int64_t n, int emulate_bf16, double* grad,
                  double* loss) {
    const bool bf = emulate_bf16 != 0;
    Mlp net(w, bf);
    const double inv = 1.0 / (3.0 * (double)n);
    // Per-thread accumulation over fixed row blocks, summed in block order.
    const int64_t block = 256;
    int64_t nb = (n + block - 1) / block;
    std::vector<std::vector<double>> part((size_t)nb, std::vector<double>(AQUA_NRC_PARAMS + 1, 0.0));
    parallel_for(nb, 0, [&](int64_t b) {
        std::vector<double>& g = part[(size_t)b];
        for (int64_t r = b * block; r < std::min(n, (b + 1) * block); ++r) {
            double h[6][64], y[3], d[64], dn[64];
            net.forward(x + 64 * r, bf, h, y);
            double dy[3];
            for (int c = 0; c < 3; ++c) {
                double t = target[3 * r + c], den = y[c] * y[c] + 0.01, e = y[c] - t;
                g[AQUA_NRC_PARAMS] += e * e / den;
                dy[c] = 2.0 * e / den * inv;
                if (bf) dy[c] = to_bf16(dy[c]);
            }
            for (int o = 0; o < 3; ++o)
                for (int i = 0; i < 64; ++i) g[(size_t)(5 * 4096 + o * 64 + i)] += dy[o] * h[5][i];
            for (int i = 0; i < 64; ++i) {
                double s = 0.0;
                for (int o = 0; o < 3; ++o) s += net.W[5][(size_t)o * 64 + i] * dy[o];
                d[i] = h[5][i] > 0.0 ? s : 0.0;
                if (bf) d[i] = to_bf16(d[i]);
            }
            for (int l = 4; l >= 0; --l) {  // d = dL/dZ_l (delta of layer l+1)
                for (int o = 0; o < 64; ++o)
                    for (int i = 0; i < 64; ++i) g[(size_t)(l * 4096 + o * 64 + i)] += d[o] * h[l][i];
                if (l == 0) break;
                for (int i = 0; i < 64; ++i) {
                    double s = 0.0;
                    for (int o = 0; o < 64; ++o) s += net.W[l][(size_t)o * 64 + i] * d[o];
                    dn[i] = h[l][i] > 0.0 ? s : 0.0;
                    if (bf) dn[i] = to_bf16(dn[i]);
                }
                memcpy(d, dn, sizeof(d));
            }
        }
    });
    for (int p = 0; p <= AQUA_NRC_PARAMS; ++p) {
        double s = 0.0;
        for (int64_t b = 0; b < nb; ++b) s += part[(size_t)b][(size_t)p];
        if (p < AQUA_NRC_PARAMS) grad[p] = s;
        else if (loss) *loss = s * inv;
    }
}

void orc_nrc_encode(const float* raw, int64_t n, const float* bmin, const float* bmax, float* x) {
    parallel_for(n, 0, [&](int64_t r) { encode_row(raw + 16 * r, bmin, bmax, x + 64 * r); });
}

double orc_srgb_to_linear(double c) { return c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4); }

int orc_render(const orc_scene* s, int precision, int32_t spp, int32_t spp_offset, int32_t max_depth,
               int32_t rr_depth, uint64_t seed, int threads, int64_t pixel_begin, int64_t pixel_end, float* out,
               double* stats) {
    return orc_render_cached(s, precision, spp, spp_offset, max_depth, rr_depth, seed, threads, pixel_begin,
                             pixel_end, -1, nullptr, out, stats);
}

static Mat<double> mat_of(const aqua_material* m, int front) {
    return make_mat<double>({m->base_color[0], m->base_color[1], m->base_color[2]}, m->metallic, m->roughness,
                            m->specular, m->specular_tint, m->sheen, m->sheen_tint, m->clearcoat,
                            m->clearcoat_roughness, m->transmission, m->ior, front != 0);
}

void orc_bsdf_eval(const aqua_material* m, int front, const double* wo, const double* wi, int64_t n, double* f,
                   double* pdf_out) {
    const Mat<double> M = mat_of(m, front);
    for (int64_t k = 0; k < n; ++k) {
        V3<double> o{wo[3 * k], wo[3 * k + 1], wo[3 * k + 2]}, i{wi[3 * k], wi[3 * k + 1], wi[3 * k + 2]};
        V3<double> v = eval(M, o, i);
        f[3 * k] = v.x; f[3 * k + 1] = v.y; f[3 * k + 2] = v.z;
        if (pdf_out) pdf_out[k] = pdf(M, o, i);
    }
}

void orc_bsdf_sample(const aqua_material* m, int front, const double* wo, const double* u, int64_t n, double* wi) {
    const Mat<double> M = mat_of(m, front);
    for (int64_t k = 0; k < n; ++k) {
        V3<double> o{wo[3 * k], wo[3 * k + 1], wo[3 * k + 2]};
        V3<double> v = sample(M, o, u[3 * k], u[3 * k + 1], u[3 * k + 2]);
        wi[3 * k] = v.x; wi[3 * k + 1] = v.y; wi[3 * k + 2] = v.z;
    }
}

uint32_t orc_pcg32_first(uint64_t initstate, uint64_t initseq, uint32_t* out, int n) {
    Pcg r;
    r.seed(initstate, initseq);
    uint32_t last = 0;
    for (int i = 0; i < n; ++i) {
        last = r.next();
        if (out) out[i] = last;
    }
    return last;
}

void orc_trace_bvh_f32(const orc_scene* s, const float* rays, int64_t n, int any_hit, float* hits,
                       uint32_t* counts, int threads) {
    parallel_for(n, threads, [&](int64_t i) {
        const float* r = rays + 8 * i;
        HitF h = trace_f(s, {r[0], r[1], r[2]}, {r[4], r[5], r[6]}, r[3], r[7], any_hit != 0);
        float* o = hits + 4 * i;
        int32_t prim = h.leaf_idx >= 0 ? (any_hit ? 1 : h.id) : -1;
        if (any_hit || h.leaf_idx < 0) { o[0] = o[1] = o[2] = 0.0f; }
        else { o[0] = h.t; o[1] = h.u; o[2] = h.v; }
        memcpy(&o[3], &prim, 4);
        if (counts) { counts[2 * i] = h.nodes; counts[2 * i + 1] = h.tris; }
    });
}

void orc_trace_brute_f32(const orc_scene* s, const float* rays, int64_t n, int any_hit, float* hits, int threads) {
    parallel_for(n, threads, [&](int64_t i) {
        const float* r = rays + 8 * i;
        V3<float> o{r[0], r[1], r[2]}, d{r[4], r[5], r[6]};
        ShearF sh = shear_f(o, d);
        float bt = r[7], bu = 0, bv = 0;
        int32_t bid = -1;
        for (int32_t k = 0; k < s->n_tris; ++k) {
            float t, u, v;
            if (hit_f(sh, tri_at(s, k), r[3], r[7], t, u, v)) {
                if (bid < 0 || t < bt || (t == bt && k < bid)) { bt = t; bu = u; bv = v; bid = k; }
                if (any_hit) break;
            }
        }
        float* out = hits + 4 * i;
        int32_t prim = bid >= 0 ? (any_hit ? 1 : bid) : -1;
        if (any_hit || bid < 0) { out[0] = out[1] = out[2] = 0.0f; }
        else { out[0] = bt; out[1] = bu; out[2] = bv; }
        memcpy(&out[3], &prim, 4);
    });
}

void orc_trace_brute_f64(const orc_scene* s, const float* rays, int64_t n, double* hits, int threads) {
    parallel_for(n, threads, [&](int64_t i) {
        const float* r = rays + 8 * i;
        V3<double> o{r[0], r[1], r[2]}, d{r[4], r[5], r[6]};
        double bt = r[7], bu = 0, bv = 0;
        int32_t bid = -1;
        for (int32_t k = 0; k < s->n_tris; ++k) {
            double t, u, v;
            if (hit_d(o, d, tri_at(s, k), (double)r[3], (double)r[7], t, u, v)) {
                if (bid < 0 || t < bt || (t == bt && k < bid)) { bt = t; bu = u; bv = v; bid = k; }
            }
        }
        double* out = hits + 4 * i;
        out[0] = bid >= 0 ? bt : 0.0;
        out[1] = bu;
        out[2] = bv;
        out[3] = (double)bid;
    });
}

}  // extern "C"

// Renders n pixels, pixel_of(k) for k in [0, n), writing pixel k's mean to
// out_of(k)[0..2]; stats as orc_render.
template <class PixelOf, class OutOf>
static void render_pixel_set(const orc_scene* s, int precision, int32_t spp, int32_t spp_offset, int32_t max_depth,
                             int32_t rr_depth, uint64_t seed, int threads, int64_t n, PixelOf pixel_of,
                             OutOf out_of, const CacheConst& cache, double* stats) {
    static const Lut lut;
    std::vector<double> cdf((size_t)std::max(s->n_lights, 1));
    double acc = 0;
    for (int i = 0; i < s->n_lights; ++i) {
        acc += (double)s->lights[i].pmf;
        cdf[(size_t)i] = (i + 1 == s->n_lights) ? 1.0 : (double)(float)acc;
    }
    std::vector<double> st((size_t)n * 3, 0.0);
    parallel_for(n, threads, [&](int64_t k) {
        uint32_t pixel = pixel_of(k);
        double sum[3] = {0, 0, 0};
        double* sk = &st[3 * (size_t)k];
        if (precision == 64)
            render_pixel<double>(s, lut, cdf, spp, spp_offset, max_depth, rr_depth, seed, pixel, sum, sk, cache);
        else
            render_pixel<float>(s, lut, cdf, spp, spp_offset, max_depth, rr_depth, seed, pixel, sum, sk, cache);
        float* o = out_of(k);
        for (int c = 0; c < 3; ++c) o[c] = (float)(sum[c] / spp);
    });
    if (stats) {
        stats[0] = stats[1] = stats[2] = 0;
        for (int64_t k = 0; k < n; ++k)
            for (int c = 0; c < 3; ++c) stats[c] += st[3 * (size_t)k + c];
    }
}

extern "C" {

int orc_render_pixels(const orc_scene* s, int precision, int32_t spp, int32_t spp_offset, int32_t max_depth,
                      int32_t rr_depth, uint64_t seed, int threads, const uint32_t* pixels, int64_t n, float* out,
                      double* stats) {
    if (!s || (n > 0 && (!pixels || !out)) || n < 0 || spp <= 0 || (precision != 32 && precision != 64)) return 1;
    const int64_t npix = (int64_t)s->cam.width * s->cam.height;
    for (int64_t k = 0; k < n; ++k)
        if ((int64_t)pixels[k] >= npix) return 1;
    CacheConst cache;
    cache.query_depth = -1;
    render_pixel_set(s, precision, spp, spp_offset, max_depth, rr_depth, seed, threads, n,
                     [&](int64_t k) { return pixels[k]; }, [&](int64_t k) { return out + 3 * k; }, cache, stats);
    return 0;
}

int orc_render_cached(const orc_scene* s, int precision, int32_t spp, int32_t spp_offset, int32_t max_depth,
                      int32_t rr_depth, uint64_t seed, int threads, int64_t pixel_begin, int64_t pixel_end,
                      int32_t query_depth, const float* cache_rgb, float* out, double* stats) {
    if (!s || !out || spp <= 0 || (precision != 32 && precision != 64)) return 1;
    CacheConst cache;
    cache.query_depth = cache_rgb ? query_depth : -1;
    if (cache_rgb)
        for (int c = 0; c < 3; ++c) cache.rgb[c] = cache_rgb[c];
    int64_t npix = (int64_t)s->cam.width * s->cam.height;
    pixel_begin = std::max<int64_t>(0, pixel_begin);
    pixel_end = std::min<int64_t>(npix, pixel_end);
    if (pixel_end <= pixel_begin) {
        if (stats) stats[0] = stats[1] = stats[2] = 0;
        return 0;
    }
    render_pixel_set(s, precision, spp, spp_offset, max_depth, rr_depth, seed, threads, pixel_end - pixel_begin,
                     [&](int64_t k) { return (uint32_t)(pixel_begin + k); },
                     [&](int64_t k) { return out + 3 * (size_t)(pixel_begin + k); }, cache, stats);
    return 0;
}

}  // extern "C"
