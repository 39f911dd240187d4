// device.cuh — the scene as the device sees it, and the traversal routine
// shared by every kernel that casts rays (render wavefront, aqua_trace,
// batched rendering).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "aq_math.h"
#include "bvh.h"

namespace aq {

struct DevMaterial {
    float4 a;  // base colour rgb (linear), texture index (int bits, -1 none)
    float4 b;  // metallic, roughness, specular, 0
};
struct DevLight {
    float4 p0;  // xyz, type (int bits)
    float4 e1;  // xyz, area
    float4 e2;  // xyz, selection pmf
    float4 le;  // radiance (quad, triangle) or intensity (point), cdf
};
struct DevTexture {
    uint32_t offset;  // first texel in the texel pool
    int32_t w, h;
    int32_t pad;
};
struct DevCamera {
    float pos[3], right[3], up[3], back[3];
    float tan_half, aspect, lens_radius, focal;
    int32_t width, height;
};
struct DevScene {
    const float4* __restrict__ nodes;  // 8 words per four-wide node, or 4 per quantized node (bvh.h)
    const float4* __restrict__ tris;   // 3 words per triangle, leaf order
    const float2* __restrict__ uvs;    // 3 per triangle, leaf order
    const DevMaterial* __restrict__ mats;
    const DevLight* __restrict__ lights;
    const DevTexture* __restrict__ texs;
    const uint32_t* __restrict__ texels;  // RGBA8, sRGB
    const float4* __restrict__ nrm;    // 3 vertex normals per triangle (xyz, 0), leaf order; null = flat
    // 2 words per material: (specular_tint, sheen, sheen_tint, clearcoat),
    // (clearcoat_roughness, transmission, ior, 0); null when no material
    // sets any of those lobes (the base-model kernels run then).
    const float4* __restrict__ mext;
    int32_t n_nodes, n_tris, n_mats, n_lights, n_texs;
    int32_t qbvh;  // 1: `nodes` holds quantized 64-byte nodes
    float env[3];
    DevCamera cam;
};

// Result of a traversal: leaf-order triangle index (or -1), its scene index,
// distance and barycentrics.
struct TraceResult {
    float t, u, v;
    int32_t tri;
    int32_t id;
};

#if defined(__CUDACC__)

template <class T>
__device__ __forceinline__ T ldg_(const T* p) { return __ldg(p); }

// Programmatic dependent launch: wait until the kernel this one was chained
// to (launched with programmatic stream serialization) has completed and
// its writes are visible. Returns at once for a kernel launched normally.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
// Lets the kernel chained after this one be scheduled once every block of
// this grid has passed this point (its blocks then take SM slots as this
// grid's blocks exit, and wait in grid_dep_wait). No effect without a
// chained kernel.
__device__ __forceinline__ void grid_dep_launch() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

// Two consecutive 16-byte words in one 256-bit load through the read-only
// (non-coherent) path (sm_100 and later); p must be 32-byte aligned. Only
// for data that nothing writes during the render (scene nodes): kernels
// chained by programmatic dependent launch may begin before their
// predecessor has finished, and the non-coherent path is outside what
// griddepcontrol.wait makes visible, so they read what earlier kernels of
// the chain wrote through coherent loads (plain or __ldcg).
__device__ __forceinline__ void ldg2x4(const float4* p, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

constexpr int kStackSize = kBvhStackSize;  // the builder checks its trees fit
constexpr int32_t kTraversalDone = (int32_t)0x80000000;

// One compare-exchange of the child-ordering network: (ta, ca) gets the
// nearer entry, ties keep their order.
__device__ __forceinline__ void order2(float& ta, int32_t& ca, float& tb, int32_t& cb) {
    const bool sw = tb < ta;
    const float t = sw ? tb : ta;
    const int32_t c = sw ? cb : ca;
    tb = sw ? ta : tb;
    cb = sw ? ca : cb;
    ta = t;
    ca = c;
}

// Visits four-wide node `node`: tests its four child boxes (slab_entry, far
// limit tfar), orders the hit children by entry distance (a five-comparator
// sorting network), pushes all but the nearest, farthest first, and returns
// the nearest. With no box hit it returns the top of the stack, or
// kTraversalDone when the stack is empty. The node (128-byte aligned) comes
// in three 256-bit loads and one 128-bit load (the counts word is not read):
// scattered lanes cost the L1 one request per load instruction, so fewer,
// wider loads relieve it.
__device__ __forceinline__ int32_t visit_wide(const DevScene& S, int32_t node, const RayPre& rp, float tfar,
                                              int32_t* stack, int& sp) {
    const float4* np = S.nodes + 8 * (size_t)node;
    float4 lx, hx, ly, hy, lz, hz;
    ldg2x4(np, lx, hx);
    ldg2x4(np + 2, ly, hy);
    ldg2x4(np + 4, lz, hz);
    const int4 ch = ldg_(reinterpret_cast<const int4*>(np + 6));
    float t0 = slab_entry(lx.x, hx.x, ly.x, hy.x, lz.x, hz.x, rp, tfar);
    float t1 = slab_entry(lx.y, hx.y, ly.y, hy.y, lz.y, hz.y, rp, tfar);
    float t2 = slab_entry(lx.z, hx.z, ly.z, hy.z, lz.z, hz.z, rp, tfar);
    float t3 = slab_entry(lx.w, hx.w, ly.w, hy.w, lz.w, hz.w, rp, tfar);
    int32_t c0 = ch.x, c1 = ch.y, c2 = ch.z, c3 = ch.w;
    order2(t0, c0, t1, c1);
    order2(t2, c2, t3, c3);
    order2(t0, c0, t2, c2);
    order2(t1, c1, t3, c3);
    order2(t1, c1, t2, c2);
    if (t3 != INFINITY) stack[sp++] = c3;
    if (t2 != INFINITY) stack[sp++] = c2;
    if (t1 != INFINITY) stack[sp++] = c1;
    if (t0 != INFINITY) return c0;
    return sp > 0 ? stack[--sp] : kTraversalDone;
}

// Plane of child byte k of a quantized word: fmaf(q, scale, origin), the
// byte turned into a float exactly by placing it under the exponent of 2^23
// (one byte permute and one subtraction).
__device__ __forceinline__ float qplane(uint32_t word, int k, float scale, float origin) {
    // result bytes: word byte k, zero, zero, 0x4B  ->  2^23 + q
    const float q = __uint_as_float(__byte_perm(word, 0x4B000000u, 0x7540u | (uint32_t)k)) - 8388608.0f;
    return fmaf(q, scale, origin);
}

// visit_wide on a quantized 64-byte node (two 256-bit loads): the child
// planes are decoded (bvh.h) and tested with the same slab_entry; empty
// slots (link ~0) are skipped. Ordering, pushes and the result are those of
// visit_wide.
__device__ __forceinline__ int32_t visit_quantized(const DevScene& S, int32_t node, const RayPre& rp, float tfar,
                                                   int32_t* stack, int& sp) {
    const float4* np = S.nodes + 4 * (size_t)node;
    float4 w0, w1, w2, w3;
    ldg2x4(np, w0, w1);
    ldg2x4(np + 2, w2, w3);
    const uint32_t ex = __float_as_uint(w0.w);
    const float sx = __uint_as_float((ex & 0xffu) << 23), sy = __uint_as_float(((ex >> 8) & 0xffu) << 23),
                sz = __uint_as_float(((ex >> 16) & 0xffu) << 23);
    const uint32_t lx = __float_as_uint(w2.x), hx = __float_as_uint(w2.y), ly = __float_as_uint(w2.z),
                   hy = __float_as_uint(w2.w), lz = __float_as_uint(w3.x), hz = __float_as_uint(w3.y);
    int32_t c0 = __float_as_int(w1.x), c1 = __float_as_int(w1.y), c2 = __float_as_int(w1.z),
            c3 = __float_as_int(w1.w);
    float t[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
        t[k] = slab_entry(qplane(lx, k, sx, w0.x), qplane(hx, k, sx, w0.x), qplane(ly, k, sy, w0.y),
                          qplane(hy, k, sy, w0.y), qplane(lz, k, sz, w0.z), qplane(hz, k, sz, w0.z), rp, tfar);
    float t0 = c0 == ~0 ? INFINITY : t[0], t1 = c1 == ~0 ? INFINITY : t[1], t2 = c2 == ~0 ? INFINITY : t[2],
          t3 = c3 == ~0 ? INFINITY : t[3];
    order2(t0, c0, t1, c1);
    order2(t2, c2, t3, c3);
    order2(t0, c0, t2, c2);
    order2(t1, c1, t3, c3);
    order2(t1, c1, t2, c2);
    if (t3 != INFINITY) stack[sp++] = c3;
    if (t2 != INFINITY) stack[sp++] = c2;
    if (t1 != INFINITY) stack[sp++] = c1;
    if (t0 != INFINITY) return c0;
    return sp > 0 ? stack[--sp] : kTraversalDone;
}

// Node formats a walk is compiled for: full-precision only, or either
// (the scene's, a warp-uniform branch). Kernels whose instruction cache is
// tight (the batch kernel) take the full-precision walk alone unless one of
// their scenes holds quantized nodes.
enum { kNodesFull = 0, kNodesAny = 1 };

// One node visit in the scene's node format.
template <int NODES = kNodesAny>
__device__ __forceinline__ int32_t visit_node(const DevScene& S, int32_t node, const RayPre& rp, float tfar,
                                              int32_t* stack, int& sp) {
    if (NODES == kNodesFull) return visit_wide(S, node, rp, tfar, stack, sp);
    return S.qbvh ? visit_quantized(S, node, rp, tfar, stack, sp) : visit_wide(S, node, rp, tfar, stack, sp);
}

// Stack-based traversal of the four-wide BVH (nearest child first, the other
// hit children pushed farthest first). ANY: stop at the first hit in (tmin,
// tmax). Otherwise the result is the lexicographic minimum (t, scene index)
// over all triangles hit: boxes are tested conservatively (slab_entry), a
// child is skipped only when its entry distance exceeds the best t, so the
// answer does not depend on visit order.
// COUNT: add inner-node visits and triangle tests to the counters.
template <bool ANY, bool COUNT>
__device__ __forceinline__ TraceResult traverse(const DevScene& S, v3 o, v3 d, float tmin, float tmax,
                                                uint32_t& n_nodes, uint32_t& n_tris) {
    RayPre rp;
    rp.o = o;
    rp.invd = mk(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
    rp.tmin = tmin;
    rp.tmax = tmax;
    RayShear sh = make_shear(o, d);
    TraceResult r;
    r.t = tmax; r.u = 0.0f; r.v = 0.0f; r.tri = -1; r.id = 0x7fffffff;
    int32_t stack[kStackSize];
    int sp = 0;
    int32_t node = 0;
    while (true) {
        while (node >= 0) {
            if (COUNT) ++n_nodes;
            node = visit_node(S, node, rp, r.t, stack, sp);
        }
        if (node == kTraversalDone) return r;
        // Leaf.
        int32_t code = ~node;
        int32_t first = code >> 3, cnt = code & 7;
        for (int k = 0; k < cnt; ++k) {
            const float4* tp = S.tris + 3 * (size_t)(first + k);
            float4 a = ldg_(tp), b = ldg_(tp + 1), c = ldg_(tp + 2);
            if (COUNT) ++n_tris;
            TriHit h = intersect_tri(sh, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), mk(c.x, c.y, c.z), tmin, tmax);
            if (h.hit) {
                int32_t id = __float_as_int(a.w);
                if (ANY) {
                    r.t = h.t; r.tri = first + k; r.id = id;
                    return r;
                }
                if (h.t < r.t || (h.t == r.t && id < r.id)) {
                    r.t = h.t; r.u = h.u; r.v = h.v; r.tri = first + k; r.id = id;
                }
            }
        }
        if (sp == 0) return r;
        node = stack[--sp];
    }
}

// Traversal with postponed leaves (Aila & Laine 2009, "Understanding the
// Efficiency of Ray Traversal on GPUs"): a lane that reaches a leaf parks it
// and keeps walking inner nodes until every lane of the warp still walking
// holds a leaf (warp vote), then all test triangles together. Boxes, culling
// and triangle tests are those of traverse(), so the result (the minimum
// (t, scene index) over all triangles hit, or any hit) is identical; only
// the order of visits, and thus the work counts, differ. `any` (stop at the
// first hit) is a run-time flag, so a kernel that traces both kinds of ray
// from one call site holds one inlined copy of the walk.
template <int NODES = kNodesAny>
__device__ __forceinline__ TraceResult traverse_fast(const DevScene& S, v3 o, v3 d, float tmin, float tmax,
                                                     bool any) {
    RayPre rp;
    rp.o = o;
    rp.invd = mk(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
    rp.tmin = tmin;
    rp.tmax = tmax;
    RayShear sh = make_shear(o, d);
    TraceResult r;
    r.t = tmax; r.u = 0.0f; r.v = 0.0f; r.tri = -1; r.id = 0x7fffffff;
    int32_t stack[kStackSize];
    int sp = 0;
    int32_t node = 0, leaf = 0;
    while (true) {
        while (node >= 0) {
            node = visit_node<NODES>(S, node, rp, r.t, stack, sp);
            if (node < 0 && node != kTraversalDone && leaf == 0) {
                leaf = node;
                node = sp > 0 ? stack[--sp] : kTraversalDone;
            }
            if (!__any_sync(__activemask(), leaf == 0)) break;
        }
        while (leaf < 0) {
            int32_t code = ~leaf;
            int32_t first = code >> 3, cnt = code & 7;
            for (int k = 0; k < cnt; ++k) {
                const float4* tp = S.tris + 3 * (size_t)(first + k);
                float4 a = ldg_(tp), b = ldg_(tp + 1), c = ldg_(tp + 2);
                TriHit h = intersect_tri(sh, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), mk(c.x, c.y, c.z), tmin, tmax);
                if (h.hit) {
                    int32_t id = __float_as_int(a.w);
                    if (any) {
                        r.t = h.t; r.tri = first + k; r.id = id;
                        return r;
                    }
                    if (h.t < r.t || (h.t == r.t && id < r.id)) {
                        r.t = h.t; r.u = h.u; r.v = h.v; r.tri = first + k; r.id = id;
                    }
                }
            }
            leaf = 0;
            if (node < 0 && node != kTraversalDone) {
                leaf = node;
                node = sp > 0 ? stack[--sp] : kTraversalDone;
            }
        }
        if (node == kTraversalDone) return r;
    }
}

// Persistent traversal of a queue of n rays with ray replacement (Aila &
// Laine 2009, sec. 4: "replacing terminated rays"): each lane holds its own
// ray; once at least kRefillLanes lanes of the warp have finished theirs (or
// all have), the idle lanes take the next rays from *cursor together (one
// atomic per warp). Between refills every lane runs rounds of
// traverse_fast: walk inner nodes with postponed leaves, then test the
// parked leaves. Boxes, culling and triangle tests are those of traverse(),
// so every ray's result is the one traverse_fast returns.
//   load(i, o, d, tmin, tmax) -> uint32_t tag: fetches ray i of the queue;
//   done(tag, r): called once per ray, by the lanes finishing in the same
//                 round together (warp collectives inside are allowed).
constexpr int kRefillLanes = 16;

// Kinds of queue: closest hits, any hits, or both mixed (the load callback
// then sets `any` per ray: load(i, o, d, tmin, tmax, any)).
enum { kQueueClosest = 0, kQueueAny = 1, kQueueMixed = 2 };

template <int KIND, class Load, class Done>
__device__ __forceinline__ void traverse_queue_kind(const DevScene& S, uint32_t n, uint32_t* cursor, Load load,
                                                    Done done) {
    const unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    RayPre rp;
    RayShear sh;
    TraceResult r;
    int32_t stack[kStackSize];
    int sp = 0;
    int32_t node = kTraversalDone, leaf = 0;
    uint32_t tag = 0;
    bool have = false, drained = false, any = KIND == kQueueAny;
    while (true) {
        const unsigned idle = __ballot_sync(kFull, !have);
        if (!drained && idle != 0u && (__popc(idle) >= kRefillLanes || idle == kFull)) {
            const int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(cursor, (uint32_t)__popc(idle));
            base = __shfl_sync(kFull, base, leader);
            if (base + (uint32_t)__popc(idle) >= n) drained = true;
            if (!have) {
                const uint32_t i = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (i < n) {
                    v3 o, d;
                    float tmin, tmax;
                    if constexpr (KIND == kQueueMixed) tag = load(i, o, d, tmin, tmax, any);
                    else tag = load(i, o, d, tmin, tmax);
                    rp.o = o;
                    rp.invd = mk(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
                    rp.tmin = tmin;
                    rp.tmax = tmax;
                    sh = make_shear(o, d);
                    r.t = tmax; r.u = 0.0f; r.v = 0.0f; r.tri = -1; r.id = 0x7fffffff;
                    sp = 0;
                    node = 0;
                    leaf = 0;
                    have = true;
                }
            }
        }
        if (!__any_sync(kFull, have)) break;
        if (!have) continue;
        // One round of traverse_fast.
        while (node >= 0) {
            node = visit_node(S, node, rp, r.t, stack, sp);
            if (node < 0 && node != kTraversalDone && leaf == 0) {
                leaf = node;
                node = sp > 0 ? stack[--sp] : kTraversalDone;
            }
            if (!__any_sync(__activemask(), leaf == 0)) break;
        }
        while (leaf < 0) {
            int32_t code = ~leaf;
            int32_t first = code >> 3, cnt = code & 7;
            bool stop = false;
            for (int k = 0; k < cnt; ++k) {
                const float4* tp = S.tris + 3 * (size_t)(first + k);
                float4 a = ldg_(tp), b = ldg_(tp + 1), c = ldg_(tp + 2);
                TriHit h = intersect_tri(sh, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), mk(c.x, c.y, c.z), rp.tmin,
                                         rp.tmax);
                if (h.hit) {
                    int32_t id = __float_as_int(a.w);
                    if (KIND == kQueueAny || (KIND == kQueueMixed && any)) {
                        r.t = h.t; r.tri = first + k; r.id = id;
                        stop = true;
                        break;
                    }
                    if (h.t < r.t || (h.t == r.t && id < r.id)) {
                        r.t = h.t; r.u = h.u; r.v = h.v; r.tri = first + k; r.id = id;
                    }
                }
            }
            leaf = 0;
            if (stop) {
                node = kTraversalDone;
                break;
            }
            if (node < 0 && node != kTraversalDone) {
                leaf = node;
                node = sp > 0 ? stack[--sp] : kTraversalDone;
            }
        }
        if (node == kTraversalDone) {
            done(tag, r);
            have = false;
        }
    }
}

template <bool ANY, class Load, class Done>
__device__ __forceinline__ void traverse_queue(const DevScene& S, uint32_t n, uint32_t* cursor, Load load,
                                               Done done) {
    traverse_queue_kind<ANY ? kQueueAny : kQueueClosest>(S, n, cursor, load, done);
}

// Warp-aggregated append: lanes with pred set get consecutive slots of *ctr.
__device__ __forceinline__ uint32_t warp_append(uint32_t* ctr, bool pred) {
    unsigned mask = __ballot_sync(__activemask(), pred);
    if (!pred) return 0;
    int lane = threadIdx.x & 31;
    int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(ctr, (uint32_t)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

#endif  // __CUDACC__

}  // namespace aq
