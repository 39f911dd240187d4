// render.cu — the wavefront path tracer.
//
// One iteration = three launches over compacted queues:
//   k_trace_ext   closest hit for every active path; optionally bins the
//                 path into a per-material queue (warp-aggregated atomics)
//   k_shade       emission (MIS), next-event estimation (one shadow ray),
//                 BSDF sampling, Russian roulette; a finished path is replaced
//                 in place by the slot's next camera sample (ray generation)
//   k_shadow      any-hit test of the shadow queue, film += unoccluded NEE
// (In the cache mode k_trace_fused walks an iteration's extension rays and
// the previous iteration's shadow rays in one launch, two launches per
// iteration.) Renders keep about 2^24 paths in flight (sample replicas).
// Path slot s owns pixels s, s + S, s + 2S, ... and runs their samples in
// order, so film updates need no atomics and the image does not depend on
// the launch shape, the slot count or the material sort.
//
// Light transport follows the reference's data semantics: camera
// `Perspective` (scenes/cbox.json:516-543), `Principled` Lambert + GGX
// (scenes/cbox.json:3-62), `Point` lights (scenes/cbox.json:544-561), quad
// area lights (CornellBox-Original.mtl:80-87), `max_depth`
// (scenes/integrator.json:5).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "internal.h"
#include "shading.cuh"

namespace aq {

struct WaveParams {
    uint64_t seed;
    int32_t spp, spp_offset, max_depth, rr_depth;
    uint32_t slots, pixels;
    uint32_t nb;  // material buckets incl. the miss bucket (0 = unsorted)
    // Radiance cache (NRC mode only).
    int32_t query_depth;       // bounce at which non-training paths query the cache (-1: by path spread)
    float spread_c;            // path-spread mode: query once spread > spread_c x a0
    uint32_t train_thresh;     // path trains when its 24-bit hash < this
    uint32_t max_train_paths;  // capacity of the per-training-path accumulators
    uint32_t max_records;      // capacity of the training-vertex records
    int32_t train_span;        // reflections a target covers: max_depth - query_depth
    int32_t record_depth;      // training paths record their vertices at bounces below this
    int32_t train_depth;       // bounce limit of training paths: record_depth + train_span
    int32_t visualize;         // 1 = the image is the cache seen at the first hit
    // Sample replicas (0 or 1 = off). With K > 1 there are K slots per pixel:
    // slot s = r * pixels + p runs samples r, r + K, r + 2K, ... of pixel p
    // into film copy r; the copies are summed in order r = 0..K-1.
    uint32_t replicas;
    // Row subset (row_step > 1): film pixel p is image pixel
    // (row_begin + (p / width) * row_step) * width + p % width.
    uint32_t row_begin, row_step, width;
};

struct WavePtrs {
    float4* ray_o;
    float4* ray_d;
    float4* hit;
    float4* tp;
    uint4* pst;
    uint32_t* q_in;
    uint32_t* q_out;
    uint32_t* bucket;
    float4* sh_o;
    float4* sh_d;
    float4* sh_c;
    float4* film;
    uint32_t* counters;
    unsigned long long* stats;
    // Radiance cache (NRC mode only).
    float4* q_pix;    // per query: (pixel bits, throughput rgb)
    float* q_raw;     // per query: 16 raw vertex features
    float4* rec;      // per training vertex: 6 words (raw 16, throughput 3, radiance-before 3, path id)
    float4* ltrain;   // per training path: radiance gathered so far
    float2* spread;   // per slot: (sum of sqrt spread terms, a0) of the path (path-spread mode)
    float4* lsnap;    // per training path and bounce k < train_depth: radiance
                      // gathered before bounce k reflected anything (x < 0: unset)
};

// Counters of the cache mode (after the material buckets).
enum { kCntQuery = 3, kCntRecord = 4, kCntTrainPath = 5 };
// Dynamic-fetch cursors of the two traversal kernels; each kernel clears
// the other's for the next launch (the shading kernel clears the trace
// cursor too, for the fused pipeline). The fused pipeline's shadow queue
// alternates between kCntShadow and kCntShadow1 with the iteration.
enum { kCntFetchTrace = 6, kCntFetchShadow = 7, kCntShadow1 = 8 };

// ---------------------------------------------------------------- helpers

__device__ __forceinline__ uint32_t slot_work(const WaveParams& P, uint32_t s) {
    if (P.replicas > 1) {
        uint32_t r = s / P.pixels;
        return r < (uint32_t)P.spp ? ((uint32_t)P.spp - r + P.replicas - 1) / P.replicas : 0u;
    }
    if (s >= P.pixels) return 0;
    uint32_t npix = (P.pixels - s + P.slots - 1) / P.slots;
    return npix * (uint32_t)P.spp;
}

// Image pixel of film pixel p (they differ for row-subset renders); the
// image pixel names the camera ray and the random-number stream.
__device__ __forceinline__ uint32_t image_pixel(const WaveParams& P, uint32_t p) {
    if (P.row_step <= 1) return p;
    uint32_t r = p / P.width;
    return (P.row_begin + r * P.row_step) * P.width + (p - r * P.width);
}

// Pixel (the film pixel of the stream), sample index and film entry of
// work item j of slot s.
struct PathId {
    uint32_t pixel, sample, film;
};
__device__ __forceinline__ PathId path_id(const WaveParams& P, uint32_t s, uint32_t j) {
    PathId id;
    if (P.replicas > 1) {
        uint32_t r = s / P.pixels;
        id.pixel = s - r * P.pixels;
        id.sample = (uint32_t)P.spp_offset + r + j * P.replicas;
        id.film = s;
    } else {
        id.pixel = s + (j / (uint32_t)P.spp) * P.slots;
        id.sample = (uint32_t)P.spp_offset + j % (uint32_t)P.spp;
        id.film = id.pixel;
    }
    return id;
}


// Starts work item j of slot s (pixel, sample), writing its camera ray. The
// path state's last word is depth (bits 0..7) | (training path id + 1) << 8;
// the id is 0 outside the cache mode.
template <bool NRC = false>
__device__ __forceinline__ bool start_path(const DevScene& S, const WaveParams& P, const WavePtrs& W,
                                           uint32_t s, uint32_t j) {
    if (j >= slot_work(P, s)) return false;
    PathId pid = path_id(P, s, j);
    uint32_t pixel = image_pixel(P, pid.pixel), sample = pid.sample;
    uint64_t st = path_rng_state(P.seed, pixel, sample), inc = pixel_inc(pixel);
    float u0 = draw(st, inc), u1 = draw(st, inc), u2 = draw(st, inc), u3 = draw(st, inc);
    v3 o, d;
    camera_ray(S.cam, pixel, u0, u1, u2, u3, o, d);
    W.ray_o[s] = make_float4(o.x, o.y, o.z, 0.0f);
    W.ray_d[s] = make_float4(d.x, d.y, d.z, INFINITY);
    W.tp[s] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    uint32_t tag = 0;
    if (NRC) {
        // Training paths: a seeded hash of (pixel, sample) picks about the
        // fraction the host asked for; they trace unbiased full paths.
        uint32_t h = (uint32_t)(splitmix64(P.seed * 0x9E3779B97F4A7C15ULL ^ ((uint64_t)pixel << 24) ^ sample) >> 40);
        if (h < P.train_thresh) {
            uint32_t id = atomicAdd(&W.counters[kCntTrainPath], 1u);
            if (id < P.max_train_paths) {
                W.ltrain[id] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                float4* snap = W.lsnap + (size_t)id * (size_t)P.train_depth;
                for (int k = 0; k < P.train_depth; ++k) snap[k] = make_float4(-1.0f, 0.0f, 0.0f, 0.0f);
                tag = (id + 1u) << 8;
            }
        }
    }
    W.pst[s] = make_uint4((uint32_t)st, (uint32_t)(st >> 32), j, tag);
    return true;
}

// Block-aggregated append: every thread of the block calls it together;
// threads with pred set get consecutive entries of *ctr, with one atomic per
// block instead of one per warp. s_warp: (warps + 1) shared words.
__device__ __forceinline__ uint32_t block_append(uint32_t* ctr, bool pred, uint32_t* s_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const unsigned m = __ballot_sync(0xffffffffu, pred);
    if (lane == 0) s_warp[warp] = (uint32_t)__popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t acc = 0;
        for (int w = 0; w < nw; ++w) {
            const uint32_t c = s_warp[w];
            s_warp[w] = acc;
            acc += c;
        }
        s_warp[nw] = acc ? atomicAdd(ctr, acc) : 0u;
    }
    __syncthreads();
    const uint32_t k = s_warp[nw] + s_warp[warp] + (uint32_t)__popc(m & ((1u << lane) - 1u));
    __syncthreads();  // s_warp is reused by the next call
    return k;
}

__device__ __forceinline__ void film_add(float4* film, uint32_t pixel, v3 c) {
    float4 f = film[pixel];
    f.x += c.x; f.y += c.y; f.z += c.z;
    film[pixel] = f;
}

// ---------------------------------------------------------------- kernels
template <bool NRC = false>
__global__ void k_raygen(DevScene S, WaveParams P, WavePtrs W) {
    uint32_t n = P.replicas > 1 ? P.slots : min(P.slots, P.pixels);
    uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid == 0) {
        W.counters[kCntQ0] = n;
        W.counters[kCntQ1] = 0;
        W.counters[kCntShadow] = 0;
    }
    for (uint32_t s = tid; s < n; s += gridDim.x * blockDim.x) {
        start_path<NRC>(S, P, W, s, 0);
        W.q_in[s] = s;
    }
}

// Raw cache features of a shading point (position, outgoing direction,
// normal, roughness, diffuse albedo, specular F0).
__device__ __forceinline__ void nrc_raw(float* o, v3 p, v3 wo, v3 n, float rough, v3 kd, v3 ks) {
    o[0] = p.x; o[1] = p.y; o[2] = p.z;
    o[3] = wo.x; o[4] = wo.y; o[5] = wo.z;
    o[6] = n.x; o[7] = n.y; o[8] = n.z;
    o[9] = rough;
    o[10] = kd.x; o[11] = kd.y; o[12] = kd.z;
    o[13] = ks.x; o[14] = ks.y; o[15] = ks.z;
}

__device__ __forceinline__ void ltrain_add(float4* L, uint32_t id, v3 c) {
    float4 v = L[id];
    v.x += c.x; v.y += c.y; v.z += c.z;
    L[id] = v;
}

template <bool SORTED, bool COUNT>
__global__ void __launch_bounds__(128) k_trace_ext(DevScene S, WaveParams P, WavePtrs W, uint32_t cnt_in,
                                                   uint32_t cnt_out) {
    grid_dep_wait();
    grid_dep_launch();
    uint32_t n = W.counters[cnt_in];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        W.counters[cnt_out] = 0;
        W.counters[kCntShadow] = 0;
        W.counters[kCntFetchShadow] = 0;
    }
    const int lane_id = threadIdx.x & 31;
    uint32_t nodes = 0, tris = 0;
    // Hit record and material bucket of slot s (lanes finishing together
    // bin together).
    auto finish = [&](uint32_t s, const TraceResult& r) {
        W.hit[s] = make_float4(r.t, r.u, r.v, __int_as_float(r.tri));
        if (SORTED) {
            uint32_t b = r.tri < 0 ? P.nb - 1
                                   : ((uint32_t)__float_as_int(ldg_(S.tris + 3 * (size_t)r.tri + 1).w) & 0xffffu);
            unsigned mask = __match_any_sync(__activemask(), b);
            int lane = threadIdx.x & 31, leader = __ffs(mask) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(&W.counters[kCntBucket0 + b], (uint32_t)__popc(mask));
            base = __shfl_sync(mask, base, leader);
            uint32_t pos = base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
            W.bucket[(size_t)b * P.slots + pos] = s;
        }
    };
    if (!COUNT) {
        // Persistent lanes with ray replacement.
        traverse_queue<false>(
            S, n, &W.counters[kCntFetchTrace],
            [&](uint32_t i, v3& o, v3& d, float& tmin, float& tmax) -> uint32_t {
                uint32_t s = W.q_in[i];
                float4 ro = W.ray_o[s], rd = W.ray_d[s];
                o = f3(ro);
                d = f3(rd);
                tmin = ro.w;
                tmax = rd.w;
                return s;
            },
            finish);
    } else {
        // Canonical counting walk; each warp takes the next 32 rays.
        while (true) {
            uint32_t base = 0;
            if (lane_id == 0) base = atomicAdd(&W.counters[kCntFetchTrace], 32u);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= n) break;
            const uint32_t i = base + (uint32_t)lane_id;
            if (i >= n) continue;
            uint32_t s = W.q_in[i];
            float4 ro = W.ray_o[s], rd = W.ray_d[s];
            finish(s, traverse<false, true>(S, f3(ro), f3(rd), ro.w, rd.w, nodes, tris));
        }
    }
    if (COUNT) {
        for (int o = 16; o > 0; o >>= 1) {
            nodes += __shfl_down_sync(0xffffffffu, nodes, o);
            tris += __shfl_down_sync(0xffffffffu, tris, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&W.stats[kStatNodes], (unsigned long long)nodes);
            atomicAdd(&W.stats[kStatTris], (unsigned long long)tris);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&W.stats[kStatExt], (unsigned long long)n);
}

// NRC: paths that are not training paths stop at bounce P.query_depth and
// queue a cache query (pixel, throughput, raw features); training paths run
// on and record every bounce (raw features, throughput, radiance gathered
// so far) so that the radiance leaving each of their vertices becomes a
// training target once the path is complete.
template <bool SORTED, bool NRC = false, bool FULL = false>
__global__ void __launch_bounds__(128, 6) k_shade(DevScene S, WaveParams P, WavePtrs W, uint32_t cnt_in,
                                               uint32_t cnt_out, uint32_t cnt_sh) {
    __shared__ float lut[256];
    __shared__ uint32_t prefix[257];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        float c = (float)i / 255.0f;
        lut[i] = c <= 0.04045f ? c / 12.92f : powf((c + 0.055f) / 1.055f, 2.4f);
    }
    grid_dep_wait();
    grid_dep_launch();
    if (blockIdx.x == 0 && threadIdx.x == 0) W.counters[kCntFetchTrace] = 0;  // for the next traversal launch
    uint32_t n;
    if (SORTED) {
        if (threadIdx.x == 0) {
            uint32_t acc = 0;
            for (uint32_t b = 0; b < P.nb; ++b) {
                prefix[b] = acc;
                acc += W.counters[kCntBucket0 + b];
            }
            prefix[P.nb] = acc;
        }
        __syncthreads();
        n = prefix[P.nb];
    } else {
        __syncthreads();
        n = W.counters[cnt_in];
    }
    uint32_t* out_cnt = &W.counters[cnt_out];
    unsigned long long done_paths = 0;
    __shared__ uint32_t s_warp[5];
    // The whole block iterates together (the out-queue append is per block).
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {
        const uint32_t i = i0 + threadIdx.x;
        uint32_t s = 0;
        bool cont = false;
        if (i < n) {
        // With sorted queues the bucket is the material, so its parameters
        // load alongside the path state instead of after the triangle.
        float4 mat_a = make_float4(0.0f, 0.0f, 0.0f, 0.0f), mat_b = mat_a;
        if (SORTED) {
            uint32_t lo = 0, hi = P.nb - 1;
            while (lo < hi) {  // last bucket b with prefix[b] <= i
                uint32_t mid = (lo + hi + 1) >> 1;
                if (prefix[mid] <= i) lo = mid;
                else hi = mid - 1;
            }
            s = W.bucket[(size_t)lo * P.slots + (i - prefix[lo])];
            if (lo + 1 < P.nb) {  // the last bucket holds the misses
                const float4* mp = reinterpret_cast<const float4*>(S.mats + lo);
                mat_a = ldg_(mp);
                mat_b = ldg_(mp + 1);
            }
        } else {
            s = W.q_in[i];
        }
        uint4 ps = W.pst[s];
        float4 tpv = W.tp[s];
        float4 h = W.hit[s];
        uint32_t j = ps.z, depth = ps.w & 0xffu, tag = ps.w & ~0xffu;
        const uint32_t train_id = (tag >> 8) - 1u;  // valid when tag != 0
        const PathId pid = path_id(P, s, j);
        const uint32_t pixel = pid.film;  // film entry owned by this slot
        uint64_t st = (uint64_t)ps.x | ((uint64_t)ps.y << 32), inc = pixel_inc(image_pixel(P, pid.pixel));
        v3 thr = f3(tpv);
        float pdf_b = tpv.w;
        int32_t tri = __float_as_int(h.w);
        if (tri < 0) {
            v3 e = mk(S.env[0], S.env[1], S.env[2]);
            if (e.x > 0.0f || e.y > 0.0f || e.z > 0.0f) {
                if (!NRC || (int)depth <= P.max_depth) film_add(W.film, pixel, thr * e);
                if (NRC && tag) ltrain_add(W.ltrain, train_id, thr * e);
            }
        } else {
            float4 rd = W.ray_d[s];
            const float4* tw = S.tris + 3 * (size_t)tri;
            float4 a = ldg_(tw), b = ldg_(tw + 1), c = ldg_(tw + 2);
            uint32_t info = (uint32_t)__float_as_int(b.w);
            v3 v0 = f3(a), e1 = f3(b) - v0, e2 = f3(c) - v0;
            v3 p = v0 + e1 * h.y + e2 * h.z;
            v3 ng = normalize(cross(e1, e2));
            v3 dir = f3(rd);
            v3 wo = -dir;
            int light = (int)(info >> 16) - 1;
            if (light >= 0) {
                DevLight L = S.lights[light];
                v3 nl = normalize(cross(f3(L.e1), f3(L.e2)));
                float cos_l = dot(nl, wo);
                if (cos_l > 0.0f) {
                    float w = 1.0f;
                    if (depth > 0 && pdf_b > 0.0f) {
                        float pl = L.e2.w * h.x * h.x / (L.e1.w * cos_l);
                        w = power_heuristic(pdf_b, pl);
                    }
                    // Past max_depth a training path gathers for its targets only:
                    // the image keeps the plain estimator's depth.
                    if (!(NRC && P.visualize) && (!NRC || (int)depth <= P.max_depth))
                        film_add(W.film, pixel, thr * f3(L.le) * w);
                    if (NRC && tag) ltrain_add(W.ltrain, train_id, thr * f3(L.le) * w);
                }
            }
            // Training paths run train_span bounces past the last vertex
            // they record, so every target covers the same reflections as
            // the path the cache replaces.
            const int depth_limit = (NRC && tag) ? P.train_depth : P.max_depth;
            if ((int)depth < depth_limit) {
                const bool front = dot(ng, wo) >= 0.0f;  // wo on the winding normal's side
                if (!front) ng = -ng;
                const v3 ns = shading_normal(S, tri, h.y, h.z, ng, wo);
                DevMaterial m;
                if (SORTED) {
                    m.a = mat_a;
                    m.b = mat_b;
                } else {
                    m = S.mats[info & 0xffffu];
                }
                v3 base = f3(m.a);
                int ti = __float_as_int(m.a.w);
                if (ti >= 0) {
                    const float2* uv = S.uvs + 3 * (size_t)tri;
                    float2 t0 = ldg_(uv), t1 = ldg_(uv + 1), t2 = ldg_(uv + 2);
                    float w0 = 1.0f - h.y - h.z;
                    float tu = t0.x * w0 + t1.x * h.y + t2.x * h.z;
                    float tv = t0.y * w0 + t1.y * h.y + t2.y * h.z;
                    base = base * tex_bilinear(S, ti, tu, tv, lut);
                }
                Bsdf B;
                if (FULL) {
                    const float4* xp = S.mext + 2 * (size_t)(info & 0xffffu);
                    const float4 x0 = ldg_(xp), x1 = ldg_(xp + 1);
                    B = make_bsdf_full(base, m.b.x, m.b.y, m.b.z, x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, front);
                } else {
                    B = make_bsdf(base, m.b.x, m.b.y, m.b.z);
                }
                bool queried = false;
                if (NRC) {
                    v3 kd = base * (1.0f - m.b.x);
                    bool query = (int)depth == P.query_depth;
                    if (P.query_depth < 0 && !tag) {
                        // Path spread (Mueller et al. 2021, sec. 5): a0 = t1^2 / (4 pi cos1)
                        // at the first vertex; later vertices add sqrt(t^2 / (pdf cos)); the
                        // path queries at vertex 2 or later once (sum)^2 > c a0.
                        const float cv = fmaxf(fabsf(dot(ns, wo)), 1e-6f);
                        float2 sp = depth == 0 ? make_float2(0.0f, h.x * h.x / (4.0f * kPi * cv)) : W.spread[s];
                        if (depth > 0) sp.x += sqrtf(h.x * h.x / (fmaxf(pdf_b, 1e-12f) * cv));
                        query = depth > 0 && sp.x * sp.x > P.spread_c * sp.y;
                        W.spread[s] = sp;
                    }
                    if (!tag && query) {
                        uint32_t k = warp_append(&W.counters[kCntQuery], true);
                        W.q_pix[k] = make_float4(__int_as_float((int)pixel), thr.x, thr.y, thr.z);
                        nrc_raw(W.q_raw + 16 * (size_t)k, p, wo, ns, m.b.y, kd, B.F0);
                        queried = true;
                    } else if (tag) {
                        float4 lb = W.ltrain[train_id];
                        W.lsnap[(size_t)train_id * (size_t)P.train_depth + depth] = lb;
                        uint32_t k = (int)depth < P.record_depth ? atomicAdd(&W.counters[kCntRecord], 1u) : 0xffffffffu;
                        if (k < P.max_records) {
                            float r[24];
                            nrc_raw(r, p, wo, ns, m.b.y, kd, B.F0);
                            r[16] = thr.x; r[17] = thr.y; r[18] = thr.z;
                            r[19] = lb.x; r[20] = lb.y; r[21] = lb.z;
                            r[22] = __int_as_float((int)train_id);
                            r[23] = __int_as_float((int)depth);
                            float4* dst = W.rec + 6 * (size_t)k;
#pragma unroll
                            for (int q = 0; q < 6; ++q)
                                dst[q] = make_float4(r[4 * q], r[4 * q + 1], r[4 * q + 2], r[4 * q + 3]);
                        }
                    }
                }
                v3 T, Bt;
                onb(ns, T, Bt);
                v3 wol = mk(dot(wo, T), dot(wo, Bt), dot(wo, ns));
                float u[kBounceDims];
#pragma unroll
                for (int k = 0; k < kBounceDims; ++k) u[k] = queried ? 0.0f : draw(st, inc);
                // Next-event estimation: one light, one point, one shadow ray.
                if (!queried && S.n_lights > 0 && wol.z > 0.0f) {
                    DevLight L = S.lights[pick_light(S, u[0])];
                    int ty = __float_as_int(L.p0.w);
                    float pmf = L.e2.w;
                    v3 contrib = mk(0, 0, 0), wi;
                    float dist = 0.0f;
                    bool below = false;  // light sample on the far side (glass lobe)
                    if (ty == AQUA_LIGHT_POINT) {
                        v3 dl = f3(L.p0) - p;
                        float d2 = dot(dl, dl);
                        dist = sqrtf(d2);
                        wi = dl * (1.0f / dist);
                        float cs = dot(wi, ns), cg = dot(wi, ng);
                        below = FULL && B.wglass > 0.0f && cs < 0.0f && cg < 0.0f;
                        if (((cs > 0.0f && cg > 0.0f) || below) && d2 > 0.0f) {
                            v3 wil = mk(dot(wi, T), dot(wi, Bt), cs);
                            contrib = thr * bsdf_eval_t<FULL>(B, wol, wil) * f3(L.le) *
                                      ((FULL ? fabsf(cs) : cs) / (d2 * pmf));
                        }
                    } else {
                        v3 le1 = f3(L.e1), le2 = f3(L.e2), xl;
                        if (ty == AQUA_LIGHT_QUAD) {
                            xl = f3(L.p0) + le1 * u[1] + le2 * u[2];
                        } else {
                            float su = sqrtf(u[1]);
                            xl = f3(L.p0) + le1 * (su * (1.0f - u[2])) + le2 * (su * u[2]);
                        }
                        v3 nl = normalize(cross(le1, le2));
                        v3 dl = xl - p;
                        float d2 = dot(dl, dl);
                        dist = sqrtf(d2);
                        wi = dl * (1.0f / dist);
                        float cl = -dot(wi, nl), cs = dot(wi, ns), cg = dot(wi, ng);
                        below = FULL && B.wglass > 0.0f && cs < 0.0f && cg < 0.0f;
                        if (cl > 0.0f && ((cs > 0.0f && cg > 0.0f) || below) && d2 > 0.0f) {
                            v3 wil = mk(dot(wi, T), dot(wi, Bt), cs);
                            float pl = pmf * d2 / (L.e1.w * cl);
                            float pb = bsdf_pdf_t<FULL>(B, wol, wil);
                            float w = power_heuristic(pl, pb);
                            contrib = thr * bsdf_eval_t<FULL>(B, wol, wil) * f3(L.le) *
                                      ((FULL ? fabsf(cs) : cs) * w / pl);
                        }
                    }
                    if (contrib.x > 0.0f || contrib.y > 0.0f || contrib.z > 0.0f) {
                        uint32_t k = warp_append(&W.counters[cnt_sh], true);
                        v3 so = offset_ray(p, below ? -ng : ng);
                        W.sh_o[k] = make_float4(so.x, so.y, so.z, __int_as_float((int)pixel));
                        W.sh_d[k] = make_float4(wi.x, wi.y, wi.z, dist * (1.0f - 1e-4f));
                        // w: 0, or the training path's id + 1 (negated: its
                        // targets only, the bounce lies past max_depth)
                        const int tid = NRC && tag ? ((int)depth < P.max_depth ? (int)(train_id + 1u)
                                                                                : -(int)(train_id + 1u))
                                                   : 0;
                        W.sh_c[k] = make_float4(contrib.x, contrib.y, contrib.z, __int_as_float(tid));
                    }
                }
                // BSDF sampling.
                v3 wil = bsdf_sample_t<FULL>(B, wol, u[3], u[4], u[5]);
                const bool through = FULL && wil.z < 0.0f;  // refracted by the glass lobe
                if (!queried && (wil.z > 0.0f || through) && wol.z > 0.0f) {
                    float pdf = bsdf_pdf_t<FULL>(B, wol, wil);
                    v3 f = bsdf_eval_t<FULL>(B, wol, wil);
                    if (pdf > 0.0f) {
                        thr = thr * f * ((FULL ? fabsf(wil.z) : wil.z) / pdf);
                        bool ok = maxc(thr) > 0.0f && isfinite(thr.x) && isfinite(thr.y) && isfinite(thr.z);
                        if (ok && (int)depth >= P.rr_depth) {
                            float q = fminf(1.0f, maxc(thr));
                            if (u[6] >= q) ok = false;
                            else thr = thr * (1.0f / q);
                        }
                        v3 wi = normalize(T * wil.x + Bt * wil.y + ns * wil.z);
                        if (through) {
                            if (!(dot(wi, ng) < 0.0f)) ok = false;  // refraction must cross the surface
                        } else if (S.nrm && !(dot(wi, ng) > 0.0f)) {
                            ok = false;  // below the geometric surface
                        }
                        if (ok) {
                            v3 no = offset_ray(p, through ? -ng : ng);
                            W.ray_o[s] = make_float4(no.x, no.y, no.z, 0.0f);
                            W.ray_d[s] = make_float4(wi.x, wi.y, wi.z, INFINITY);
                            W.tp[s] = make_float4(thr.x, thr.y, thr.z, pdf);
                            W.pst[s] = make_uint4((uint32_t)st, (uint32_t)(st >> 32), j, (depth + 1) | tag);
                            cont = true;
                        }
                    }
                }
            }
        }
        if (!cont) {
            ++done_paths;
            cont = start_path<NRC>(S, P, W, s, j + 1);
        }
        }
        const uint32_t k = block_append(out_cnt, cont, s_warp);
        if (cont) W.q_out[k] = s;
    }
    for (int o = 16; o > 0; o >>= 1) done_paths += __shfl_down_sync(0xffffffffu, done_paths, o);
    if ((threadIdx.x & 31) == 0 && done_paths) atomicAdd(&W.stats[kStatPaths], done_paths);
}

// Unoccluded shadow ray i adds its contribution to the slot's film entry
// (and, on a training path, to the path's radiance).
template <bool NRC>
__device__ __forceinline__ void shadow_done(const WaveParams& P, const WavePtrs& W, uint32_t i, const TraceResult& r) {
    if (r.tri < 0) {
        float4 c = W.sh_c[i];
        uint32_t pixel = (uint32_t)__float_as_int(W.sh_o[i].w);
        const int id = __float_as_int(c.w);  // training path id + 1, negated past max_depth
        if (!(NRC && P.visualize) && id >= 0) film_add(W.film, pixel, mk(c.x, c.y, c.z));
        if (NRC && id != 0) ltrain_add(W.ltrain, (uint32_t)((id > 0 ? id : -id) - 1), mk(c.x, c.y, c.z));
    }
}

template <bool COUNT, bool NRC = false>
__global__ void __launch_bounds__(128) k_shadow(DevScene S, WaveParams P, WavePtrs W) {
    grid_dep_wait();
    grid_dep_launch();
    uint32_t n = W.counters[kCntShadow];
    if (blockIdx.x == 0) {
        for (uint32_t b = threadIdx.x; b < P.nb; b += blockDim.x) W.counters[kCntBucket0 + b] = 0;
        if (threadIdx.x == 0) W.counters[kCntFetchTrace] = 0;
    }
    const int lane_id = threadIdx.x & 31;
    uint32_t nodes = 0, tris = 0;
    auto finish = [&](uint32_t i, const TraceResult& r) { shadow_done<NRC>(P, W, i, r); };
    if (!COUNT) {
        traverse_queue<true>(
            S, n, &W.counters[kCntFetchShadow],
            [&](uint32_t i, v3& o, v3& d, float& tmin, float& tmax) -> uint32_t {
                float4 ro = W.sh_o[i], rd = W.sh_d[i];
                o = f3(ro);
                d = f3(rd);
                tmin = 0.0f;
                tmax = rd.w;
                return i;
            },
            finish);
    } else {
        while (true) {
            uint32_t base = 0;
            if (lane_id == 0) base = atomicAdd(&W.counters[kCntFetchShadow], 32u);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= n) break;
            const uint32_t i = base + (uint32_t)lane_id;
            if (i >= n) continue;
            float4 o = W.sh_o[i], d = W.sh_d[i];
            finish(i, traverse<true, true>(S, f3(o), f3(d), 0.0f, d.w, nodes, tris));
        }
    }
    if (COUNT) {
        for (int o = 16; o > 0; o >>= 1) {
            nodes += __shfl_down_sync(0xffffffffu, nodes, o);
            tris += __shfl_down_sync(0xffffffffu, tris, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&W.stats[kStatShNodes], (unsigned long long)nodes);
            atomicAdd(&W.stats[kStatShTris], (unsigned long long)tris);
        }
    }
    if (threadIdx.x == 0 && blockIdx.x == 0) atomicAdd(&W.stats[kStatShadow], (unsigned long long)n);
}

// Fused traversal of the cache mode's unsorted pipeline: the extension rays of this
// iteration (queue cnt_in, closest hit) and the shadow rays the previous
// shading launch queued (counter sh_in, any hit) in one persistent launch
// with one fetch cursor, so neither waits for the other's last rays. It
// clears the queue and the shadow counter that the next shading launch
// fills (cnt_out, sh_out). Film updates keep their order per slot: a
// slot's shadow contribution of bounce k lands before bounce k + 1 is
// shaded, as in the three-launch pipeline.
template <bool NRC = false>
__global__ void __launch_bounds__(128) k_trace_fused(DevScene S, WaveParams P, WavePtrs W, uint32_t cnt_in,
                                                     uint32_t cnt_out, uint32_t sh_in, uint32_t sh_out) {
    grid_dep_wait();
    grid_dep_launch();
    const uint32_t n_ext = W.counters[cnt_in], n_sh = W.counters[sh_in];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        W.counters[cnt_out] = 0;
        W.counters[sh_out] = 0;
    }
    constexpr uint32_t kShadowTag = 0x80000000u;
    traverse_queue_kind<kQueueMixed>(
        S, n_ext + n_sh, &W.counters[kCntFetchTrace],
        [&](uint32_t i, v3& o, v3& d, float& tmin, float& tmax, bool& any) -> uint32_t {
            if (i < n_ext) {
                uint32_t s = W.q_in[i];
                float4 ro = W.ray_o[s], rd = W.ray_d[s];
                o = f3(ro);
                d = f3(rd);
                tmin = ro.w;
                tmax = rd.w;
                any = false;
                return s;
            }
            const uint32_t j = i - n_ext;
            float4 ro = W.sh_o[j], rd = W.sh_d[j];
            o = f3(ro);
            d = f3(rd);
            tmin = 0.0f;
            tmax = rd.w;
            any = true;
            return j | kShadowTag;
        },
        [&](uint32_t tag, const TraceResult& r) {
            if (tag & kShadowTag) shadow_done<NRC>(P, W, tag & ~kShadowTag, r);
            else W.hit[tag] = make_float4(r.t, r.u, r.v, __int_as_float(r.tri));
        });
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(&W.stats[kStatExt], (unsigned long long)n_ext);
        atomicAdd(&W.stats[kStatShadow], (unsigned long long)n_sh);
    }
}

// out = film / spp (or out += film). With sample replicas the K film copies
// are summed in replica order first.
__global__ void k_resolve(const float4* film, float* out, uint32_t pixels, float scale, int accumulate,
                          uint32_t replicas = 1) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < pixels; p += gridDim.x * blockDim.x) {
        float4 f = film[p];
        for (uint32_t r = 1; r < replicas; ++r) {
            float4 g = film[(size_t)r * pixels + p];
            f.x += g.x; f.y += g.y; f.z += g.z;
        }
        if (accumulate) {
            out[3 * (size_t)p + 0] += f.x;
            out[3 * (size_t)p + 1] += f.y;
            out[3 * (size_t)p + 2] += f.z;
        } else {
            out[3 * (size_t)p + 0] = f.x * scale;
            out[3 * (size_t)p + 1] = f.y * scale;
            out[3 * (size_t)p + 2] = f.z * scale;
        }
    }
}

// ---------------------------------------------------------------- host side
static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

constexpr uint64_t kStageTimingStride = 8;

static void ensure_workspace(aqua_ctx* ctx, size_t slots, size_t buckets, size_t pixels) {
    Workspace& w = ctx->ws;
    if (w.block.ptr && w.slots >= slots && w.buckets >= buckets && w.pixels >= pixels) return;
    slots = std::max(slots, w.slots);
    buckets = std::max(buckets, w.buckets);
    pixels = std::max(pixels, w.pixels);
    dev_free(w.block);
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
    size_t o_ro = take(16 * slots), o_rd = take(16 * slots), o_hit = take(16 * slots), o_tp = take(16 * slots),
           o_pst = take(16 * slots), o_q0 = take(4 * slots), o_q1 = take(4 * slots),
           o_bk = take(4 * slots * std::max<size_t>(buckets, 1)), o_sho = take(16 * slots),
           o_shd = take(16 * slots), o_shc = take(16 * slots), o_film = take(16 * pixels),
           o_cnt = take(4 * (kCntBucket0 + std::max<size_t>(buckets, 1) + 8)), o_st = take(8 * 16),
           o_out = take(12 * pixels);
    dev_alloc(ctx, w.block, off);
    char* b = (char*)w.block.ptr;
    w.ray_o = (float4*)(b + o_ro); w.ray_d = (float4*)(b + o_rd); w.hit = (float4*)(b + o_hit);
    w.tp = (float4*)(b + o_tp); w.pst = (uint4*)(b + o_pst);
    w.q[0] = (uint32_t*)(b + o_q0); w.q[1] = (uint32_t*)(b + o_q1);
    w.bucket = (uint32_t*)(b + o_bk);
    w.sh_o = (float4*)(b + o_sho); w.sh_d = (float4*)(b + o_shd); w.sh_c = (float4*)(b + o_shc);
    w.film = (float4*)(b + o_film);
    w.counters = (uint32_t*)(b + o_cnt);
    w.stats = (unsigned long long*)(b + o_st);
    w.out_rgb = (float*)(b + o_out);
    w.slots = slots; w.buckets = buckets; w.pixels = pixels;
}

void workspace_release(aqua_ctx* ctx) {
    dev_free(ctx->ws.block);
    ctx->ws = Workspace{};
}

template <class K>
static int grid_for(aqua_ctx* ctx, K kernel, int block, int blocks_per_sm) {
    int per_sm = blocks_per_sm;
    if (per_sm <= 0) {
        AQ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0));
        per_sm = std::max(per_sm, 1);
    }
    return ctx->num_sms * per_sm;
}

namespace {
// Event pairs around launches of one stage, summed after the render.
struct StageTimer {
    aqua_ctx* ctx;
    bool on;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pairs;
    size_t* next;
    cudaEvent_t get() {
        if (*next >= ctx->events.size()) {
            cudaEvent_t e;
            AQ_CUDA(cudaEventCreate(&e));
            ctx->events.push_back(e);
        }
        return ctx->events[(*next)++];
    }
    void begin() {
        if (!on) return;
        pairs.push_back({get(), nullptr});
        AQ_CUDA(cudaEventRecord(pairs.back().first, ctx->stream));
    }
    void end() {
        if (!on) return;
        pairs.back().second = get();
        AQ_CUDA(cudaEventRecord(pairs.back().second, ctx->stream));
    }
    double total_ms() {
        double t = 0.0;
        for (auto& p : pairs) {
            float ms = 0.0f;
            AQ_CUDA(cudaEventElapsedTime(&ms, p.first, p.second));
            t += ms;
        }
        return t;
    }
};

// Paths in flight: about 2^24 (16M) when `deep`, else 2^20 (with the
// material sort, whose per-material queues hold one entry per path and
// material, and in the cache mode, whose per-frame buffers follow the
// slots): below that many pixels, K sample replicas per pixel (K <= spp);
// otherwise one slot per pixel, up to 2^24 slots (2^21 when not deep). Every wavefront iteration pays a fixed cost (the stages' ramp
// and drain), so deep queues pay: on GB300 the Cornell GGX 1024^2 256-spp
// render takes 145.8 ms with 16M paths in flight against 182.4 ms with 1M
// (unsorted both), the interior at 1080p 204.6 against 251.6 ms, the
// sphere field 73.4 against 122.6 ms; 32M gains under 1% more.
struct SlotPlan {
    size_t slots;
    uint32_t replicas;
};
SlotPlan plan_slots(size_t pixels, int spp, const aqua_tuning& tune, bool deep) {
    const size_t target = (size_t)1 << (deep ? 24 : 20);
    size_t k = 1;
    if (tune.replicas > 0) k = (size_t)tune.replicas;
    else if (tune.slots <= 0 && pixels < target) k = (target + pixels - 1) / pixels;
    k = std::max<size_t>(1, std::min<size_t>(k, (size_t)spp));
    k = std::min<size_t>(k, ((size_t)1 << 24) / pixels + 1);
    SlotPlan p;
    if (k > 1) {
        p.slots = k * pixels;
        p.replicas = (uint32_t)k;
    } else {
        size_t slots = tune.slots > 0 ? (size_t)tune.slots : std::min<size_t>(pixels, std::max(target, (size_t)1 << 21));
        p.slots = std::min(slots, pixels);
        p.replicas = 1;
        if ((uint64_t)spp * ((pixels + p.slots - 1) / p.slots) > 0xFFFFFFFFull)
            throw Error(AQUA_ERR_INVALID_ARG, "spp x pixels per slot exceeds 2^32");
    }
    return p;
}
}  // namespace

// Rows of the camera image a render covers (aqua_integrator_cfg row subset);
// sets the parameters' row fields and returns the film's pixel count.
static size_t plan_rows(const aqua_integrator_cfg& cfg, const DevCamera& cam, WaveParams& P) {
    const size_t w = (size_t)cam.width, h = (size_t)cam.height;
    size_t rows = h;
    P.row_begin = 0;
    P.row_step = 1;
    P.width = (uint32_t)w;
    if (cfg.row_step > 1) {
        if (cfg.row_begin < 0 || cfg.row_begin >= cfg.row_step || (size_t)cfg.row_begin >= h)
            throw Error(AQUA_ERR_INVALID_ARG, "row_begin must lie in [0, row_step) and below the image height");
        rows = (h - (size_t)cfg.row_begin + (size_t)cfg.row_step - 1) / (size_t)cfg.row_step;
        P.row_begin = (uint32_t)cfg.row_begin;
        P.row_step = (uint32_t)cfg.row_step;
    } else if (cfg.row_begin != 0 || cfg.row_step < 0) {
        throw Error(AQUA_ERR_INVALID_ARG, "row_begin must be 0 and row_step >= 0 for whole images");
    }
    return w * rows;
}

void render_path(aqua_ctx* ctx, aqua_scene* sc, const aqua_integrator_cfg& cfg, const aqua_tuning& tune,
                 float* rgb_out, uint32_t flags, aqua_stats* stats) {
    const DevScene& S = sc->ds;
    if (cfg.spp <= 0) throw Error(AQUA_ERR_INVALID_ARG, "spp must be positive");
    check_depths(cfg.max_depth, cfg.rr_depth);
    WaveParams P{};
    size_t pixels = plan_rows(cfg, S.cam, P);
    if (pixels == 0 || pixels > (1u << 27)) throw Error(AQUA_ERR_INVALID_ARG, "resolution out of range");
    bool sorted = tune.sort_by_material > 0 && S.n_mats + 1 <= 256;
    const SlotPlan plan = plan_slots(pixels, cfg.spp, tune, !sorted);
    const size_t slots = plan.slots;
    size_t nb = sorted ? (size_t)S.n_mats + 1 : 0;
    ensure_workspace(ctx, slots, nb, pixels * plan.replicas);
    Workspace& w = ctx->ws;
    cudaStream_t st = ctx->stream;

    P.replicas = plan.replicas;
    P.seed = cfg.seed;
    P.spp = cfg.spp;
    P.spp_offset = cfg.spp_offset;
    P.max_depth = cfg.max_depth;
    P.rr_depth = cfg.rr_depth;
    P.slots = (uint32_t)slots;
    P.pixels = (uint32_t)pixels;
    P.nb = (uint32_t)nb;
    WavePtrs W;
    W.ray_o = w.ray_o; W.ray_d = w.ray_d; W.hit = w.hit; W.tp = w.tp; W.pst = w.pst;
    W.bucket = w.bucket; W.sh_o = w.sh_o; W.sh_d = w.sh_d; W.sh_c = w.sh_c; W.film = w.film;
    W.counters = w.counters; W.stats = w.stats;

    bool count = (flags & AQUA_RENDER_COUNT) != 0;
    bool timing = (flags & AQUA_RENDER_STAGE_TIMING) != 0;
    int bt = tune.block_trace > 0 ? tune.block_trace : 128;
    int bs = tune.block_shade > 0 ? tune.block_shade : 128;
    if (bt != 128 && bt != 64 && bt != 32) throw Error(AQUA_ERR_INVALID_ARG, "block_trace must be 32, 64 or 128");
    if (bs != 128 && bs != 64 && bs != 32) throw Error(AQUA_ERR_INVALID_ARG, "block_shade must be 32, 64 or 128");

    auto trace_k = sorted ? (count ? k_trace_ext<true, true> : k_trace_ext<true, false>)
                          : (count ? k_trace_ext<false, true> : k_trace_ext<false, false>);
    const bool full = S.mext != nullptr;  // some material sets the full model's lobes
    auto shade_k = full ? (sorted ? k_shade<true, false, true> : k_shade<false, false, true>)
                        : (sorted ? k_shade<true> : k_shade<false>);
    auto shadow_k = count ? k_shadow<true> : k_shadow<false>;
    int g_trace = grid_for(ctx, trace_k, bt, tune.blocks_per_sm);
    int g_shade = grid_for(ctx, shade_k, bs, tune.blocks_per_sm);
    int g_shadow = grid_for(ctx, shadow_k, bt, tune.blocks_per_sm);

    cudaEvent_t ev0, ev1;
    size_t next_event = 0;
    StageTimer tt{ctx, timing, {}, &next_event}, ts{ctx, timing, {}, &next_event}, tsh{ctx, timing, {}, &next_event};
    ev0 = tt.get();
    ev1 = tt.get();

    AQ_CUDA(cudaMemsetAsync(w.film, 0, 16 * pixels * plan.replicas, st));
    AQ_CUDA(cudaMemsetAsync(w.stats, 0, 8 * 16, st));
    AQ_CUDA(cudaMemsetAsync(w.counters, 0, 4 * (kCntBucket0 + std::max<size_t>(nb, 1)), st));
    AQ_CUDA(cudaEventRecord(ev0, st));
    uint64_t launches = 0;
    W.q_in = w.q[0];
    W.q_out = w.q[1];
    {
        int g = (int)std::min<size_t>((slots + 255) / 256, (size_t)ctx->num_sms * 16);
        k_raygen<<<std::max(g, 1), 256, 0, st>>>(S, P, W);
        AQ_CUDA(cudaGetLastError());
        ++launches;
    }
    const int chunk = tune.iters_per_graph > 0 ? tune.iters_per_graph : 16;
    uint64_t iter = 0;
    unsigned int* pc = ctx->pinned_counter;
    cudaEvent_t chunk_ev[2] = {tt.get(), tt.get()};
    int c = 0;
    const uint64_t max_iters = (uint64_t)(cfg.max_depth + 2) * (uint64_t)cfg.spp *
                                   ((pixels + slots - 1) / slots) + 64;
    while (true) {
        for (int k = 0; k < chunk; ++k, ++iter) {
            uint32_t in = (uint32_t)(iter & 1), out = 1u - in;
            W.q_in = w.q[in];
            W.q_out = w.q[out];
            // Stage timing brackets every kStageTimingStride-th iteration so
            // the events barely perturb the launch stream.
            bool timed = timing && (iter % kStageTimingStride) == 0;
            if (timed) tt.begin();
            launch_chained(trace_k, g_trace, bt, 0, st, S, P, W, in, out);
            if (timed) { tt.end(); ts.begin(); }
            launch_chained(shade_k, g_shade, bs, 0, st, S, P, W, in, out, (uint32_t)kCntShadow);
            if (timed) { ts.end(); tsh.begin(); }
            launch_chained(shadow_k, g_shadow, bt, 0, st, S, P, W);
            if (timed) tsh.end();
            launches += 3;
        }
        AQ_CUDA(cudaGetLastError());
        AQ_CUDA(cudaMemcpyAsync(&pc[c & 1], &w.counters[iter & 1], 4, cudaMemcpyDeviceToHost, st));
        AQ_CUDA(cudaEventRecord(chunk_ev[c & 1], st));
        if (c > 0) {
            AQ_CUDA(cudaEventSynchronize(chunk_ev[(c - 1) & 1]));
            if (pc[(c - 1) & 1] == 0) break;
        }
        ++c;
        if (iter > max_iters) {
            AQ_CUDA(cudaStreamSynchronize(st));
            if (pc[(c - 1) & 1] != 0)
                throw Error(AQUA_ERR_TIMEOUT, "wavefront did not drain within the iteration bound");
            break;
        }
    }
    float* dst = (flags & AQUA_RENDER_DEVICE_FILM) ? rgb_out : w.out_rgb;
    bool acc = (flags & AQUA_RENDER_ACCUMULATE) != 0;
    if (acc && !(flags & AQUA_RENDER_DEVICE_FILM))
        AQ_CUDA(cudaMemcpyAsync(dst, rgb_out, 12 * pixels, cudaMemcpyHostToDevice, st));
    {
        int g = (int)std::min<size_t>((pixels + 255) / 256, (size_t)ctx->num_sms * 16);
        k_resolve<<<g, 256, 0, st>>>(w.film, dst, (uint32_t)pixels, 1.0f / (float)cfg.spp, acc ? 1 : 0,
                                     plan.replicas);
        AQ_CUDA(cudaGetLastError());
        ++launches;
    }
    AQ_CUDA(cudaEventRecord(ev1, st));
    if (!(flags & AQUA_RENDER_DEVICE_FILM))
        AQ_CUDA(cudaMemcpyAsync(rgb_out, w.out_rgb, 12 * pixels, cudaMemcpyDeviceToHost, st));
    unsigned long long hs[16];
    AQ_CUDA(cudaMemcpyAsync(hs, w.stats, 8 * 16, cudaMemcpyDeviceToHost, st));
    AQ_CUDA(cudaStreamSynchronize(st));
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        float ms = 0.0f;
        AQ_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
        stats->device_ms = ms;
        stats->paths = hs[kStatPaths];
        stats->ext_rays = hs[kStatExt];
        stats->shadow_rays = hs[kStatShadow];
        stats->iterations = iter;
        // With stage timing: the launches whose times the *_ms fields sum.
        stats->trace_launches = timing ? tt.pairs.size() : iter;
        stats->shade_launches = timing ? ts.pairs.size() : iter;
        stats->shadow_launches = timing ? tsh.pairs.size() : iter;
        stats->total_launches = launches;
        stats->node_visits = hs[kStatNodes];
        stats->tri_tests = hs[kStatTris];
        stats->shadow_node_visits = hs[kStatShNodes];
        stats->shadow_tri_tests = hs[kStatShTris];
        if (timing) {
            stats->trace_ms = tt.total_ms();
            stats->shade_ms = ts.total_ms();
            stats->shadow_ms = tsh.total_ms();
        }
    }
}

// ---------------------------------------------------------------- radiance cache frame
// film[pixel] += throughput * max(cache(x), 0) for every queued query. Several
// samples of one pixel may have queried, so the add is atomic.
__global__ void k_nrc_resolve(const float4* __restrict__ q_pix, const float* __restrict__ pred, uint32_t n,
                              float4* film) {
    grid_dep_wait();
    grid_dep_launch();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 q = __ldcg(q_pix + i);
        uint32_t pixel = (uint32_t)__float_as_int(q.x);
        float* f = reinterpret_cast<float*>(film + pixel);
        atomicAdd(f + 0, q.y * fmaxf(__ldcg(pred + 3 * (size_t)i + 0), 0.0f));
        atomicAdd(f + 1, q.z * fmaxf(__ldcg(pred + 3 * (size_t)i + 1), 0.0f));
        atomicAdd(f + 2, q.w * fmaxf(__ldcg(pred + 3 * (size_t)i + 2), 0.0f));
    }
}

// Training targets: radiance leaving each recorded vertex toward its
// predecessor = (radiance of the whole path - radiance gathered before the
// vertex reflected anything) / throughput at the vertex, per channel.
// Records are scattered by i -> (a*i + b) mod n so that consecutive
// training batches mix paths, bounces and materials.
constexpr float kNrcMinThroughput = 1e-3f;
constexpr float kNrcMaxTarget = 1e3f;

__global__ void k_nrc_targets(const float4* __restrict__ rec, uint32_t n, const float4* __restrict__ ltrain,
                              const float4* __restrict__ lsnap, int train_span, int train_depth, uint64_t a,
                              uint64_t b, float* __restrict__ raw_out, float* __restrict__ t_out) {
    grid_dep_wait();
    grid_dep_launch();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4* r = rec + 6 * (size_t)i;
        uint32_t j = (uint32_t)((a * (uint64_t)i + b) % (uint64_t)n);
        float4* ro = reinterpret_cast<float4*>(raw_out + 16 * (size_t)j);
        ro[0] = r[0]; ro[1] = r[1]; ro[2] = r[2]; ro[3] = r[3];
        float4 w4 = r[4], w5 = r[5];
        // w4 = (beta.xyz, L_before.x), w5 = (L_before.yz, id, depth d).
        // Radiance of reflections d .. d + span - 1 = (gathered before bounce
        // d + span) - (gathered before bounce d); past the path's end the
        // path's total.
        uint32_t id = (uint32_t)__float_as_int(w5.z);
        int d = __float_as_int(w5.w);
        float4 L = ltrain[id];
        int k = d + train_span;
        if (k < train_depth) {
            float4 s = lsnap[(size_t)id * (size_t)train_depth + k];
            if (s.x >= 0.0f) L = s;
        }
        float t0 = fmaxf(L.x - w4.w, 0.0f) / fmaxf(w4.x, kNrcMinThroughput);
        float t1 = fmaxf(L.y - w5.x, 0.0f) / fmaxf(w4.y, kNrcMinThroughput);
        float t2 = fmaxf(L.z - w5.y, 0.0f) / fmaxf(w4.z, kNrcMinThroughput);
        t_out[3 * (size_t)j + 0] = fminf(t0, kNrcMaxTarget);
        t_out[3 * (size_t)j + 1] = fminf(t1, kNrcMaxTarget);
        t_out[3 * (size_t)j + 2] = fminf(t2, kNrcMaxTarget);
    }
}

// Vertices a training path records in path-spread mode (bounces 0..3).
constexpr int kSpreadRecordDepth = 4;

static void ensure_nrc_workspace(aqua_ctx* ctx, size_t queries, size_t records, size_t snaps) {
    NrcWorkspace& w = ctx->nrc_ws;
    if (w.block.ptr && w.queries >= queries && w.records >= records && w.snaps >= snaps) return;
    queries = std::max(queries, w.queries);
    records = std::max(records, w.records);
    snaps = std::max(snaps, w.snaps);
    dev_free(w.block);
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
    size_t o_qp = take(16 * queries), o_qr = take(64 * queries), o_qx = take(128 * queries),
           o_qo = take(12 * queries), o_rec = take(96 * records), o_lt = take(16 * records),
           o_tr = take(64 * records), o_tx = take(128 * records), o_tt = take(12 * records),
           o_sn = take(16 * records * snaps), o_sp = take(8 * queries);
    dev_alloc(ctx, w.block, off);
    char* b = (char*)w.block.ptr;
    w.q_pix = (float4*)(b + o_qp);
    w.q_raw = (float*)(b + o_qr);
    w.q_x = (uint16_t*)(b + o_qx);
    w.q_pred = (float*)(b + o_qo);
    w.rec = (float4*)(b + o_rec);
    w.ltrain = (float4*)(b + o_lt);
    w.t_raw = (float*)(b + o_tr);
    w.t_x = (uint16_t*)(b + o_tx);
    w.t_target = (float*)(b + o_tt);
    w.lsnap = (float4*)(b + o_sn);
    w.spread = (float2*)(b + o_sp);  // one per path slot (slots <= queries)
    w.queries = queries;
    w.records = records;
    w.snaps = snaps;
}

static uint64_t gcd64(uint64_t a, uint64_t b) {
    while (b) { uint64_t t = a % b; a = b; b = t; }
    return a;
}

void render_nrc(aqua_ctx* ctx, aqua_scene* sc, const aqua_integrator_cfg& cfg, const aqua_tuning& tune,
                aqua_nrc* nrc, float* rgb_out, uint32_t flags, aqua_stats* stats) {
    const DevScene& S = sc->ds;
    NrcNet& net = nrc->net;
    if (cfg.spp <= 0) throw Error(AQUA_ERR_INVALID_ARG, "spp must be positive");
    check_depths(cfg.max_depth, cfg.rr_depth);
    if (cfg.nrc_train_samples < 0) throw Error(AQUA_ERR_INVALID_ARG, "nrc_train_samples must be >= 0");
    if (cfg.batch_size <= 0) throw Error(AQUA_ERR_INVALID_ARG, "batch_size must be positive");
    WaveParams P{};
    size_t pixels = plan_rows(cfg, S.cam, P);
    if (pixels == 0 || pixels > (1u << 27)) throw Error(AQUA_ERR_INVALID_ARG, "resolution out of range");
    const SlotPlan plan = plan_slots(pixels, cfg.spp, tune, false);
    const size_t slots = plan.slots;
    if ((uint64_t)pixels * (uint64_t)cfg.spp > ((uint64_t)1 << 31))
        throw Error(AQUA_ERR_INVALID_ARG, "one cache frame is limited to 2^31 samples");
    bool sorted = tune.sort_by_material > 0 && S.n_mats + 1 <= 256;
    size_t nb = sorted ? (size_t)S.n_mats + 1 : 0;
    ensure_workspace(ctx, slots, nb, pixels * plan.replicas);
    size_t cap_q = pixels * (size_t)cfg.spp;
    size_t cap_r = std::max<size_t>((size_t)cfg.nrc_train_samples, 1);
    // nrc_query_vertex = AQUA_NRC_QUERY_SPREAD: query where the path spread
    // exceeds c a0 (at vertex 2 or later); targets then span max_depth - 1.
    const bool by_spread = !cfg.visualize_cache && cfg.nrc_query_vertex == AQUA_NRC_QUERY_SPREAD;
    const int query_depth = cfg.visualize_cache ? 0 : by_spread ? -1 : std::max(0, cfg.nrc_query_vertex - 1);
    const int train_span = std::max(1, cfg.max_depth - (by_spread ? 1 : query_depth));
    // By path spread most queries fall on vertices 2-4, so training paths
    // record their first four vertices only and end train_span bounces past
    // the fourth: shorter tails of the few-ray iterations that follow the
    // queries. With a fixed query vertex they record every vertex below
    // max_depth.
    const int record_depth = by_spread ? std::min(cfg.max_depth, kSpreadRecordDepth) : cfg.max_depth;
    const int train_depth = std::min(record_depth + train_span, 250);
    ensure_nrc_workspace(ctx, cap_q, cap_r, (size_t)train_depth);
    Workspace& w = ctx->ws;
    NrcWorkspace& nw = ctx->nrc_ws;
    cudaStream_t st = ctx->stream;

    // Positions are encoded relative to the scene's bounding box.
    {
        for (int k = 0; k < 3; ++k) {
            net.bmin[k] = sc->bvh.lo[k];
            net.bext[k] = std::max(sc->bvh.hi[k] - sc->bvh.lo[k], 1e-6f);
        }
    }
    const bool visualize = cfg.visualize_cache != 0;
    P.replicas = plan.replicas;
    P.seed = cfg.seed;
    P.spp = cfg.spp;
    P.spp_offset = cfg.spp_offset;
    P.max_depth = cfg.max_depth;
    P.rr_depth = cfg.rr_depth;
    P.slots = (uint32_t)slots;
    P.pixels = (uint32_t)pixels;
    P.nb = (uint32_t)nb;
    P.query_depth = query_depth;
    P.spread_c = 0.01f;  // Mueller et al. 2021
    // Fraction of paths that train: aimed at nrc_train_samples records per
    // frame (first frame: assume 3 recorded vertices per training path).
    double frac = 0.0;
    if (!visualize && cfg.nrc_train_samples > 0)
        frac = net.train_frac > 0.0 ? net.train_frac
                                    : (double)cfg.nrc_train_samples / (3.0 * (double)pixels * cfg.spp);
    frac = std::min(frac, 1.0);
    P.train_thresh = (uint32_t)std::min(16777216.0, frac * 16777216.0);
    P.max_train_paths = (uint32_t)cap_r;
    P.max_records = (uint32_t)cap_r;
    P.train_span = train_span;
    P.record_depth = record_depth;
    P.train_depth = train_depth;
    P.visualize = visualize ? 1 : 0;
    WavePtrs W{};
    W.ray_o = w.ray_o; W.ray_d = w.ray_d; W.hit = w.hit; W.tp = w.tp; W.pst = w.pst;
    W.bucket = w.bucket; W.sh_o = w.sh_o; W.sh_d = w.sh_d; W.sh_c = w.sh_c; W.film = w.film;
    W.counters = w.counters; W.stats = w.stats;
    W.q_pix = nw.q_pix; W.q_raw = nw.q_raw; W.rec = nw.rec; W.ltrain = nw.ltrain; W.lsnap = nw.lsnap;
    W.spread = nw.spread;

    auto trace_k = sorted ? k_trace_ext<true, false> : k_trace_ext<false, false>;
    auto shade_k = S.mext ? (sorted ? k_shade<true, true, true> : k_shade<false, true, true>)
                          : (sorted ? k_shade<true, true> : k_shade<false, true>);
    auto shadow_k = k_shadow<false, true>;
    int g_trace = grid_for(ctx, trace_k, 128, tune.blocks_per_sm);
    int g_shade = grid_for(ctx, shade_k, 128, tune.blocks_per_sm);
    int g_shadow = grid_for(ctx, shadow_k, 128, tune.blocks_per_sm);
    // Unsorted cache frames fuse each iteration's extension rays with the
    // previous iteration's shadow rays (k_trace_fused): a 1-spp frame holds
    // one path per pixel, and after the queries only training paths go on,
    // so most of its iterations trace few rays and are bound by the latency
    // of one walk; fused, the two walks overlap (frame 4.42 -> 3.55 ms on
    // the 1080p interior). Deep plain renders stay on three launches, where
    // the fused launch measured 2.3% slower (Cornell GGX 1024^2).
    const bool fused = !sorted;
    auto fused_k = k_trace_fused<true>;
    int g_fused = fused ? grid_for(ctx, fused_k, 128, tune.blocks_per_sm) : 0;

    cudaEvent_t ev[4];
    size_t next_event = 0;
    StageTimer tm{ctx, true, {}, &next_event};
    for (auto& e : ev) e = tm.get();
    AQ_CUDA(cudaMemsetAsync(w.film, 0, 16 * pixels * plan.replicas, st));
    AQ_CUDA(cudaMemsetAsync(w.stats, 0, 8 * 16, st));
    AQ_CUDA(cudaMemsetAsync(w.counters, 0, 4 * (kCntBucket0 + std::max<size_t>(nb, 1)), st));
    AQ_CUDA(cudaEventRecord(ev[0], st));
    uint64_t launches = 0;
    W.q_in = w.q[0];
    W.q_out = w.q[1];
    {
        int g = (int)std::min<size_t>((slots + 255) / 256, (size_t)ctx->num_sms * 16);
        k_raygen<true><<<std::max(g, 1), 256, 0, st>>>(S, P, W);
        AQ_CUDA(cudaGetLastError());
        ++launches;
    }
    // A 1-spp frame drains within train_depth + 1 iterations: no empty
    // iterations before the host's check.
    const int chunk = std::min(tune.iters_per_graph > 0 ? tune.iters_per_graph : 16, train_depth + 2);
    const uint64_t max_iters =
        (uint64_t)(train_depth + 2) * (uint64_t)cfg.spp * ((pixels + slots - 1) / slots) + 64;
    uint64_t iter = 0;
    unsigned int* pc = ctx->pinned_counter;
    while (true) {
        for (int k = 0; k < chunk; ++k, ++iter) {
            uint32_t in = (uint32_t)(iter & 1), out = 1u - in;
            W.q_in = w.q[in];
            W.q_out = w.q[out];
            if (fused) {
                const uint32_t sh_now = in ? kCntShadow1 : kCntShadow, sh_prev = in ? kCntShadow : kCntShadow1;
                launch_chained(fused_k, g_fused, 128, 0, st, S, P, W, in, out, sh_prev, sh_now);
                launch_chained(shade_k, g_shade, 128, 0, st, S, P, W, in, out, sh_now);
                launches += 2;
                continue;
            }
            launch_chained(trace_k, g_trace, 128, 0, st, S, P, W, in, out);
            launch_chained(shade_k, g_shade, 128, 0, st, S, P, W, in, out, (uint32_t)kCntShadow);
            launch_chained(shadow_k, g_shadow, 128, 0, st, S, P, W);
            launches += 3;
        }
        AQ_CUDA(cudaGetLastError());
        AQ_CUDA(cudaMemcpyAsync(&pc[8], &w.counters[iter & 1], 4, cudaMemcpyDeviceToHost, st));
        AQ_CUDA(cudaMemcpyAsync(&pc[9], &w.counters[kCntQuery], 12, cudaMemcpyDeviceToHost, st));
        AQ_CUDA(cudaStreamSynchronize(st));
        if (pc[8] == 0) break;
        if (iter > max_iters) throw Error(AQUA_ERR_TIMEOUT, "wavefront did not drain within the iteration bound");
    }
    if (fused) {  // the shadow rays of the last shading launch
        const uint32_t in = (uint32_t)(iter & 1), out = 1u - in;
        const uint32_t sh_last = in ? kCntShadow : kCntShadow1, sh_other = in ? kCntShadow1 : kCntShadow;
        W.q_in = w.q[in];
        W.q_out = w.q[out];
        launch_chained(fused_k, g_fused, 128, 0, st, S, P, W, in, out, sh_last, sh_other);
        ++launches;
    }
    AQ_CUDA(cudaEventRecord(ev[1], st));
    const uint32_t nq = pc[9], nrec = std::min(pc[10], P.max_records), ntp = pc[11];
    // Cache queries: encode, infer, add throughput x prediction.
    if (nq > 0) {
        nrc_encode_dev(ctx, net, nw.q_raw, (int)nq, nw.q_x);
        nrc_forward_dev(ctx, net, nw.q_x, (int)nq, nw.q_pred);
        int g = (int)std::min<size_t>((nq + 255) / 256, (size_t)ctx->num_sms * 16);
        launch_chained(k_nrc_resolve, dim3(g), dim3(256), 0, st, (const float4*)nw.q_pix, (const float*)nw.q_pred, nq,
                       w.film);
        AQ_CUDA(cudaGetLastError());
        launches += 3;
    }
    AQ_CUDA(cudaEventRecord(ev[2], st));
    // Online training on this frame's records.
    double loss = 0.0;
    int steps = 0;
    if (nrec > 0 && !visualize) {
        uint64_t a = 2654435761ull % nrec, b = 0x9E37ull % nrec;
        if (a == 0) a = 1;
        while (gcd64(a, nrec) != 1) ++a;
        int g = (int)std::min<size_t>((nrec + 255) / 256, (size_t)ctx->num_sms * 16);
        k_nrc_targets<<<g, 256, 0, st>>>(nw.rec, nrec, nw.ltrain, nw.lsnap, train_span, train_depth, a, b, nw.t_raw,
                                          nw.t_target);  // after an event record: nothing to chain to
        AQ_CUDA(cudaGetLastError());
        nrc_encode_dev(ctx, net, nw.t_raw, (int)nrec, nw.t_x);
        launches += 2;
        int batch = cfg.batch_size;
        steps = (int)((nrec + (uint32_t)batch - 1) / (uint32_t)batch);
        if (cfg.training_iters > 0) steps = std::min(steps, cfg.training_iters);
        for (int sidx = 0; sidx < steps; ++sidx) {
            size_t r0 = (size_t)sidx * (size_t)batch;
            int rows = (int)std::min<size_t>((size_t)batch, nrec - r0);
            nrc_train_step_dev(ctx, net, nw.t_x + 64 * r0, nw.t_target + 3 * r0, rows);
            launches += net.forward_tc ? 4 : 6;
        }
        AQ_CUDA(cudaMemcpyAsync(&loss, net.loss, 8, cudaMemcpyDeviceToHost, st));
        // Aim the next frame's training-path fraction at the record budget.
        double per_path = ntp > 0 ? (double)pc[10] / (double)std::min<uint32_t>(ntp, P.max_train_paths) : 3.0;
        double want = (double)cfg.nrc_train_samples / std::max(per_path, 1.0);
        net.train_frac = std::min(1.0, want / ((double)pixels * cfg.spp));
    }
    AQ_CUDA(cudaEventRecord(ev[3], st));
    float* dst = (flags & AQUA_RENDER_DEVICE_FILM) ? rgb_out : w.out_rgb;
    bool acc = (flags & AQUA_RENDER_ACCUMULATE) != 0;
    if (acc && !(flags & AQUA_RENDER_DEVICE_FILM))
        AQ_CUDA(cudaMemcpyAsync(dst, rgb_out, 12 * pixels, cudaMemcpyHostToDevice, st));
    {
        int g = (int)std::min<size_t>((pixels + 255) / 256, (size_t)ctx->num_sms * 16);
        k_resolve<<<g, 256, 0, st>>>(w.film, dst, (uint32_t)pixels, 1.0f / (float)cfg.spp, acc ? 1 : 0,
                                     plan.replicas);
        AQ_CUDA(cudaGetLastError());
        ++launches;
    }
    if (!(flags & AQUA_RENDER_DEVICE_FILM))
        AQ_CUDA(cudaMemcpyAsync(rgb_out, w.out_rgb, 12 * pixels, cudaMemcpyDeviceToHost, st));
    unsigned long long hs[16];
    AQ_CUDA(cudaMemcpyAsync(hs, w.stats, 8 * 16, cudaMemcpyDeviceToHost, st));
    AQ_CUDA(cudaStreamSynchronize(st));
    nrc_check_tc(ctx, net);
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        float ms = 0.0f, q_ms = 0.0f, t_ms = 0.0f;
        AQ_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[3]));
        AQ_CUDA(cudaEventElapsedTime(&q_ms, ev[1], ev[2]));
        AQ_CUDA(cudaEventElapsedTime(&t_ms, ev[2], ev[3]));
        stats->device_ms = ms;
        stats->nrc_ms = q_ms + t_ms;
        stats->paths = hs[kStatPaths];
        stats->ext_rays = hs[kStatExt];
        stats->shadow_rays = hs[kStatShadow];
        stats->iterations = iter;
        stats->trace_launches = stats->shade_launches = stats->shadow_launches = iter;
        stats->total_launches = launches;
        stats->nrc_queries = nq;
        stats->nrc_train_records = nrec;
        stats->nrc_loss = nrec > 0 && steps > 0 ? loss / (double)(std::min<size_t>((size_t)cfg.batch_size,
                                                                                  nrec - (size_t)(steps - 1) * cfg.batch_size) * 3)
                                                : 0.0;
    }
}

// ---------------------------------------------------------------- no-allocation variant
// Some callers cannot let a library call cudaMalloc: engines that own all
// device memory through their own arena and a fixed budget, and hosts where
// the implicit device synchronisation of cudaMalloc/cudaFree would stall
// other work on the GPU. For them this variant runs the same wavefront
// kernels on a fixed scratch area that lives in this file as a static device
// array, so a render call allocates nothing. The caller still passes the
// scene (loaded earlier) and a device buffer for the image.
//
// Scratch layout: path state for kNoAllocSlots slots (ray origin, direction,
// hit, throughput, rng/work/depth: 16 B each; two 4 B queues; a 48 B shadow
// record) + a 16 B film entry for up to kNoAllocPixels pixels + counters.
// Every GPU that loads this library holds the array (about 17.3 MB) until
// the process exits. All calls share it and it keeps the last call's
// contents; each call clears the film, counters and statistics it needs.
// Calls whose work overlaps on the GPU (two contexts or streams at once)
// race on the array.
constexpr size_t kNoAllocSlots = (size_t)1 << 16;
constexpr size_t kNoAllocPixels = (size_t)1 << 19;
constexpr size_t kNoAllocCounters = 64;  // uint32, >= kCntBucket0 + 8
constexpr size_t kNoAllocStats = 16;     // uint64
constexpr size_t kNoAllocStateBytes = kNoAllocSlots * (5 * 16 + 2 * 4 + 3 * 16);
constexpr size_t kNoAllocBytes =
    kNoAllocStateBytes + kNoAllocPixels * 16 + kNoAllocCounters * 4 + kNoAllocStats * 8;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_base[kNoAllocMaxDevices] = {};

// Device address of the scratch array on the current device. In host code
// `g_noalloc_scratch` names a host-side stand-in, not device memory, so the
// address is looked up once per device (the first call on that device does
// it, which also loads the module that holds the array) and cached.
void* noalloc_base(int device) {
    if (device < 0 || device >= kNoAllocMaxDevices)
        throw Error(AQUA_ERR_UNSUPPORTED, "device ordinal beyond the no-allocation table");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_base[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            throw Error(AQUA_ERR_CUDA, std::string("cudaGetSymbolAddress(no-allocation scratch): ") +
                                           cudaGetErrorString(e));
        g_noalloc_base[device] = p;
    }
    return g_noalloc_base[device];
}
}  // namespace

size_t render_noalloc_max_pixels() { return kNoAllocPixels; }

void render_noalloc(aqua_ctx* ctx, aqua_scene* sc, const aqua_integrator_cfg& cfg, float* rgb_out,
                    aqua_stats* stats) {
    const DevScene& S = sc->ds;
    if (cfg.spp <= 0) throw Error(AQUA_ERR_INVALID_ARG, "spp must be positive");
    check_depths(cfg.max_depth, cfg.rr_depth);
    WaveParams P{};
    size_t pixels = plan_rows(cfg, S.cam, P);
    if (pixels == 0) throw Error(AQUA_ERR_INVALID_ARG, "resolution out of range");
    if (pixels > kNoAllocPixels)
        throw Error(AQUA_ERR_INVALID_ARG, "aqua_render_noalloc: " + std::to_string(pixels) +
                                              " pixels exceed the fixed scratch limit of " +
                                              std::to_string(kNoAllocPixels) + " pixels");
    size_t slots = std::min(pixels, kNoAllocSlots);
    if ((uint64_t)cfg.spp * ((pixels + slots - 1) / slots) > 0xFFFFFFFFull)
        throw Error(AQUA_ERR_INVALID_ARG, "spp x pixels per slot exceeds 2^32");
    if (((uintptr_t)rgb_out & 3) != 0) throw Error(AQUA_ERR_INVALID_ARG, "rgb_out must be 4-byte aligned");
    char* base = (char*)noalloc_base(ctx->device);
    cudaStream_t st = ctx->stream;

    P.seed = cfg.seed;  // no replicas, no cache mode
    P.spp = cfg.spp;
    P.spp_offset = cfg.spp_offset;
    P.max_depth = cfg.max_depth;
    P.rr_depth = cfg.rr_depth;
    P.slots = (uint32_t)slots;
    P.pixels = (uint32_t)pixels;
    P.nb = 0;  // unsorted shading: no per-material buckets
    WavePtrs W;
    size_t off = 0;
    auto take = [&](size_t bytes) { char* p = base + off; off += bytes; return p; };
    W.ray_o = (float4*)take(16 * kNoAllocSlots);
    W.ray_d = (float4*)take(16 * kNoAllocSlots);
    W.hit = (float4*)take(16 * kNoAllocSlots);
    W.tp = (float4*)take(16 * kNoAllocSlots);
    W.pst = (uint4*)take(16 * kNoAllocSlots);
    uint32_t* q[2];
    q[0] = (uint32_t*)take(4 * kNoAllocSlots);
    q[1] = (uint32_t*)take(4 * kNoAllocSlots);
    W.sh_o = (float4*)take(16 * kNoAllocSlots);
    W.sh_d = (float4*)take(16 * kNoAllocSlots);
    W.sh_c = (float4*)take(16 * kNoAllocSlots);
    W.film = (float4*)take(16 * kNoAllocPixels);
    W.counters = (uint32_t*)take(4 * kNoAllocCounters);
    W.stats = (unsigned long long*)take(8 * kNoAllocStats);
    W.bucket = nullptr;

    // Leftovers of the previous call must not leak into this one.
    AQ_CUDA(cudaMemsetAsync(W.film, 0, 16 * pixels, st));
    AQ_CUDA(cudaMemsetAsync(W.counters, 0, 4 * kNoAllocCounters, st));
    AQ_CUDA(cudaMemsetAsync(W.stats, 0, 8 * kNoAllocStats, st));

    auto trace_k = k_trace_ext<false, false>;
    auto shade_k = S.mext ? k_shade<false, false, true> : k_shade<false>;
    auto shadow_k = k_shadow<false>;
    int g_trace = grid_for(ctx, trace_k, 128, 0);
    int g_shade = grid_for(ctx, shade_k, 128, 0);
    int g_shadow = grid_for(ctx, shadow_k, 128, 0);
    uint64_t launches = 0;
    W.q_in = q[0];
    W.q_out = q[1];
    {
        int g = (int)std::min<size_t>((slots + 255) / 256, (size_t)ctx->num_sms * 16);
        k_raygen<<<std::max(g, 1), 256, 0, st>>>(S, P, W);
        AQ_CUDA(cudaGetLastError());
        ++launches;
    }
    const int chunk = 16;
    const uint64_t max_iters =
        (uint64_t)(cfg.max_depth + 2) * (uint64_t)cfg.spp * ((pixels + slots - 1) / slots) + 64;
    uint64_t iter = 0;
    unsigned int* pc = ctx->pinned_counter;  // pinned when the context was created
    while (true) {
        for (int k = 0; k < chunk; ++k, ++iter) {
            uint32_t in = (uint32_t)(iter & 1), out = 1u - in;
            W.q_in = q[in];
            W.q_out = q[out];
            launch_chained(trace_k, g_trace, 128, 0, st, S, P, W, in, out);
            launch_chained(shade_k, g_shade, 128, 0, st, S, P, W, in, out, (uint32_t)kCntShadow);
            launch_chained(shadow_k, g_shadow, 128, 0, st, S, P, W);
            launches += 3;
        }
        AQ_CUDA(cudaGetLastError());
        AQ_CUDA(cudaMemcpyAsync(&pc[4], &W.counters[iter & 1], 4, cudaMemcpyDeviceToHost, st));
        AQ_CUDA(cudaStreamSynchronize(st));
        if (pc[4] == 0) break;
        if (iter > max_iters) throw Error(AQUA_ERR_TIMEOUT, "wavefront did not drain within the iteration bound");
    }
    {
        int g = (int)std::min<size_t>((pixels + 255) / 256, (size_t)ctx->num_sms * 16);
        k_resolve<<<g, 256, 0, st>>>(W.film, rgb_out, (uint32_t)pixels, 1.0f / (float)cfg.spp, 0);
        AQ_CUDA(cudaGetLastError());
        ++launches;
    }
    unsigned long long hs[kNoAllocStats];
    AQ_CUDA(cudaMemcpyAsync(hs, W.stats, sizeof(hs), cudaMemcpyDeviceToHost, st));
    AQ_CUDA(cudaStreamSynchronize(st));
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->paths = hs[kStatPaths];
        stats->ext_rays = hs[kStatExt];
        stats->shadow_rays = hs[kStatShadow];
        stats->iterations = iter;
        stats->trace_launches = iter;
        stats->shade_launches = iter;
        stats->shadow_launches = iter;
        stats->total_launches = launches;
    }
}

}  // namespace aq
