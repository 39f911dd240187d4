// batch.cu — batched rendering of many independent jobs (views of several
// scenes, uneven resolutions and sample counts) in one persistent launch,
// replayed from a captured CUDA graph.
//
// Every lane of the persistent kernel owns one pixel at a time and keeps one
// path of it in flight: a path advances one bounce per loop iteration, and
// when it ends the lane starts the pixel's next sample at once (path
// regeneration), so lanes do not wait for the longest path of their warp.
// When a pixel has all its samples the lane writes it and, together with
// the other idle lanes of its warp, takes the next pixels from a global
// counter; jobs are laid out shortest first (pixels x spp), so small jobs
// complete early. Contributions are summed in the wavefront's order
// (emission, then next-event estimation, bounce after bounce, sample after
// sample), so a job's image matches aqua_render's. The lane that finishes a
// job's last pixel stamps the device clock, giving per-job latencies.
//
// Path semantics are those of the wavefront (render.cu): `Perspective`
// camera (scenes/cbox.json:516-543), Lambert + GGX `Principled`
// (scenes/cbox.json:3-62), point and area lights with power-heuristic MIS,
// Russian roulette from bounce rr_depth, `max_depth` (integrator.json:5).
#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "internal.h"
#include "shading.cuh"

namespace aq {

// Idle lanes of a warp fetch new pixels together once this many are idle
// (or all are).
constexpr int kBatchRefill = 1;

__device__ __forceinline__ unsigned long long device_clock_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The state of a lane's path between rays. A lane traces one ray per loop
// iteration: the path's extension ray (o, dir), or, when `shadow` is set,
// the shadow ray of the last vertex's light sample (from o along sdir up to
// stmax), whose contribution is added when it is unoccluded; `alive` then
// says whether the path goes on with the extension ray (o, dir) afterwards.
struct LanePath {
    v3 o, dir, thr;
    v3 so;  // shadow-ray origin when it differs from o (full model: glass)
    float pdf_b;
    int depth;
    uint64_t st, inc;
    v3 sdir, contrib;
    float stmax;
    bool shadow, alive;
};

// Camera ray of sample `sample` of `pixel`.
__device__ __forceinline__ void start_sample(const DevJob& J, uint32_t pixel, uint32_t sample, LanePath& P) {
    P.st = path_rng_state(J.seed, pixel, sample);
    P.inc = pixel_inc(pixel);
    float u0 = draw(P.st, P.inc), u1 = draw(P.st, P.inc), u2 = draw(P.st, P.inc), u3 = draw(P.st, P.inc);
    camera_ray(J.cam, pixel, u0, u1, u2, u3, P.o, P.dir);
    P.thr = mk(1.0f, 1.0f, 1.0f);
    P.pdf_b = 0.0f;
    P.depth = 0;
    P.shadow = false;
    P.alive = true;
}

// BSDF sampling and Russian roulette at shading point p: the next extension
// ray, or false when the path ends.
template <bool FULL>
__device__ __forceinline__ bool continue_path(const Bsdf& B, v3 wol, const float* u, v3 T, v3 Bt, v3 ns, v3 ng,
                                              v3 p, bool smooth, int rr_depth, LanePath& P) {
    v3 wil = bsdf_sample_t<FULL>(B, wol, u[3], u[4], u[5]);
    const bool through = FULL && wil.z < 0.0f;  // refracted by the glass lobe
    if (!((wil.z > 0.0f || through) && wol.z > 0.0f)) return false;
    float pdf = bsdf_pdf_t<FULL>(B, wol, wil);
    v3 f = bsdf_eval_t<FULL>(B, wol, wil);
    if (!(pdf > 0.0f)) return false;
    v3 thr = P.thr * f * ((FULL ? fabsf(wil.z) : wil.z) / pdf);
    bool ok = maxc(thr) > 0.0f && isfinite(thr.x) && isfinite(thr.y) && isfinite(thr.z);
    if (ok && P.depth >= rr_depth) {
        float q = fminf(1.0f, maxc(thr));
        if (u[6] >= q) ok = false;
        else thr = thr * (1.0f / q);
    }
    if (!ok) return false;
    const v3 dir = normalize(T * wil.x + Bt * wil.y + ns * wil.z);
    if (through) {
        if (!(dot(dir, ng) < 0.0f)) return false;  // refraction must cross the surface
    } else if (smooth && !(dot(dir, ng) > 0.0f)) {
        return false;  // below the geometric surface
    }
    P.thr = thr;
    P.dir = dir;
    P.o = offset_ray(p, through ? -ng : ng);
    P.pdf_b = pdf;
    P.depth = P.depth + 1;
    return true;
}

// The vertex a closest-hit ray found: emission with MIS, next-event
// estimation (schedules the shadow ray of one light sample), BSDF sampling
// and Russian roulette. Contributions are added to `sum` in the wavefront's
// order (the light sample's once its shadow ray is traced). Returns false
// when the path ends (a scheduled shadow ray is still traced).
template <bool FULL>
__device__ __forceinline__ bool shade_hit(const DevScene& S, int max_depth, int rr_depth, const float* lut,
                                          const TraceResult& h, LanePath& P, v3& sum) {
    const v3 thr = P.thr;
    const int depth = P.depth;
    if (h.tri < 0) {
        v3 e = mk(S.env[0], S.env[1], S.env[2]);
        if (e.x > 0.0f || e.y > 0.0f || e.z > 0.0f) sum = sum + thr * e;
        return false;
    }
    const float4* tw = S.tris + 3 * (size_t)h.tri;
    float4 a = ldg_(tw), b = ldg_(tw + 1), c = ldg_(tw + 2);
    uint32_t info = (uint32_t)__float_as_int(b.w);
    v3 v0 = f3(a), e1 = f3(b) - v0, e2 = f3(c) - v0;
    v3 p = v0 + e1 * h.u + e2 * h.v;
    v3 ng = normalize(cross(e1, e2));
    v3 wo = -P.dir;
    int light = (int)(info >> 16) - 1;
    if (light >= 0) {
        DevLight L = S.lights[light];
        v3 nl = normalize(cross(f3(L.e1), f3(L.e2)));
        float cos_l = dot(nl, wo);
        if (cos_l > 0.0f) {
            float w = 1.0f;
            if (depth > 0 && P.pdf_b > 0.0f) {
                float pl = L.e2.w * h.t * h.t / (L.e1.w * cos_l);
                w = power_heuristic(P.pdf_b, pl);
            }
            sum = sum + thr * f3(L.le) * w;
        }
    }
    if (depth >= max_depth) return false;
    const bool front = dot(ng, wo) >= 0.0f;  // wo on the winding normal's side
    if (!front) ng = -ng;
    const v3 ns = shading_normal(S, h.tri, h.u, h.v, ng, wo);
    DevMaterial m = S.mats[info & 0xffffu];
    v3 base = f3(m.a);
    int ti = __float_as_int(m.a.w);
    if (ti >= 0) {
        const float2* uv = S.uvs + 3 * (size_t)h.tri;
        float2 t0 = ldg_(uv), t1 = ldg_(uv + 1), t2 = ldg_(uv + 2);
        float w0 = 1.0f - h.u - h.v;
        float tu = t0.x * w0 + t1.x * h.u + t2.x * h.v;
        float tv = t0.y * w0 + t1.y * h.u + t2.y * h.v;
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
    v3 T, Bt;
    onb(ns, T, Bt);
    v3 wol = mk(dot(wo, T), dot(wo, Bt), dot(wo, ns));
    float u[kBounceDims];
#pragma unroll
    for (int k = 0; k < kBounceDims; ++k) u[k] = draw(P.st, P.inc);
    if (S.n_lights > 0 && wol.z > 0.0f) {
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
                contrib = thr * bsdf_eval_t<FULL>(B, wol, wil) * f3(L.le) * ((FULL ? fabsf(cs) : cs) / (d2 * pmf));
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
                contrib = thr * bsdf_eval_t<FULL>(B, wol, wil) * f3(L.le) * ((FULL ? fabsf(cs) : cs) * w / pl);
            }
        }
        if (contrib.x > 0.0f || contrib.y > 0.0f || contrib.z > 0.0f) {
            // The shadow ray leaves from the offset point on the light's
            // side; the extension ray sets its own origin afterwards.
            P.shadow = true;
            P.o = offset_ray(p, ng);
            if (FULL) P.so = offset_ray(p, below ? -ng : ng);
            P.sdir = wi;
            P.stmax = dist * (1.0f - 1e-4f);
            P.contrib = contrib;
        }
    }
    const bool alive = continue_path<FULL>(B, wol, u, T, Bt, ns, ng, p, S.nrm != nullptr, rr_depth, P);
    P.alive = alive;
    return alive;
}

// Persistent kernel over all jobs' pixels. counters[0] = next pixel of the
// whole batch, counters[1 + j] = finished pixels of job j. clocks[0] = launch
// time, clocks[1 + j] = completion time of job j.
// 4 resident blocks of 256 (64 registers): the spilled path state costs less
// than the latency the extra warps hide (measured on the 64-job batch: 48,
// 64 and 80 registers and the compiler's own 107 compared).
template <bool FULL, int NODES>
__global__ void __launch_bounds__(256, 4) k_batch(const DevScene* __restrict__ scenes, const DevJob* __restrict__ jobs, int njobs,
                        uint32_t total_pixels, uint32_t* __restrict__ counters,
                        unsigned long long* __restrict__ clocks, unsigned long long* __restrict__ stats) {
    __shared__ float lut[256];
    __shared__ uint32_t first_pixel[kMaxBatchJobs + 1];
    fill_srgb_lut(lut);
    for (int j = threadIdx.x; j < njobs; j += blockDim.x) first_pixel[j] = jobs[j].pixel_begin;
    if (threadIdx.x == 0) first_pixel[njobs] = total_pixels;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicCAS(&clocks[0], 0ull, device_clock_ns());
    __syncthreads();
    const unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    uint32_t n_ext = 0, n_sh = 0, n_paths = 0;
    bool have = false, drained = false;
    int job = 0;
    uint32_t pixel = 0, sample = 0;
    v3 sum = mk(0.0f, 0.0f, 0.0f);
    LanePath P;
    while (true) {
        // Idle lanes take the next pixels of the batch together.
        const unsigned idle = __ballot_sync(kFull, !have);
        if (!drained && idle != 0u && (__popc(idle) >= kBatchRefill || idle == kFull)) {
            const int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(&counters[0], (uint32_t)__popc(idle));
            base = __shfl_sync(kFull, base, leader);
            if ((uint64_t)base + (uint64_t)__popc(idle) >= (uint64_t)total_pixels) drained = true;
            if (!have) {
                const uint32_t item = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (item < total_pixels) {
                    int lo = 0, hi = njobs - 1;
                    while (lo < hi) {  // last job whose first pixel <= item
                        int mid = (lo + hi + 1) >> 1;
                        if (first_pixel[mid] <= item) lo = mid;
                        else hi = mid - 1;
                    }
                    job = lo;
                    pixel = item - first_pixel[lo];
                    sample = 0;
                    sum = mk(0.0f, 0.0f, 0.0f);
                    start_sample(jobs[job], pixel, 0, P);
                    have = true;
                }
            }
        }
        if (!__any_sync(kFull, have)) break;
        if (!have) continue;
        const DevJob& J = jobs[job];
        const DevScene& S = scenes[J.scene];
        // One ray per iteration, from one call site: the pending shadow ray,
        // else the extension ray.
        const bool any = P.shadow;
        if (any) ++n_sh;
        else ++n_ext;
        const TraceResult h = traverse_fast<NODES>(S, (FULL && any) ? P.so : P.o, any ? P.sdir : P.dir, 0.0f,
                                            any ? P.stmax : INFINITY, any);
        bool alive;
        if (any) {
            if (h.tri < 0) sum = sum + P.contrib;
            P.shadow = false;
            alive = P.alive;
        } else {
            alive = shade_hit<FULL>(S, J.max_depth, J.rr_depth, lut, h, P, sum);
            if (P.shadow) continue;
        }
        if (alive) continue;
        // The path ended: the pixel's next sample, or the pixel is done.
        if (++sample < (uint32_t)J.spp) {
            start_sample(J, pixel, sample, P);
            continue;
        }
        n_paths += (uint32_t)J.spp;
        const float inv = 1.0f / (float)J.spp;
        J.out[3 * (size_t)pixel + 0] = sum.x * inv;
        J.out[3 * (size_t)pixel + 1] = sum.y * inv;
        J.out[3 * (size_t)pixel + 2] = sum.z * inv;
        have = false;
        // Count finished pixels per job (one atomic per job among the lanes
        // finishing now); the lane that completes a job stamps the clock.
        const unsigned same = __match_any_sync(__activemask(), job);
        if (lane == __ffs(same) - 1) {
            const uint32_t k = (uint32_t)__popc(same);
            if (atomicAdd(&counters[1 + job], k) + k == J.pixels) clocks[1 + job] = device_clock_ns();
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        n_ext += __shfl_down_sync(kFull, n_ext, o);
        n_sh += __shfl_down_sync(kFull, n_sh, o);
        n_paths += __shfl_down_sync(kFull, n_paths, o);
    }
    if (lane == 0) {
        atomicAdd(&stats[0], (unsigned long long)n_paths);
        atomicAdd(&stats[1], (unsigned long long)n_ext);
        atomicAdd(&stats[2], (unsigned long long)n_sh);
    }
}

// ---------------------------------------------------------------- host side
static bool same_batch(const BatchGraph& g, const std::vector<DevJob>& jobs, const std::vector<DevScene>& scenes,
                       int block, int grid) {
    return g.exec && g.block == block && g.grid == grid && g.jobs.size() == jobs.size() &&
           g.scenes.size() == scenes.size() &&
           memcmp(g.jobs.data(), jobs.data(), jobs.size() * sizeof(DevJob)) == 0 &&
           memcmp(g.scenes.data(), scenes.data(), scenes.size() * sizeof(DevScene)) == 0;
}

void batch_release(aqua_ctx* ctx) {
    BatchGraph& g = ctx->batch;
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.graph) cudaGraphDestroy(g.graph);
    dev_free(g.buf);
    g = BatchGraph{};
}

// One persistent launch over `jobs` (graph-replayed when the job list
// repeats): device time, counters and per-job completion clocks.
struct BatchResult {
    double ms = 0.0;
    uint64_t paths = 0, ext = 0, shadow = 0;
    std::vector<unsigned long long> clocks;
};

static BatchResult launch_jobs(aqua_ctx* ctx, std::vector<DevJob>& jobs, std::vector<DevScene>& scenes,
                               uint32_t total_pixels, const aqua_tuning& tune) {
    const size_t n = jobs.size();
    int block = tune.block_trace > 0 ? tune.block_trace : 128;
    if (block != 64 && block != 128 && block != 256) throw Error(AQUA_ERR_INVALID_ARG, "block size must be 64, 128 or 256");
    bool full = false;  // some scene's materials set the full model's lobes
    for (const DevScene& sc : scenes) full = full || sc.mext != nullptr;
    bool qbvh = false;  // some scene walks quantized nodes
    for (const DevScene& sc : scenes) qbvh = qbvh || sc.qbvh != 0;
    auto kernel = full ? (qbvh ? k_batch<true, kNodesAny> : k_batch<true, kNodesFull>)
                       : (qbvh ? k_batch<false, kNodesAny> : k_batch<false, kNodesFull>);
    int per_sm = tune.blocks_per_sm;
    if (per_sm <= 0) {
        AQ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0));
        per_sm = std::max(per_sm, 1);
    }
    int grid = ctx->num_sms * per_sm;
    cudaStream_t st = ctx->stream;
    BatchGraph& g = ctx->batch;
    bool reuse = same_batch(g, jobs, scenes, block, grid) && tune.use_graph != 0;
    if (!reuse) {
        batch_release(ctx);
        size_t off = 0;
        auto take = [&](size_t b) { size_t o = off; off = (off + b + 255) / 256 * 256; return o; };
        size_t o_s = take(sizeof(DevScene) * scenes.size()), o_j = take(sizeof(DevJob) * n),
               o_c = take(4 * (n + 1)), o_t = take(8 * (n + 1)), o_st = take(8 * 4);
        dev_alloc(ctx, g.buf, off);
        char* b = (char*)g.buf.ptr;
        g.d_scenes = (DevScene*)(b + o_s);
        g.d_jobs = (DevJob*)(b + o_j);
        g.d_counters = (uint32_t*)(b + o_c);
        g.d_clocks = (unsigned long long*)(b + o_t);
        g.d_stats = (unsigned long long*)(b + o_st);
        AQ_CUDA(cudaMemcpyAsync(g.d_scenes, scenes.data(), sizeof(DevScene) * scenes.size(), cudaMemcpyHostToDevice, st));
        AQ_CUDA(cudaMemcpyAsync(g.d_jobs, jobs.data(), sizeof(DevJob) * n, cudaMemcpyHostToDevice, st));
        g.jobs = jobs;
        g.scenes = scenes;
        g.block = block;
        g.grid = grid;
        g.units = total_pixels;
        // One launch of the whole batch: counter resets + the persistent kernel.
        auto enqueue = [&](cudaStream_t s) {
            AQ_CUDA(cudaMemsetAsync(g.d_counters, 0, 4 * (n + 1), s));
            AQ_CUDA(cudaMemsetAsync(g.d_clocks, 0, 8 * (n + 1), s));
            AQ_CUDA(cudaMemsetAsync(g.d_stats, 0, 8 * 4, s));
            kernel<<<grid, block, 0, s>>>(g.d_scenes, g.d_jobs, (int)n, total_pixels, g.d_counters, g.d_clocks,
                                           g.d_stats);
            AQ_CUDA(cudaGetLastError());
        };
        if (tune.use_graph != 0) {
            AQ_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            try {
                enqueue(st);
            } catch (...) {
                cudaGraph_t tmp;
                cudaStreamEndCapture(st, &tmp);
                if (tmp) cudaGraphDestroy(tmp);
                throw;
            }
            AQ_CUDA(cudaStreamEndCapture(st, &g.graph));
            AQ_CUDA(cudaGraphInstantiate(&g.exec, g.graph, 0));
        }
    }
    EventPair ev;
    AQ_CUDA(cudaEventRecord(ev.e[0], st));
    if (g.exec) {
        AQ_CUDA(cudaGraphLaunch(g.exec, st));
    } else {
        AQ_CUDA(cudaMemsetAsync(g.d_counters, 0, 4 * (n + 1), st));
        AQ_CUDA(cudaMemsetAsync(g.d_clocks, 0, 8 * (n + 1), st));
        AQ_CUDA(cudaMemsetAsync(g.d_stats, 0, 8 * 4, st));
        kernel<<<grid, block, 0, st>>>(g.d_scenes, g.d_jobs, (int)n, total_pixels, g.d_counters, g.d_clocks,
                                        g.d_stats);
        AQ_CUDA(cudaGetLastError());
    }
    AQ_CUDA(cudaEventRecord(ev.e[1], st));
    std::vector<unsigned long long> clocks(n + 1);
    unsigned long long hs[4] = {0, 0, 0, 0};
    AQ_CUDA(cudaMemcpyAsync(clocks.data(), g.d_clocks, 8 * (n + 1), cudaMemcpyDeviceToHost, st));
    AQ_CUDA(cudaMemcpyAsync(hs, g.d_stats, 8 * 4, cudaMemcpyDeviceToHost, st));
    AQ_CUDA(cudaStreamSynchronize(st));
    const float ms = ev.ms();
    BatchResult r;
    r.ms = ms;
    r.paths = hs[0];
    r.ext = hs[1];
    r.shadow = hs[2];
    r.clocks = std::move(clocks);
    return r;
}


void render_batch(aqua_ctx* ctx, const aqua_job* in, size_t n, const aqua_tuning& tune, aqua_batch_stats* stats) {
    if (n == 0) return;
    if (n > (size_t)kMaxBatchJobs) throw Error(AQUA_ERR_INVALID_ARG, "at most 1024 jobs per batch");
    std::vector<DevScene> scenes;
    std::map<const aqua_scene*, int> scene_index;
    std::vector<DevJob> jobs(n);
    uint32_t total_pixels = 0;
    for (size_t i = 0; i < n; ++i) {
        const aqua_job& j = in[i];
        if (!j.scene || !j.rgb_out) throw Error(AQUA_ERR_INVALID_ARG, "job " + std::to_string(i) + ": scene and rgb_out must be non-NULL");
        if (j.width <= 0 || j.height <= 0 || j.width > 16384 || j.height > 16384)
            throw Error(AQUA_ERR_INVALID_ARG, "job " + std::to_string(i) + ": resolution out of range");
        if (j.spp <= 0 || j.max_depth < 0 || j.max_depth > 250)
            throw Error(AQUA_ERR_INVALID_ARG, "job " + std::to_string(i) + ": spp must be > 0 and max_depth in [0, 250]");
        if (((uintptr_t)j.rgb_out & 3) != 0) throw Error(AQUA_ERR_INVALID_ARG, "rgb_out must be 4-byte aligned");
        auto it = scene_index.find(j.scene);
        int si;
        if (it == scene_index.end()) {
            si = (int)scenes.size();
            scene_index[j.scene] = si;
            scenes.push_back(j.scene->ds);
        } else {
            si = it->second;
        }
        aqua_camera cam = j.scene->host.cam;
        cam.width = j.width;
        cam.height = j.height;
        DevJob& d = jobs[i];
        memset(&d, 0, sizeof(d));
        d.cam = dev_camera(cam);
        d.out = j.rgb_out;
        d.seed = j.seed;
        d.scene = si;
        d.spp = j.spp;
        d.max_depth = j.max_depth;
        d.rr_depth = 3;
        d.pixels = (uint32_t)j.width * (uint32_t)j.height;
    }
    // Shortest job first: the kernel hands out pixels in the order of the
    // device job list, so ordering it by work (pixels x spp) lets small jobs
    // finish early without changing any job's image. rank[i] = position of
    // input job i.
    std::vector<size_t> order(n), rank(n);
    for (size_t i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        return (uint64_t)jobs[a].pixels * (uint64_t)jobs[a].spp < (uint64_t)jobs[b].pixels * (uint64_t)jobs[b].spp;
    });
    std::vector<DevJob> sorted(n);
    for (size_t k = 0; k < n; ++k) {
        sorted[k] = jobs[order[k]];
        rank[order[k]] = k;
        sorted[k].pixel_begin = total_pixels;
        if ((uint64_t)total_pixels + sorted[k].pixels > 0xFFFFFF00ull)
            throw Error(AQUA_ERR_INVALID_ARG, "a batch holds at most 2^32 - 256 pixels");
        total_pixels += sorted[k].pixels;
    }
    BatchResult r = launch_jobs(ctx, sorted, scenes, total_pixels, tune);
    if (stats) {
        stats->device_ms = r.ms;
        stats->paths = r.paths;
        if (stats->job_ms)
            for (size_t i = 0; i < n; ++i) {
                const unsigned long long c = r.clocks[1 + rank[i]];
                stats->job_ms[i] = c >= r.clocks[0] ? (double)(c - r.clocks[0]) * 1e-6 : -1.0;
            }
    }
}

void render_persistent(aqua_ctx* ctx, aqua_scene* sc, const aqua_integrator_cfg& cfg, const aqua_tuning& tune,
                       float* rgb_out, uint32_t flags, aqua_stats* stats) {
    if (cfg.spp <= 0) throw Error(AQUA_ERR_INVALID_ARG, "spp must be positive");
    check_depths(cfg.max_depth, cfg.rr_depth);
    const aqua_camera& cam = sc->host.cam;
    const size_t pixels = (size_t)cam.width * (size_t)cam.height;
    if (pixels == 0 || pixels > 0xFFFFFF00ull) throw Error(AQUA_ERR_INVALID_ARG, "image size out of range");
    const bool device_film = (flags & AQUA_RENDER_DEVICE_FILM) != 0;
    float* film = rgb_out;
    if (!device_film) {
        if (ctx->persist_film.bytes < 12 * pixels) {
            dev_free(ctx->persist_film);
            dev_alloc(ctx, ctx->persist_film, 12 * pixels);
        }
        film = (float*)ctx->persist_film.ptr;
    } else if (((uintptr_t)rgb_out & 3) != 0) {
        throw Error(AQUA_ERR_INVALID_ARG, "rgb_out must be 4-byte aligned");
    }
    std::vector<DevScene> scenes{sc->ds};
    std::vector<DevJob> jobs(1);
    DevJob& d = jobs[0];
    memset(&d, 0, sizeof(d));
    d.cam = dev_camera(cam);
    d.out = film;
    d.seed = cfg.seed;
    d.scene = 0;
    d.spp = cfg.spp;
    d.max_depth = cfg.max_depth;
    d.rr_depth = cfg.rr_depth;
    d.pixels = (uint32_t)pixels;
    d.pixel_begin = 0;
    BatchResult r = launch_jobs(ctx, jobs, scenes, (uint32_t)pixels, tune);
    if (!device_film) {
        AQ_CUDA(cudaMemcpyAsync(rgb_out, film, 12 * pixels, cudaMemcpyDeviceToHost, ctx->stream));
        AQ_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->paths = r.paths;
        stats->ext_rays = r.ext;
        stats->shadow_rays = r.shadow;
        stats->device_ms = r.ms;
        stats->total_launches = 1;
    }
}

}  // namespace aq
