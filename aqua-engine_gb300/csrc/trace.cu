// trace.cu — aqua_trace: closest-hit or any-hit queries for a caller's ray
// set. This is the traversal the parity tests compare, ray for ray, with the
// FP32 CPU traversal of the same flattened BVH.
#include <algorithm>
#include <cstring>

#include "internal.h"

namespace aq {

template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(128) k_trace_user(DevScene S, const float4* __restrict__ rays, size_t n,
                                                    float4* __restrict__ hits, unsigned long long* stats) {
    uint32_t nodes = 0, tris = 0;
    auto store = [&](size_t i, const TraceResult& r) {
        float4 h;
        if (ANY) h = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(r.tri >= 0 ? 1 : -1));
        else if (r.tri < 0) h = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
        else h = make_float4(r.t, r.u, r.v, __int_as_float(r.id));
        hits[i] = h;
    };
    if (!COUNT && n < (1ull << 31)) {
        // The renderer's traversal: persistent lanes with ray replacement;
        // stats[2] is the queue cursor.
        traverse_queue<ANY>(
            S, (uint32_t)n, reinterpret_cast<uint32_t*>(stats + 2),
            [&](uint32_t i, v3& o, v3& d, float& tmin, float& tmax) -> uint32_t {
                float4 a = ldg_(rays + 2 * (size_t)i), b = ldg_(rays + 2 * (size_t)i + 1);
                o = mk(a.x, a.y, a.z);
                d = mk(b.x, b.y, b.z);
                tmin = a.w;
                tmax = b.w;
                return i;
            },
            store);
        return;
    }
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float4 a = ldg_(rays + 2 * i), b = ldg_(rays + 2 * i + 1);
        store(i, COUNT ? traverse<ANY, true>(S, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), a.w, b.w, nodes, tris)
                       : traverse_fast(S, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), a.w, b.w, ANY));
    }
    if (COUNT) {
        for (int o = 16; o > 0; o >>= 1) {
            nodes += __shfl_down_sync(0xffffffffu, nodes, o);
            tris += __shfl_down_sync(0xffffffffu, tris, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&stats[0], (unsigned long long)nodes);
            atomicAdd(&stats[1], (unsigned long long)tris);
        }
    }
}

void trace_rays(aqua_ctx* ctx, aqua_scene* sc, const aqua_ray* rays, size_t n, aqua_hit* out, uint32_t flags,
                aqua_trace_counts* counts) {
    static_assert(sizeof(aqua_ray) == 32, "aqua_ray must be 32 bytes");
    static_assert(sizeof(aqua_hit) == 16, "aqua_hit must be 16 bytes");
    cudaStream_t st = ctx->stream;
    bool dev = (flags & AQUA_TRACE_DEVICE_PTRS) != 0;
    bool any = (flags & AQUA_TRACE_ANY_HIT) != 0;
    bool count = (flags & AQUA_TRACE_COUNT) != 0;
    if (counts) memset(counts, 0, sizeof(*counts));
    if (n == 0) return;
    const float4* d_rays;
    float4* d_hits;
    if (dev) {
        if (((uintptr_t)rays & 15) || ((uintptr_t)out & 15))
            throw Error(AQUA_ERR_INVALID_ARG, "device ray and hit arrays must be 16-byte aligned");
        d_rays = (const float4*)rays;
        d_hits = (float4*)out;
    } else {
        if (ctx->trace_rays.bytes < 32 * n) { dev_free(ctx->trace_rays); dev_alloc(ctx, ctx->trace_rays, 32 * n); }
        if (ctx->trace_hits.bytes < 16 * n) { dev_free(ctx->trace_hits); dev_alloc(ctx, ctx->trace_hits, 16 * n); }
        AQ_CUDA(cudaMemcpyAsync(ctx->trace_rays.ptr, rays, 32 * n, cudaMemcpyHostToDevice, st));
        d_rays = (const float4*)ctx->trace_rays.ptr;
        d_hits = (float4*)ctx->trace_hits.ptr;
    }
    if (!ctx->trace_stats.ptr) dev_alloc(ctx, ctx->trace_stats, 64);
    unsigned long long* d_stats = (unsigned long long*)ctx->trace_stats.ptr;
    AQ_CUDA(cudaMemsetAsync(d_stats, 0, 24, st));  // node and triangle counters, queue cursor
    auto k = any ? (count ? k_trace_user<true, true> : k_trace_user<true, false>)
                 : (count ? k_trace_user<false, true> : k_trace_user<false, false>);
    int per_sm = 1;
    AQ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 128, 0));
    size_t need = (n + 127) / 128;
    int grid = (int)std::min<size_t>(need, (size_t)ctx->num_sms * (size_t)std::max(per_sm, 1));
    EventPair ev;
    AQ_CUDA(cudaEventRecord(ev.e[0], st));
    k<<<grid, 128, 0, st>>>(sc->ds, d_rays, n, d_hits, d_stats);
    AQ_CUDA(cudaGetLastError());
    AQ_CUDA(cudaEventRecord(ev.e[1], st));
    if (!dev) AQ_CUDA(cudaMemcpyAsync(out, d_hits, 16 * n, cudaMemcpyDeviceToHost, st));
    unsigned long long hs[2] = {0, 0};
    if (counts) AQ_CUDA(cudaMemcpyAsync(hs, d_stats, 16, cudaMemcpyDeviceToHost, st));
    AQ_CUDA(cudaStreamSynchronize(st));
    const float ms = ev.ms();
    if (counts) {
        counts->node_visits = hs[0];
        counts->tri_tests = hs[1];
        counts->kernel_ms = ms;
    }
}

}  // namespace aq
