// internal.h — the opaque handles behind the C ABI and the entry points the
// CUDA translation units export to the ABI layer.
#pragma once

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/aqua.h"
#include "bvh.h"
#include "device.cuh"
#include "scene.h"

namespace aq {

// Error carrying an aqua_status across internal layers; the ABI layer turns
// it into a return code and aqua_last_error text.
struct Error : std::runtime_error {
    aqua_status status;
    Error(aqua_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

// Depth limits shared by every render entry point. A path's depth lives in
// the low 8 bits of its state word (one more than max_depth is stored after
// the last bounce), so max_depth stays at or below 250; rr_depth is a bounce
// index in the same range (a value above max_depth turns roulette off).
inline void check_depths(int32_t max_depth, int32_t rr_depth) {
    if (max_depth < 0 || max_depth > 250) throw Error(AQUA_ERR_INVALID_ARG, "max_depth must be in [0, 250]");
    if (rr_depth < 0 || rr_depth > 250) throw Error(AQUA_ERR_INVALID_ARG, "rr_depth must be in [0, 250]");
}

#define AQ_CUDA(call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            throw ::aq::Error(e_ == cudaErrorMemoryAllocation ? AQUA_ERR_OOM : AQUA_ERR_CUDA,  \
                              std::string(#call) + ": " + cudaGetErrorString(e_));             \
    } while (0)

// A pair of CUDA events for timing one stretch of a stream, destroyed with
// the object (also when a CUDA call in between throws).
struct EventPair {
    cudaEvent_t e[2] = {nullptr, nullptr};
    EventPair() {
        cudaError_t r = cudaEventCreate(&e[0]);
        if (r == cudaSuccess) r = cudaEventCreate(&e[1]);
        if (r != cudaSuccess) {
            if (e[0]) cudaEventDestroy(e[0]);
            AQ_CUDA(r);
        }
    }
    ~EventPair() {
        for (auto x : e)
            if (x) cudaEventDestroy(x);
    }
    EventPair(const EventPair&) = delete;
    EventPair& operator=(const EventPair&) = delete;
    float ms() const {
        float t = 0.0f;
        AQ_CUDA(cudaEventElapsedTime(&t, e[0], e[1]));
        return t;
    }
};

#if defined(__CUDACC__)
// Launches kernel k chained to the previous work in stream st (programmatic
// dependent launch): its blocks may be scheduled while the previous kernel's
// last blocks drain, and it waits for that kernel (grid_dep_wait) before its
// first dependent read. Hides the launch gap between dependent kernels.
template <class... KArgs, class... Args>
void launch_chained(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t lc = {};
    lc.gridDim = grid;
    lc.blockDim = block;
    lc.dynamicSmemBytes = smem;
    lc.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    AQ_CUDA(cudaLaunchKernelEx(&lc, k, args...));
}
#endif

// Device buffer owned by a context; size in bytes.
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
};

// Render workspace: path state and queues of the wavefront, sized on demand.
struct Workspace {
    size_t slots = 0;       // capacity in path slots
    size_t buckets = 0;     // material buckets (materials + 1 for misses)
    size_t pixels = 0;      // film capacity
    DevBuf block;           // one allocation, carved below
    float4* ray_o = nullptr;  // (o.xyz, tmin)
    float4* ray_d = nullptr;  // (d.xyz, tmax)
    float4* hit = nullptr;    // (t, u, v, leaf-order tri or -1)
    float4* tp = nullptr;     // (throughput.rgb, pdf of the last BSDF sample)
    uint4* pst = nullptr;     // (rng lo, rng hi, work index, depth)
    uint32_t* q[2] = {nullptr, nullptr};
    uint32_t* bucket = nullptr;  // buckets x slots
    float4* sh_o = nullptr;   // (o.xyz, pixel bits)
    float4* sh_d = nullptr;   // (d.xyz, tmax)
    float4* sh_c = nullptr;   // (contribution.rgb, 0)
    float4* film = nullptr;   // per-pixel sum
    uint32_t* counters = nullptr;   // see kCnt*
    unsigned long long* stats = nullptr;  // see kStat*
    float* out_rgb = nullptr;  // staging for host films (pixels * 3)
};

// Radiance-cache network: FP32 master weights + Adam state, bf16 fragment
// tables for the tensor-core kernels, and training scratch.
struct NrcNet {
    DevBuf block;            // weights, Adam moments, gradient, fragments, loss
    float* w = nullptr;      // master weights [W1..W5 64x64, W6 3x64]
    float* m = nullptr;
    float* v = nullptr;
    float* grad = nullptr;   // last step's gradient
    uint2* frag = nullptr;   // forward B fragments
    uint2* fragT = nullptr;  // backward B fragments
    double* loss = nullptr;  // loss sum of the last step
    float* ema = nullptr;    // exponential moving average of w (inference weights)
    uint2* frag_inf = nullptr;  // forward fragments of the inference weights
    uint8_t* img_tc = nullptr;  // inference weights in the tcgen05 shared-memory layout
    uint8_t* img_tc_w = nullptr;  // the trained weights w in that layout (training forward)
    uint8_t* img_tc_bwd = nullptr;  // W6^T, W5^T..W2^T of w in that layout (backward)
    uint32_t* tc_err = nullptr; // set by the tcgen05 kernel when a wait expired
    int forward_tc = 0;         // 1: inference runs on tcgen05 (else mma.sync)
    float ema_decay = 0.0f;  // 0 = inference uses w itself
    DevBuf train;            // training scratch, sized by train_rows
    int train_rows = 0;
    float* ty = nullptr;       // forward outputs (rows x 3)
    uint32_t* acts = nullptr;  // H1..H5 bf16 (5 x rows x 64)
    uint32_t* deltas = nullptr;// delta1..delta5 bf16 (5 x rows x 64)
    uint32_t* d6 = nullptr;    // dY bf16 (rows x 16)
    float* partial = nullptr;  // per-chunk weight gradients
    int64_t step = 0;
    float lr = 1e-2f, beta1 = 0.9f, beta2 = 0.99f, eps = 1e-8f;
    float bmin[3] = {0, 0, 0}, bext[3] = {1, 1, 1};
    uint64_t launches = 0;
    double train_frac = 0.0;  // fraction of paths that train, adapted per frame
};

// Per-context buffers of a radiance-cache frame.
struct NrcWorkspace {
    DevBuf block;
    size_t queries = 0, records = 0;  // capacities
    float4* q_pix = nullptr;     // (pixel bits, throughput) per query
    float* q_raw = nullptr;      // 16 raw features per query
    uint16_t* q_x = nullptr;     // encoded queries (bf16 x 64)
    float* q_pred = nullptr;     // cache output per query
    float4* rec = nullptr;       // training-vertex records (6 words each)
    float4* ltrain = nullptr;    // radiance per training path
    float4* lsnap = nullptr;     // per training path and bounce: radiance before it
    float2* spread = nullptr;    // per path slot: path-spread sum and a0
    size_t snaps = 0;            // bounces per training path (capacity)
    float* t_raw = nullptr;      // permuted training features
    uint16_t* t_x = nullptr;     // encoded training inputs
    float* t_target = nullptr;   // training targets
};

// Batched rendering (batch.cu): one job as the persistent kernel sees it.
constexpr int kMaxBatchJobs = 1024;
struct DevJob {
    DevCamera cam;           // the scene's camera at the job's resolution
    float* out;              // width * height * 3 floats
    uint64_t seed;
    int32_t scene, spp, max_depth, rr_depth;
    uint32_t pixels, pixel_begin;    // pixels of the job, its first pixel in the batch
};

// The last batch, kept so an identical batch replays its CUDA graph.
struct BatchGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    DevBuf buf;
    DevScene* d_scenes = nullptr;
    DevJob* d_jobs = nullptr;
    uint32_t* d_counters = nullptr;
    unsigned long long* d_clocks = nullptr;
    unsigned long long* d_stats = nullptr;
    std::vector<DevJob> jobs;
    std::vector<DevScene> scenes;
    int block = 0, grid = 0;
    uint32_t units = 0;
};

enum { kCntQ0 = 0, kCntQ1 = 1, kCntShadow = 2, kCntBucket0 = 10 };
enum { kStatExt = 0, kStatShadow, kStatPaths, kStatNodes, kStatTris, kStatShNodes, kStatShTris, kStatCount };

}  // namespace aq

struct aqua_scene {
    aq::HostScene host;
    aq::FlatBvh bvh;
    std::vector<float> qnodes;         // quantized copy of bvh (kBvhQNodeFloats per node)
    int32_t bvh_format = AQUA_BVH_AUTO;  // requested node format
    int32_t bvh_format_used = AQUA_BVH_FULL;  // the format of the device image
    void* pinned = nullptr;    // staged device image of the scene
    bool pinned_is_cuda = false;
    size_t bytes = 0;          // bytes of the device image
    aq::DevBuf dev;            // device copy
    aq::DevScene ds{};         // pointers into dev
    bool uploaded = false;
};

struct aqua_nrc {
    aq::NrcNet net;
    aq::DevBuf stage_in, stage_tgt, stage_out;  // staging for host-pointer calls
    float last_ms = 0.0f;                        // device time of the last AQUA_NRC_TIMING call
};

struct aqua_ctx {
    int device = 0;
    bool host_only = false;    // AQUA_DEVICE_HOST_ONLY: loaders and exports only
    int num_sms = 0;
    int verbose = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    uint64_t alloc_count = 0;
    uint64_t fail_alloc_after = 0;
    aq::Workspace ws;
    aq::NrcWorkspace nrc_ws;
    aq::BatchGraph batch;
    unsigned int* pinned_counter = nullptr;  // host-mapped copy of queue counts
    std::vector<cudaEvent_t> events;         // pool for stage timing
    aq::DevBuf trace_rays, trace_hits;       // staging for host-pointer traces
    aq::DevBuf persist_film;                 // device film of host-film persistent renders
    bool nrc_tc_ready = false;               // tcgen05 inference kernel configured on this device
    bool nrc_tc_bwd_ready = false;           // and the tcgen05 backward kernel
    bool nrc_tc_wg_ready = false;            // and the tcgen05 weight-gradient kernel
    aq::DevBuf trace_stats;
};

namespace aq {

// Device allocation through the context (honours the fail_alloc_after hook).
void dev_alloc(aqua_ctx* ctx, DevBuf& b, size_t bytes);
void dev_free(DevBuf& b);

// Builds the device image of a scene (BVH, triangle words, materials,
// lights, textures) in pinned memory and copies it to the device.
// Quantized nodes are chosen automatically above this many bytes of
// full-precision nodes (8 GiB): on GB300 the decode's extra instructions
// cost more than the halved node bytes save (the 1.15M-triangle interior
// traced 7% slower, the 4.0M-triangle sphere field 5%), so they pay only
// where the tree's memory footprint matters.
constexpr size_t kQuantizeAbove = (size_t)8 << 30;
void scene_build_device(aqua_ctx* ctx, aqua_scene* s, bool rebuild_bvh = true);
void scene_upload(aqua_ctx* ctx, aqua_scene* s);
void scene_release(aqua_scene* s);
DevCamera dev_camera(const aqua_camera& c);

void trace_rays(aqua_ctx* ctx, aqua_scene* s, const aqua_ray* rays, size_t n, aqua_hit* out,
                uint32_t flags, aqua_trace_counts* counts);
void render_path(aqua_ctx* ctx, aqua_scene* s, const aqua_integrator_cfg& cfg, const aqua_tuning& tune,
                 float* rgb_out, uint32_t flags, aqua_stats* stats);
void workspace_release(aqua_ctx* ctx);
// One frame of the cached renderer (render.cu): wavefront with cache
// queries and training paths, inference, online training.
void render_nrc(aqua_ctx* ctx, aqua_scene* s, const aqua_integrator_cfg& cfg, const aqua_tuning& tune,
                aqua_nrc* nrc, float* rgb_out, uint32_t flags, aqua_stats* stats);

// Batched rendering (batch.cu).
void render_batch(aqua_ctx* ctx, const aqua_job* jobs, size_t n, const aqua_tuning& tune, aqua_batch_stats* stats);
// One image with the batch kernel (AQUA_KERNEL_PERSISTENT).
void render_persistent(aqua_ctx* ctx, aqua_scene* s, const aqua_integrator_cfg& cfg, const aqua_tuning& tune,
                       float* rgb_out, uint32_t flags, aqua_stats* stats);
void batch_release(aqua_ctx* ctx);

// Radiance-cache network (nrc.cu).
void nrc_alloc(aqua_ctx* ctx, NrcNet& net);
void nrc_release(NrcNet& net);
void nrc_init_weights(aqua_ctx* ctx, NrcNet& net, uint64_t seed);
void nrc_set_weights(aqua_ctx* ctx, NrcNet& net, const float* host_w);
void nrc_pack(aqua_ctx* ctx, NrcNet& net);
void nrc_forward_dev(aqua_ctx* ctx, NrcNet& net, const uint16_t* X, int n, float* out);
void nrc_train_step_dev(aqua_ctx* ctx, NrcNet& net, const uint16_t* X, const float* target, int n);
void nrc_encode_dev(aqua_ctx* ctx, NrcNet& net, const float* raw, int n, uint16_t* X);
// tcgen05 inference (nrc_tc.cu)
size_t nrc_tc_weight_bytes();
// All three tcgen05 weight images: forward of w and of inf, backward of w.
void nrc_pack_tc(aqua_ctx* ctx, const float* w, const float* inf, void* img_w, void* img_inf, void* img_bwd);
void nrc_forward_tc_dev(aqua_ctx* ctx, const void* img, const uint16_t* X, int n, float* out, uint32_t* err,
                        uint32_t* acts = nullptr, double* loss_zero = nullptr);
size_t nrc_tc_bwd_bytes();
void nrc_backward_tc_dev(aqua_ctx* ctx, const void* img, const float* Y, const float* T, int n, float inv_count,
                         const uint32_t* acts, uint32_t* deltas, uint32_t* d6, double* loss, uint32_t* err);
// Weight gradients of one training batch on tcgen05: per-chunk partials
// (chunk-major, kNrcParams each) for the Adam kernel; returns the chunk count.
int nrc_wgrad_tc_dev(aqua_ctx* ctx, const uint16_t* X, const uint32_t* acts, const uint32_t* deltas,
                     const uint32_t* d6, int n, float* partial, uint32_t* err);
// Throws when a tcgen05 launch since the last check gave up waiting (syncs the stream).
void nrc_check_tc(aqua_ctx* ctx, NrcNet& net);

// Render on the library's fixed static scratch array; no device allocation.
void render_noalloc(aqua_ctx* ctx, aqua_scene* s, const aqua_integrator_cfg& cfg, float* rgb_out,
                    aqua_stats* stats);
size_t render_noalloc_max_pixels();

}  // namespace aq
