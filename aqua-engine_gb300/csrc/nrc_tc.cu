// nrc_tc.cu — radiance-cache inference on the 5th-generation tensor cores:
// tcgen05.mma with the accumulator in tensor memory (TMEM), inputs brought in
// by TMA.
//
// One persistent CTA per SM holds the network's bf16 weights (42 KB) in shared
// memory once and runs kTcFwdGroups independent warpgroups. A warpgroup owns
// 96 TMEM columns (64 for the FP32 accumulator, 32 for the next layer's bf16
// activations; five groups fill 480 of the SM's 512) and a 128-row input
// tile in shared memory, and works through its tiles alone:
//   - its first thread loads the next input tile with TMA (eight 128 x 8-column
//     boxes) as soon as layer 1 has read the current one;
//   - per layer the same thread issues four tcgen05.mma.kind::f16 (M = 128,
//     N = 64, or 16 for the output layer, K = 16 each; BF16 x BF16 -> FP32)
//     and commits them to the group's mbarrier. Layer 1 reads A from shared
//     memory, layers 2-6 read it from TMEM;
//   - each warp reads its 32 TMEM lanes (rows) of the accumulator with
//     tcgen05.ld, applies ReLU, rounds to bf16 pairs and stores them back to
//     the activation columns with tcgen05.st.
// Activations never leave TMEM, and while one group is in its epilogue the
// tensor core serves the others.
//
// Shared-memory operands use the K-major layout without swizzle, with the
// 8-row x 16-byte core matrices of one 8-column K slice stored back to back:
// element (r, k) of an R-row tile sits at (k / 8) * R * 16 + r * 16 + (k % 8) * 2.
// So the leading byte offset (next core matrix along K) is R * 16 and the
// stride byte offset (next 8 rows) is 128, and a TMA box of 8 columns x 128
// rows lands as one contiguous K slice.
//
// Every mbarrier wait is bounded. A group whose wait expires agrees on it
// with a barrier reduction, records an error flag, waits (bounded) for what
// it still has in flight and leaves; TMEM is freed on every path.
#include <algorithm>
#include <mutex>

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "internal.h"
#include "nrc.h"

namespace aq {

constexpr int kTcRows = 128;                      // rows per tile (MMA M)
constexpr int kTcGroups = 4;                      // warpgroups (tiles in flight) per CTA, training kernels
constexpr int kTcThreads = 128 * kTcGroups;
constexpr int kTcTileBytes = kTcRows * 64 * 2;    // 16 KB per input or activation tile
constexpr int kTcLayerBytes = kNrcTcLayerBytes;  // 8 KB hidden-layer weights
constexpr int kTcOutRows = kNrcTcOutRows;        // output layer padded to N = 16 (3 used)
constexpr int kTcOutBytes = kTcOutRows * 64 * 2;  // 2 KB
constexpr int kTcWeightBytes = 5 * kTcLayerBytes + kTcOutBytes;  // 42 KB
constexpr uint32_t kTcGroupCols = 128;            // accumulator 64 + activations 32, rounded up
constexpr uint32_t kTcActCol = 64;                // activation columns within a group
constexpr uint32_t kTcTmemCols = kTcGroupCols * kTcGroups;  // a power of two >= 32
constexpr uint32_t kTcWaitLimit = 1u << 22;       // try_wait rounds before a wait gives up
// Inference: five groups (tiles in flight; four measured 9% slower),
// accumulators at columns 64 g, activations after all accumulators at
// 64 * 5 + 32 g. The weights and five input tiles take 123 KB of shared
// memory, which keeps two CTAs (and two full TMEM allocations) off one SM.
constexpr int kTcFwdGroups = 5;
constexpr int kTcFwdThreads = 128 * kTcFwdGroups;
constexpr int kTcFwdSmemBytes = std::max(kTcWeightBytes + kTcFwdGroups * kTcTileBytes + 1024, 120 * 1024);
constexpr uint32_t kTcFwdActBase = 64u * kTcFwdGroups;
static_assert(kTcFwdActBase + 32u * kTcFwdGroups <= kTcTmemCols, "inference TMEM columns");
static_assert(kTcFwdSmemBytes <= 227 * 1024, "shared memory per CTA");
static_assert((kTcTmemCols & (kTcTmemCols - 1)) == 0 && kTcTmemCols >= 32 && kTcTmemCols <= 512, "TMEM alloc");
static_assert(kTcWeightBytes % 1024 == 0 && kTcTileBytes % 1024 == 0, "tiles stay 1024-byte aligned");

// Byte offset of element (r, k) in an R-row operand tile.
__host__ __device__ constexpr uint32_t tc_offset(int rows, int r, int k) { return nrc_tc_offset(rows, r, k); }

// All three weight images from the FP32 weights w and the inference
// weights inf (nrc_tc_param_offsets; the caller zeroes the padding first):
// forward images of w (training) and of inf (inference), backward image of w.
__global__ void k_nrc_pack_tc(const float* __restrict__ w, const float* __restrict__ inf, uint8_t* __restrict__ img_w,
                              uint8_t* __restrict__ img_inf, uint8_t* __restrict__ img_bwd) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;  // one parameter
    if (p >= kNrcParams) return;
    uint32_t fwd;
    int32_t bwd;
    nrc_tc_param_offsets(p, fwd, bwd);
    const __nv_bfloat16 b = __float2bfloat16_rn(w[p]);
    *reinterpret_cast<__nv_bfloat16*>(img_w + fwd) = b;
    *reinterpret_cast<__nv_bfloat16*>(img_inf + fwd) = __float2bfloat16_rn(inf[p]);
    if (bwd >= 0) *reinterpret_cast<__nv_bfloat16*>(img_bwd + bwd) = b;
}

// ---------------------------------------------------------------- PTX wrappers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start address, leading byte offset (next
// core matrix along K), stride byte offset (next 8 rows), all >> 4; bit 46 =
// descriptor version 1; swizzle none.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)(128u >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::f16: D = F32 (bits 4-5), A = B = BF16 (bits
// 7-9, 10-12), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t tc_idesc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// Same with A (128 rows x 16 bf16, two per 32-bit column) read from TMEM.
__device__ __forceinline__ void tc_mma_ts(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n"
        "}\n" ::"r"(tmem_d),
        "r"(tmem_a), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                 : "memory");
}

// Bounded wait on an mbarrier phase; false when the limit expired.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (uint32_t it = 0; it < kTcWaitLimit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n"
            ".reg .pred p;\n"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n"
            "}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Barrier over one warpgroup (named barrier `id`, 128 threads) that also
// returns whether any of its threads passed `pred`.
__device__ __forceinline__ bool group_any(int id, bool pred) {
    uint32_t r;
    asm volatile(
        "{\n"
        ".reg .pred p, q;\n"
        "setp.ne.u32 p, %1, 0;\n"
        "bar.red.or.pred q, %2, 128, p;\n"
        "selp.u32 %0, 1, 0, q;\n"
        "}\n"
        : "=r"(r)
        : "r"((uint32_t)pred), "r"(id)
        : "memory");
    return r != 0;
}

// Barrier over one warpgroup (named barrier `id`, 128 threads).
__device__ __forceinline__ void group_sync(int id) { asm volatile("bar.sync %0, 128;\n" ::"r"(id) : "memory"); }

// One input tile: eight boxes of 8 columns x 128 rows, 16 KB on one mbarrier.
__device__ __forceinline__ void tma_load_tile(const CUtensorMap* map, uint32_t dst, uint32_t mbar, int row0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mbar), "r"((uint32_t)kTcTileBytes)
                 : "memory");
#pragma unroll
    for (int kc = 0; kc < 8; ++kc)
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
                dst + (uint32_t)(kc * kTcRows * 16)),
            "l"(reinterpret_cast<uint64_t>(map)), "r"(kc * 8), "r"(row0), "r"(mbar)
            : "memory");
}

#define AQ_TC_LD16(taddr, r)                                                                               \
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, " \
                 "[%16];\n"                                                                                \
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),     \
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), \
                   "=r"(r[14]), "=r"(r[15])                                                                \
                 : "r"(taddr))

#define AQ_TC_ST16(taddr, r)                                                                               \
    asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "                                          \
                 "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};\n" ::"r"(taddr),              \
                 "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),    \
                 "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]) \
                 : "memory")

__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }
__device__ __forceinline__ void tc_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// ReLU and round-to-nearest-even to a bf16 pair: `lo` (the even K index) in
// the low half, `hi` in the high half.
__device__ __forceinline__ uint32_t relu_pack2(uint32_t lo, uint32_t hi) {
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;\n" : "=r"(d) : "f"(__uint_as_float(hi)), "f"(__uint_as_float(lo)));
    return d;
}

// ---------------------------------------------------------------- kernel
// X (through `xmap`): n rows x 64 bf16; out: n x 3 fp32; err: set to 1 when a
// wait expired. acts (training, may be null): the hidden activations H1..H5
// as bf16 rows, acts[l][row][64], for the backward pass.
__global__ void __launch_bounds__(kTcFwdThreads, 1)
    k_nrc_forward_tc(const __grid_constant__ CUtensorMap xmap, int n, const uint4* __restrict__ wimg,
                     float* __restrict__ out, uint32_t* __restrict__ err, uint4* __restrict__ acts,
                     double* __restrict__ loss_zero) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t bar_in[kTcFwdGroups], bar_mma[kTcFwdGroups];
    __shared__ uint32_t tmem_base_slot;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = warp >> 2, q = warp & 3, gt = tid & 127;
    const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
    uint8_t* sbase = smem_raw + (base - smem_u32(smem_raw));
    const uint32_t sW = base;
    const uint32_t sI = base + kTcWeightBytes + (uint32_t)g * kTcTileBytes;  // this group's input tile

    grid_dep_wait();  // the weights and inputs come from the kernels before
    grid_dep_launch();
    if (loss_zero && blockIdx.x == 0 && tid == 0) *loss_zero = 0.0;  // the training step's loss word
    for (int i = tid; i < kTcWeightBytes / 16; i += kTcFwdThreads) reinterpret_cast<uint4*>(sbase)[i] = __ldcg(wimg + i);
    if (tid < kTcFwdGroups) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&bar_in[tid])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&bar_mma[tid])) : "memory");
    }
    if (tid == 0) {
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&xmap)) : "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         smem_u32(&tmem_base_slot)),
                     "r"(kTcTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();

    const uint32_t tmem = tmem_base_slot + (uint32_t)g * 64u;                    // this group's accumulator
    const uint32_t tact = tmem_base_slot + kTcFwdActBase + (uint32_t)g * 32u;   // and activations
    const uint32_t lanes = (uint32_t)(q * 32) << 16;                             // this warp's lanes
    const uint32_t mb_in = smem_u32(&bar_in[g]), mb_mma = smem_u32(&bar_mma[g]);
    const int bar_id = 1 + g;
    const int tiles = (n + kTcRows - 1) / kTcRows;
    const int stride = (int)gridDim.x * kTcFwdGroups;
    const int row = q * 32 + lane;  // TMEM lane = tile row
    uint32_t ph_in = 0, ph_mma = 0;      // parity of the next phase to wait for
    uint32_t tma_par = 0, mma_par = 0;   // parity the work in flight will complete
    bool fail = false, tma_pending = false, mma_pending = false;

    // Tiles interleave across CTAs first, so a small batch still spreads
    // over many SMs.
    int tile = (int)blockIdx.x + g * (int)gridDim.x;
    if (gt == 0 && tile < tiles) {
        tma_load_tile(&xmap, sI, mb_in, tile * kTcRows);
        tma_pending = true;
        tma_par = ph_in;
    }
    while (tile < tiles) {
        bool ok = true;
        if (gt == 0) {
            ok = mbar_wait(mb_in, ph_in);
            if (ok) tma_pending = false;
        }
        ph_in ^= 1u;
        if (group_any(bar_id, !ok)) { fail = true; break; }
        const int next = tile + stride;
        for (int l = 0; l < 6; ++l) {
            const bool last = l == 5;
            if (gt == 0) {
                tc_fence_after();
                const uint32_t idesc = tc_idesc(kTcRows, last ? kTcOutRows : 64);
                const uint32_t b0 = sW + (uint32_t)l * kTcLayerBytes;
                const uint32_t blbo = (last ? kTcOutRows : 64) * 16;
                // K = 64 as four K = 16 steps: two core matrices of B each, and
                // of A two core matrices (layer 1) or eight TMEM columns.
                if (l == 0) {
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        tc_mma(tmem, tc_desc(sI + (uint32_t)k * 2u * (kTcRows * 16), kTcRows * 16),
                               tc_desc(b0 + (uint32_t)k * 2u * blbo, blbo), idesc, k > 0 ? 1u : 0u);
                } else {
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        tc_mma_ts(tmem, tact + (uint32_t)k * 8u, tc_desc(b0 + (uint32_t)k * 2u * blbo, blbo), idesc,
                                  k > 0 ? 1u : 0u);
                }
                tc_commit(mb_mma);
                mma_pending = true;
                mma_par = ph_mma;
            }
            ok = mbar_wait(mb_mma, ph_mma);
            ph_mma ^= 1u;
            ok = __all_sync(0xffffffffu, ok);  // tcgen05.ld below is warp-collective
            if (gt == 0 && ok) mma_pending = false;
            // The input tile is free once layer 1 has read it: fetch the next one.
            if (l == 0 && gt == 0 && ok && next < tiles) {
                tma_load_tile(&xmap, sI, mb_in, next * kTcRows);
                tma_pending = true;
                tma_par = ph_in;
            }
            tc_fence_after();
            if (ok) {
                if (!last) {
                    uint32_t r[64], a[32];
                    AQ_TC_LD16(tmem + lanes + 0u, (r + 0));
                    AQ_TC_LD16(tmem + lanes + 16u, (r + 16));
                    AQ_TC_LD16(tmem + lanes + 32u, (r + 32));
                    AQ_TC_LD16(tmem + lanes + 48u, (r + 48));
                    tc_wait_ld();
#pragma unroll
                    for (int c = 0; c < 32; ++c) a[c] = relu_pack2(r[2 * c], r[2 * c + 1]);
                    AQ_TC_ST16(tact + lanes + 0u, (a + 0));
                    AQ_TC_ST16(tact + lanes + 16u, (a + 16));
                    const int grow = tile * kTcRows + row;
                    if (acts && grow < n) {
                        uint4* dst = acts + ((size_t)l * (size_t)n + (size_t)grow) * 8;
#pragma unroll
                        for (int q4 = 0; q4 < 8; ++q4)
                            dst[q4] = make_uint4(a[4 * q4], a[4 * q4 + 1], a[4 * q4 + 2], a[4 * q4 + 3]);
                    }
                    tc_wait_st();
                } else {
                    uint32_t r[16];
                    AQ_TC_LD16(tmem + lanes, r);
                    tc_wait_ld();
                    const int grow = tile * kTcRows + row;
                    if (grow < n) {
                        out[(size_t)grow * 3 + 0] = __uint_as_float(r[0]);
                        out[(size_t)grow * 3 + 1] = __uint_as_float(r[1]);
                        out[(size_t)grow * 3 + 2] = __uint_as_float(r[2]);
                    }
                }
            }
            tc_fence_before();
            if (group_any(bar_id, !ok)) { fail = true; break; }
        }
        if (fail) break;
        tile = next;
    }
    if (fail && gt == 0) {
        atomicExch(err, 1u);
        // Let what this group still has in flight land (bounded) before TMEM is freed.
        if (mma_pending) mbar_wait(mb_mma, mma_par);
        if (tma_pending) mbar_wait(mb_in, tma_par);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem_base_slot),
                     "r"(kTcTmemCols)
                     : "memory");
    }
}

// ---------------------------------------------------------------- backward
// The training step's backward pass on the same machinery (relative L2 loss
// of Mueller et al. 2021 with y^2 held constant, as k_nrc_backward). Per
// 128-row tile: dY (16 columns, 3 used) from Y and the targets becomes the
// A operand in TMEM; dH5 = dY x W6 (one K = 16 MMA); then for layers 5..1
// the epilogue masks dH with ReLU'(H) read from the stored activations,
// rounds to bf16, writes delta_l for the weight gradients and, above layer
// 1, stores it back to TMEM as the A operand of dH_{l-1} = delta_l x W_l.
// Weight image (rows = N = 64 inputs, K = outputs): W6^T (K = 16) then
// W5^T..W2^T (K = 64).
constexpr int kTcBwdW6Bytes = kNrcTcBwdW6Bytes;                    // 2 KB
constexpr int kTcBwdBytes = kTcBwdW6Bytes + 4 * kTcLayerBytes;      // 34 KB
constexpr int kTcBwdSmemBytes = std::max(kTcBwdBytes + 1024, 120 * 1024);  // one CTA per SM
constexpr float kTcLossEps = 0.01f;

__device__ __forceinline__ uint32_t pack2_rn(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;\n" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}

#define AQ_TC_ST8(taddr, r)                                                                            \
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};\n" ::"r"(taddr), \
                 "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7])  \
                 : "memory")

// Y, T: n x 3 fp32 (outputs, targets); acts: H1..H5 bf16 rows; deltas:
// delta_1..delta_5 bf16 rows; d6: dY as 16 bf16 per row; loss: += sum of
// the per-element losses; err: 1 when a wait expired.
__global__ void __launch_bounds__(kTcThreads, 1)
    k_nrc_backward_tc(const float* __restrict__ Y, const float* __restrict__ T, int n, float inv_count,
                      const uint4* __restrict__ wimg, const uint4* __restrict__ acts, uint4* __restrict__ deltas,
                      uint4* __restrict__ d6, double* __restrict__ loss, uint32_t* __restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t bar_mma[kTcGroups];
    __shared__ uint32_t tmem_base_slot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = warp >> 2, q = warp & 3, gt = tid & 127;
    const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
    uint8_t* sbase = smem_raw + (base - smem_u32(smem_raw));
    grid_dep_wait();
    grid_dep_launch();
    for (int i = tid; i < kTcBwdBytes / 16; i += kTcThreads) reinterpret_cast<uint4*>(sbase)[i] = __ldcg(wimg + i);
    if (tid < kTcGroups)
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&bar_mma[tid])) : "memory");
    if (tid == 0) asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         smem_u32(&tmem_base_slot)),
                     "r"(kTcTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_slot + (uint32_t)g * kTcGroupCols;
    const uint32_t tact = tmem + kTcActCol;
    const uint32_t lanes = (uint32_t)(q * 32) << 16;
    const uint32_t mb = smem_u32(&bar_mma[g]);
    const int bar_id = 1 + g;
    const int tiles = (n + kTcRows - 1) / kTcRows;
    const int row = q * 32 + lane;
    uint32_t ph = 0, mma_par = 0;
    bool fail = false, pending = false;
    float lsum = 0.0f;
    for (int tile = (int)blockIdx.x + g * (int)gridDim.x; tile < tiles; tile += (int)gridDim.x * kTcGroups) {
        const int grow = tile * kTcRows + row;
        const bool valid = grow < n;
        // dY of this row (columns 0..2), packed as 16 bf16.
        float gy[3] = {0.0f, 0.0f, 0.0f};
        if (valid) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float y = __ldcg(Y + (size_t)grow * 3 + c), t = __ldcg(T + (size_t)grow * 3 + c);
                float den = y * y + kTcLossEps, d = y - t;
                lsum += d * d / den;
                gy[c] = 2.0f * d / den * inv_count;
            }
        }
        uint32_t a6[8] = {pack2_rn(gy[0], gy[1]), pack2_rn(gy[2], 0.0f), 0u, 0u, 0u, 0u, 0u, 0u};
        if (valid) {
            d6[(size_t)grow * 2] = make_uint4(a6[0], a6[1], 0u, 0u);
            d6[(size_t)grow * 2 + 1] = make_uint4(0u, 0u, 0u, 0u);
        }
        AQ_TC_ST8(tact + lanes, a6);
        asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
        tc_fence_before();
        group_sync(bar_id);  // dY is in TMEM before the first MMA
        for (int l = 4; l >= 0; --l) {  // this MMA gives dH of hidden layer l + 1
            if (gt == 0) {
                tc_fence_after();
                const uint32_t idesc = tc_idesc(kTcRows, 64);
                if (l == 4) {
                    tc_mma_ts(tmem, tact, tc_desc(base, 64 * 16), idesc, 0u);
                } else {
                    const uint32_t b0 = base + kTcBwdW6Bytes + (uint32_t)(3 - l) * kTcLayerBytes;
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        tc_mma_ts(tmem, tact + (uint32_t)k * 8u, tc_desc(b0 + (uint32_t)k * 2u * (64 * 16), 64 * 16),
                                  idesc, k > 0 ? 1u : 0u);
                }
                tc_commit(mb);
                pending = true;
                mma_par = ph;
            }
            bool ok = mbar_wait(mb, ph);
            ph ^= 1u;
            ok = __all_sync(0xffffffffu, ok);
            if (gt == 0 && ok) pending = false;
            tc_fence_after();
            if (ok) {
                uint32_t r[64], a[32];
                AQ_TC_LD16(tmem + lanes + 0u, (r + 0));
                AQ_TC_LD16(tmem + lanes + 16u, (r + 16));
                AQ_TC_LD16(tmem + lanes + 32u, (r + 32));
                AQ_TC_LD16(tmem + lanes + 48u, (r + 48));
                tc_wait_ld();
                // ReLU'(Z) from the stored activation H = ReLU(Z) in bf16.
                uint4 h[8];
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    h[j] = valid ? __ldcg(acts + ((size_t)l * (size_t)n + (size_t)grow) * 8 + (size_t)j) : make_uint4(0, 0, 0, 0);
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const uint32_t hw[4] = {h[j].x, h[j].y, h[j].z, h[j].w};
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int c = 4 * j + e;  // bf16 pair (2c, 2c + 1)
                        float lo = __uint_as_float(r[2 * c]), hi = __uint_as_float(r[2 * c + 1]);
                        if (!(__uint_as_float(hw[e] << 16) > 0.0f)) lo = 0.0f;
                        if (!(__uint_as_float(hw[e] & 0xffff0000u) > 0.0f)) hi = 0.0f;
                        a[c] = pack2_rn(lo, hi);
                    }
                }
                if (valid) {
                    uint4* dst = deltas + ((size_t)l * (size_t)n + (size_t)grow) * 8;
#pragma unroll
                    for (int j = 0; j < 8; ++j) dst[j] = make_uint4(a[4 * j], a[4 * j + 1], a[4 * j + 2], a[4 * j + 3]);
                }
                if (l > 0) {
                    AQ_TC_ST16(tact + lanes + 0u, (a + 0));
                    AQ_TC_ST16(tact + lanes + 16u, (a + 16));
                    tc_wait_st();
                }
            }
            tc_fence_before();
            if (group_any(bar_id, !ok)) {
                fail = true;
                break;
            }
        }
        if (fail) break;
    }
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
    if (lane == 0 && lsum != 0.0f) atomicAdd(loss, (double)lsum);
    if (fail && gt == 0) {
        atomicExch(err, 1u);
        if (pending) mbar_wait(mb, mma_par);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem_base_slot),
                     "r"(kTcTmemCols)
                     : "memory");
    }
}

// ---------------------------------------------------------------- host side
size_t nrc_tc_weight_bytes() { return (size_t)kTcWeightBytes; }

void nrc_pack_tc(aqua_ctx* ctx, const float* w, const float* inf, void* img_w, void* img_inf, void* img_bwd) {
    AQ_CUDA(cudaMemsetAsync(img_w, 0, kTcWeightBytes, ctx->stream));
    AQ_CUDA(cudaMemsetAsync(img_inf, 0, kTcWeightBytes, ctx->stream));
    AQ_CUDA(cudaMemsetAsync(img_bwd, 0, kTcBwdBytes, ctx->stream));
    k_nrc_pack_tc<<<(kNrcParams + 255) / 256, 256, 0, ctx->stream>>>(w, inf, (uint8_t*)img_w, (uint8_t*)img_inf,
                                                                     (uint8_t*)img_bwd);
    AQ_CUDA(cudaGetLastError());
}

static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, []() {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        (void)cudaGetLastError();
    });
    if (!fn) throw Error(AQUA_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    return fn;
}

void nrc_forward_tc_dev(aqua_ctx* ctx, const void* img, const uint16_t* X, int n, float* out, uint32_t* err,
                        uint32_t* acts, double* loss_zero) {
    if (n <= 0) return;
    if (((uintptr_t)X & 15) != 0) throw Error(AQUA_ERR_INVALID_ARG, "x must be 16-byte aligned");
    CUtensorMap map;
    const cuuint64_t dims[2] = {64, (cuuint64_t)n};
    const cuuint64_t strides[1] = {128};  // bytes per row
    const cuuint32_t box[2] = {8, (cuuint32_t)kTcRows};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = tensor_map_encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<uint16_t*>(X), dims,
                                      strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw Error(AQUA_ERR_CUDA, "cuTensorMapEncodeTiled failed for the query rows");
    if (!ctx->nrc_tc_ready) {  // once per context (one device)
        AQ_CUDA(cudaFuncSetAttribute(k_nrc_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcFwdSmemBytes));
        ctx->nrc_tc_ready = true;
    }
    const int tiles = (n + kTcRows - 1) / kTcRows;
    const int grid = std::max(1, std::min(tiles, ctx->num_sms));
    launch_chained(k_nrc_forward_tc, dim3(grid), dim3(kTcFwdThreads), kTcFwdSmemBytes, ctx->stream, map, n,
                   reinterpret_cast<const uint4*>(img), out, err, reinterpret_cast<uint4*>(acts), loss_zero);
    AQ_CUDA(cudaGetLastError());
}


// ---------------------------------------------------------------- weight gradients
// dW_L = D_L^T x H_L over a chunk of rows (split-K, wgrad_chunk_rows; the Adam
// kernel sums the chunk partials in order). Layer L of blockIdx.y: 0..4 ->
// W1..W5 (H_0 = X, D = delta_{L+1}, 64 columns), 5 -> W6 (H_5, D = dY, 16
// columns, 3 used). One tcgen05.mma per K = 16 rows: A = D^T (M = 128: the
// 64 or 16 output features in rows 0.., zero rows above), B = H^T (N = 64
// input features), both K-major with K = batch rows, accumulating in TMEM
// (128 lanes x 64 FP32 columns). The 256 threads read each 128-row slice of
// D and H with coalesced 16-byte loads (issued one slice ahead, into
// registers), store it row-major to shared memory and transpose it there into
// the no-swizzle core-matrix layout (8 batch rows of one feature = one
// 16-byte core-matrix row); thread 0 issues the slice's MMAs and commits them
// to an mbarrier, which the next slice's transpose waits for. The 84 KB of
// shared memory let two CTAs share an SM. All waits are bounded.
constexpr int kWgTcThreads = 256;
constexpr int kWgTcChunk = 512;                 // rows per CTA (split-K chunk), at least
constexpr int kWgTcMaxChunks = 64;              // larger batches get longer chunks
constexpr int kWgTcSlice = 128;                 // rows per staged slice (MMA K = 8 x 16)
constexpr int kWgTcABytes = 128 * kWgTcSlice * 2;  // A: 128 feature rows x 128 K
constexpr int kWgTcBBytes = 64 * kWgTcSlice * 2;   // B: 64 feature rows x 128 K
constexpr int kWgTcRawStride = 144;  // bytes per raw staged row: 128 + 16 (16-byte aligned; 8 rows start on 8 banks)
constexpr int kWgTcRawBytes = kWgTcSlice * kWgTcRawStride;
constexpr int kWgTcSmem = kWgTcABytes + kWgTcBBytes + 2 * kWgTcRawBytes + 1024;
constexpr int kWgTcLoads = kWgTcSlice * 8 / kWgTcThreads;  // 16-byte loads per thread per matrix and slice
static_assert(kWgTcChunk % kWgTcSlice == 0, "whole slices per chunk");
static_assert(2 * kWgTcSmem <= 227 * 1024, "two CTAs per SM");
// Rows per chunk for a batch of n rows: at least kWgTcChunk, and long enough
// that at most kWgTcMaxChunks partials reach the Adam kernel, which sums
// every parameter's partials in order (one thread per parameter).
static int wgrad_chunk_rows(int n) {
    const int per = (n + kWgTcMaxChunks - 1) / kWgTcMaxChunks;
    return std::max(kWgTcChunk, (per + kWgTcChunk - 1) / kWgTcChunk * kWgTcChunk);
}

__global__ void __launch_bounds__(kWgTcThreads, 2) k_nrc_wgrad_tc(const uint16_t* __restrict__ X,
                                                                  const uint16_t* __restrict__ acts,
                                                                  const uint16_t* __restrict__ deltas,
                                                                  const uint16_t* __restrict__ d6, int n,
                                                                  int chunk_rows, float* __restrict__ partial,
                                                                  uint32_t* __restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int L = blockIdx.y, ch = blockIdx.x;
    const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
    uint8_t* sbase = smem_raw + (base - smem_u32(smem_raw));
    const uint32_t sA = base, sB = base + (uint32_t)kWgTcABytes;
    uint8_t* a = sbase;
    uint8_t* bb = sbase + kWgTcABytes;
    uint8_t* rawH = bb + kWgTcBBytes;
    uint8_t* rawD = rawH + kWgTcRawBytes;
    const int dcols = L == 5 ? 16 : 64;
    const uint16_t* H = L == 0 ? X : acts + (size_t)(L - 1) * (size_t)n * 64;
    const uint16_t* D = L == 5 ? d6 : deltas + (size_t)L * (size_t)n * 64;

    // A's rows from dcols up stay zero for the whole chunk.
    for (int i = tid; i < kWgTcABytes / 16; i += kWgTcThreads) reinterpret_cast<uint4*>(a)[i] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    grid_dep_wait();  // the activations and deltas come from the kernels before
    grid_dep_launch();
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_slot)),
                     "r"(64u)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = tc_idesc(128, 64);
    const int row_begin = ch * chunk_rows;
    const int slices = min(chunk_rows, n - row_begin + kWgTcSlice - 1) / kWgTcSlice;
    // Raw row-major staging of one slice: H rows (128 B) and D rows (128 or
    // 32 B), read with coalesced 16-byte loads into registers (zero past n).
    const int dq = dcols / 8;  // 16-byte words per D row
    uint4 rh[kWgTcLoads], rd[kWgTcLoads];
    auto load_rows = [&](int r0) {
#pragma unroll
        for (int q = 0; q < kWgTcLoads; ++q) {
            const int idx = tid + kWgTcThreads * q, row = r0 + (idx >> 3);
            rh[q] = row < n ? __ldca(reinterpret_cast<const uint4*>(H + (size_t)row * 64) + (idx & 7)) : make_uint4(0, 0, 0, 0);
            const int row_d = r0 + idx / dq;
            rd[q] = (idx < kWgTcSlice * dq && row_d < n)
                        ? __ldca(reinterpret_cast<const uint4*>(D + (size_t)row_d * dcols) + idx % dq)
                        : make_uint4(0, 0, 0, 0);
        }
    };
    auto store_raw = [&]() {
#pragma unroll
        for (int q = 0; q < kWgTcLoads; ++q) {
            const int idx = tid + kWgTcThreads * q;
            *reinterpret_cast<uint4*>(rawH + (size_t)(idx >> 3) * kWgTcRawStride + (size_t)(idx & 7) * 16) = rh[q];
            if (idx < kWgTcSlice * dq)
                *reinterpret_cast<uint4*>(rawD + (size_t)(idx / dq) * kWgTcRawStride + (size_t)(idx % dq) * 16) =
                    rd[q];
        }
    };
    load_rows(row_begin);
    uint32_t par = 0;      // parity of the mbarrier's next completion
    bool pending = false;  // the last slice's MMAs not yet waited for
    bool ok = true;
    for (int sl = 0; sl < slices; ++sl) {
        // The slice's rows (prefetched) go to the raw buffers as they are;
        // the next slice's rows are requested before this one is transposed.
        store_raw();
        if (sl + 1 < slices) load_rows(row_begin + (sl + 1) * kWgTcSlice);
        // The previous slice's MMAs must have read A and B before the
        // transpose overwrites them.
        bool w = true;
        if (pending && tid == 0) w = mbar_wait(smem_u32(&bar), par);
        ok = __syncthreads_and(w) != 0;  // also: the raw buffers are complete
        if (!ok) break;  // still pending: the drain below waits for it
        if (pending) {
            par ^= 1u;
            pending = false;
        }
        // Transpose: feature f of rows 8j..8j+7 -> one 16-byte core-matrix row.
        for (int it = tid; it < (64 + dcols) * 16; it += kWgTcThreads) {
            const bool isA = it >= 64 * 16;
            const int k = isA ? it - 64 * 16 : it;
            const int cols = isA ? dcols : 64;
            const int f = k % cols, j = k / cols;  // consecutive threads: consecutive features
            const uint8_t* src = (isA ? rawD : rawH) + (size_t)(8 * j) * kWgTcRawStride + (size_t)f * 2;
            uint32_t v[4];
#pragma unroll
            for (int q = 0; q < 4; ++q)
                v[q] = (uint32_t)*reinterpret_cast<const uint16_t*>(src + (size_t)(2 * q) * kWgTcRawStride) |
                       ((uint32_t)*reinterpret_cast<const uint16_t*>(src + (size_t)(2 * q + 1) * kWgTcRawStride)
                        << 16);
            const int R = isA ? 128 : 64;
            *reinterpret_cast<uint4*>((isA ? a : bb) + (size_t)j * R * 16 + (size_t)f * 16) =
                make_uint4(v[0], v[1], v[2], v[3]);
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();  // the transpose is complete (and the raw buffers free)
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (int k = 0; k < kWgTcSlice / 16; ++k)
                tc_mma(tmem, tc_desc(sA + (uint32_t)k * 2u * (128 * 16), 128 * 16),
                       tc_desc(sB + (uint32_t)k * 2u * (64 * 16), 64 * 16), idesc, (sl > 0 || k > 0) ? 1u : 0u);
            tc_commit(smem_u32(&bar));
        }
        pending = true;
    }
    // Drain: wait (bounded) for the commit still pending, so no MMA runs when
    // the accumulator is read or the TMEM is freed.
    if (pending) {
        bool w = tid == 0 ? mbar_wait(smem_u32(&bar), par) : true;
        ok = (__syncthreads_and(w) != 0) && ok;
    }
    tc_fence_after();
    if (ok) {
        // Lanes 0..63 hold rows (output features) 0..63; warps 0 and 1 read them.
        const int orow = warp * 32 + lane;
        if (warp < 2) {
            uint32_t r[64];
            const uint32_t lanes = (uint32_t)(warp * 32) << 16;
            AQ_TC_LD16(tmem + lanes + 0u, (r + 0));
            AQ_TC_LD16(tmem + lanes + 16u, (r + 16));
            AQ_TC_LD16(tmem + lanes + 32u, (r + 32));
            AQ_TC_LD16(tmem + lanes + 48u, (r + 48));
            tc_wait_ld();
            const int mrows = L == 5 ? kNrcOut : 64;
            if (orow < mrows) {
                float4* P = reinterpret_cast<float4*>(partial + (size_t)ch * kNrcParams + (size_t)L * 4096 +
                                                      (size_t)orow * 64);
#pragma unroll
                for (int c = 0; c < 16; ++c)
                    P[c] = make_float4(__uint_as_float(r[4 * c]), __uint_as_float(r[4 * c + 1]),
                                       __uint_as_float(r[4 * c + 2]), __uint_as_float(r[4 * c + 3]));
            }
        }
    } else if (tid == 0) {
        atomicExch(err, 1u);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(64u) : "memory");
    }
}

int nrc_wgrad_tc_dev(aqua_ctx* ctx, const uint16_t* X, const uint32_t* acts, const uint32_t* deltas,
                     const uint32_t* d6, int n, float* partial, uint32_t* err) {
    if (n <= 0) return 0;
    if (!ctx->nrc_tc_wg_ready) {
        AQ_CUDA(cudaFuncSetAttribute(k_nrc_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kWgTcSmem));
        ctx->nrc_tc_wg_ready = true;
    }
    const int rows = wgrad_chunk_rows(n);
    const int chunks = (n + rows - 1) / rows;
    launch_chained(k_nrc_wgrad_tc, dim3(chunks, 6), dim3(kWgTcThreads), kWgTcSmem, ctx->stream, X,
                   reinterpret_cast<const uint16_t*>(acts), reinterpret_cast<const uint16_t*>(deltas),
                   reinterpret_cast<const uint16_t*>(d6), n, rows, partial, err);
    AQ_CUDA(cudaGetLastError());
    return chunks;
}

size_t nrc_tc_bwd_bytes() { return (size_t)kTcBwdBytes; }

void nrc_backward_tc_dev(aqua_ctx* ctx, const void* img, const float* Y, const float* T, int n, float inv_count,
                         const uint32_t* acts, uint32_t* deltas, uint32_t* d6, double* loss, uint32_t* err) {
    if (n <= 0) return;
    if (!ctx->nrc_tc_bwd_ready) {
        AQ_CUDA(cudaFuncSetAttribute(k_nrc_backward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     kTcBwdSmemBytes));
        ctx->nrc_tc_bwd_ready = true;
    }
    const int tiles = (n + kTcRows - 1) / kTcRows;
    const int grid = std::max(1, std::min(tiles, ctx->num_sms));
    launch_chained(k_nrc_backward_tc, dim3(grid), dim3(kTcThreads), kTcBwdSmemBytes, ctx->stream, Y, T, n,
                   inv_count, reinterpret_cast<const uint4*>(img), reinterpret_cast<const uint4*>(acts),
                   reinterpret_cast<uint4*>(deltas), reinterpret_cast<uint4*>(d6), loss, err);
    AQ_CUDA(cudaGetLastError());
}

}  // namespace aq
