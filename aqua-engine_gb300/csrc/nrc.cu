// nrc.cu — the radiance cache's network on tensor cores: fused forward (all
// six layers of a 16-row tile stay in registers), fused backward (all layers'
// input gradients), weight gradients as split-K GEMMs, Adam, and the
// input-encoding kernel. BF16 operands, FP32 accumulation.
//
// MMA layout (m16n8k16, bf16 -> f32): a warp owns a 16-row tile. The
// accumulator fragment of layer l (rows lane/4 and lane/4+8, columns
// 2*(lane%4)+{0,1} of each 8-wide n-tile) is, after ReLU and packing to
// bf16, exactly the A fragment of layer l+1, so activations never leave the
// registers. Weights are staged in shared memory already permuted into
// B-fragment order (one 8-byte load per lane per MMA, conflict-free).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "internal.h"
#include "nrc.h"

namespace aq {

// ---------------------------------------------------------------- fragment tables
// Forward B fragments: layers 0..4 (W1..W5) [nt 8][kt 4][lane 32], then W6
// [kt 4][lane 32] (n-tile 0, outputs 3..7 zero).
constexpr int kFragFwd = kNrcHiddenLayers * 8 * 4 * 32 + 4 * 32;  // uint2
// Backward B fragments: W6 for dY x W6 [nt 8][lane 32] (K = 16, rows 3..15
// zero), then W5..W2 [layer 3..0][nt 8][kt 4][lane 32].
constexpr int kFragBwd = 8 * 32 + 4 * 8 * 4 * 32;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float bf16_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint2 b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

__device__ __forceinline__ uint16_t bf16_bits(float x) {
    __nv_bfloat16 h = __float2bfloat16_rn(x);
    return *reinterpret_cast<uint16_t*>(&h);
}

// Builds both fragment tables from the FP32 master weights.
__global__ void k_nrc_pack(const float* __restrict__ w, uint2* __restrict__ fwd, uint2* __restrict__ bwd) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kFragFwd) {
        int lane = i & 31, r = lane >> 2, c2 = (lane & 3) * 2;
        float v[4];
        if (i < kNrcHiddenLayers * 8 * 4 * 32) {
            int kt = (i >> 5) & 3, nt = (i >> 7) & 7, l = i >> 10;
            const float* W = w + l * 4096;
            int n = nt * 8 + r, k0 = kt * 16 + c2;
            v[0] = W[n * 64 + k0]; v[1] = W[n * 64 + k0 + 1];
            v[2] = W[n * 64 + k0 + 8]; v[3] = W[n * 64 + k0 + 9];
        } else {
            int kt = (i >> 5) & 3;
            const float* W = w + 5 * 4096;
            int n = r, k0 = kt * 16 + c2;
            bool ok = n < kNrcOut;
            v[0] = ok ? W[n * 64 + k0] : 0.0f; v[1] = ok ? W[n * 64 + k0 + 1] : 0.0f;
            v[2] = ok ? W[n * 64 + k0 + 8] : 0.0f; v[3] = ok ? W[n * 64 + k0 + 9] : 0.0f;
        }
        fwd[i] = make_uint2(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]));
    }
    int j = i - kFragFwd;
    if (bwd && j >= 0 && j < kFragBwd) {
        int lane = j & 31, r = lane >> 2, c2 = (lane & 3) * 2;
        float v[4];
        if (j < 8 * 32) {
            int nt = j >> 5;
            const float* W = w + 5 * 4096;
            int n = nt * 8 + r, k0 = c2;  // k = output index (< 3 valid)
            v[0] = k0 < 3 ? W[k0 * 64 + n] : 0.0f;
            v[1] = k0 + 1 < 3 ? W[(k0 + 1) * 64 + n] : 0.0f;
            v[2] = 0.0f;
            v[3] = 0.0f;
        } else {
            int jj = j - 8 * 32;
            int kt = (jj >> 5) & 3, nt = (jj >> 7) & 7, t = jj >> 10;  // t = 0..3 -> W5..W2
            const float* W = w + (4 - t) * 4096;
            int n = nt * 8 + r, k0 = kt * 16 + c2;  // k = output index of that layer
            v[0] = W[k0 * 64 + n]; v[1] = W[(k0 + 1) * 64 + n];
            v[2] = W[(k0 + 8) * 64 + n]; v[3] = W[(k0 + 9) * 64 + n];
        }
        bwd[j] = make_uint2(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]));
    }
}

// ---------------------------------------------------------------- forward
// X: n rows of 64 bf16 (32 u32). out: n x 3 fp32. With TRAIN the post-ReLU
// activations H1..H5 (bf16, the values the next layer consumed) go to acts.
template <bool TRAIN>
__global__ void __launch_bounds__(128) k_nrc_forward(const uint32_t* __restrict__ X, int n,
                                                     const uint2* __restrict__ wfrag, float* __restrict__ out,
                                                     uint32_t* __restrict__ acts) {
    __shared__ uint2 sW[kFragFwd];
    for (int i = threadIdx.x; i < kFragFwd; i += blockDim.x) sW[i] = wfrag[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, c = lane & 3;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int tile = warp; tile * 16 < n; tile += nwarps) {
        const int r0 = tile * 16 + (lane >> 2), r1 = r0 + 8;
        const bool ok0 = r0 < n, ok1 = r1 < n;
        uint32_t a[4][4];
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            a[kt][0] = ok0 ? X[(size_t)r0 * 32 + kt * 8 + c] : 0u;
            a[kt][1] = ok1 ? X[(size_t)r1 * 32 + kt * 8 + c] : 0u;
            a[kt][2] = ok0 ? X[(size_t)r0 * 32 + kt * 8 + 4 + c] : 0u;
            a[kt][3] = ok1 ? X[(size_t)r1 * 32 + kt * 8 + 4 + c] : 0u;
        }
#pragma unroll 1
        for (int l = 0; l < kNrcHiddenLayers; ++l) {
            float acc[8][4];
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
            for (int kt = 0; kt < 4; ++kt)
#pragma unroll
                for (int nt = 0; nt < 8; ++nt) mma_bf16(acc[nt], a[kt], sW[((l * 8 + nt) * 4 + kt) * 32 + lane]);
#pragma unroll
            for (int kt = 0; kt < 4; ++kt) {
                a[kt][0] = pack_bf16(fmaxf(acc[2 * kt][0], 0.0f), fmaxf(acc[2 * kt][1], 0.0f));
                a[kt][1] = pack_bf16(fmaxf(acc[2 * kt][2], 0.0f), fmaxf(acc[2 * kt][3], 0.0f));
                a[kt][2] = pack_bf16(fmaxf(acc[2 * kt + 1][0], 0.0f), fmaxf(acc[2 * kt + 1][1], 0.0f));
                a[kt][3] = pack_bf16(fmaxf(acc[2 * kt + 1][2], 0.0f), fmaxf(acc[2 * kt + 1][3], 0.0f));
            }
            if (TRAIN) {
                uint32_t* H = acts + (size_t)l * (size_t)n * 32;
#pragma unroll
                for (int kt = 0; kt < 4; ++kt) {
                    if (ok0) { H[(size_t)r0 * 32 + kt * 8 + c] = a[kt][0]; H[(size_t)r0 * 32 + kt * 8 + 4 + c] = a[kt][2]; }
                    if (ok1) { H[(size_t)r1 * 32 + kt * 8 + c] = a[kt][1]; H[(size_t)r1 * 32 + kt * 8 + 4 + c] = a[kt][3]; }
                }
            }
        }
        float o[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        const uint2* sWo = sW + kNrcHiddenLayers * 8 * 4 * 32;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) mma_bf16(o, a[kt], sWo[kt * 32 + lane]);
        if (c == 0) {
            if (ok0) { out[(size_t)r0 * 3 + 0] = o[0]; out[(size_t)r0 * 3 + 1] = o[1]; }
            if (ok1) { out[(size_t)r1 * 3 + 0] = o[2]; out[(size_t)r1 * 3 + 1] = o[3]; }
        } else if (c == 1) {
            if (ok0) out[(size_t)r0 * 3 + 2] = o[0];
            if (ok1) out[(size_t)r1 * 3 + 2] = o[2];
        }
    }
}

// ---------------------------------------------------------------- backward
// Relative L2 loss (Mueller et al. 2021): L = mean over rows and channels of
// (y - t)^2 / (y^2 + eps), y^2 treated as a constant. Writes
// dY (bf16, 16 columns, 3 used) and the input gradients of layers 5..1
// (bf16 delta_l = dL/dZ_l), and adds the loss sum to *loss.
constexpr float kNrcLossEps = 0.01f;

__global__ void __launch_bounds__(128) k_nrc_backward(const float* __restrict__ Y, const float* __restrict__ T,
                                                      int n, float inv_count, const uint2* __restrict__ wfragT,
                                                      const uint32_t* __restrict__ acts,
                                                      uint32_t* __restrict__ deltas, uint32_t* __restrict__ d6,
                                                      double* __restrict__ loss) {
    __shared__ uint2 sW[kFragBwd];
    for (int i = threadIdx.x; i < kFragBwd; i += blockDim.x) sW[i] = wfragT[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, c = lane & 3;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    float lsum = 0.0f;
    for (int tile = warp; tile * 16 < n; tile += nwarps) {
        const int r0 = tile * 16 + (lane >> 2), r1 = r0 + 8;
        const bool ok0 = r0 < n, ok1 = r1 < n;
        // dY for columns 2c, 2c+1 of rows r0, r1 (only columns 0..2 exist).
        float g[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            int row = e < 2 ? r0 : r1, col = 2 * c + (e & 1);
            bool ok = (e < 2 ? ok0 : ok1) && col < kNrcOut;
            if (ok) {
                float y = Y[(size_t)row * 3 + col], t = T[(size_t)row * 3 + col];
                float den = y * y + kNrcLossEps;
                float d = y - t;
                lsum += d * d / den;
                g[e] = 2.0f * d / den * inv_count;
            }
        }
        uint32_t a6[4] = {pack_bf16(g[0], g[1]), pack_bf16(g[2], g[3]), 0u, 0u};
        if (ok0) { d6[(size_t)r0 * 8 + c] = a6[0]; d6[(size_t)r0 * 8 + 4 + c] = 0u; }
        if (ok1) { d6[(size_t)r1 * 8 + c] = a6[1]; d6[(size_t)r1 * 8 + 4 + c] = 0u; }
        // dH5 = dY x W6, masked by ReLU'(Z5).
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
            mma_bf16(acc[nt], a6, sW[nt * 32 + lane]);
        }
        uint32_t a[4][4];
#pragma unroll 1
        for (int l = 4; l >= 0; --l) {  // acc holds dH_{l+1}; mask with H_{l+1} = acts[l]
            const uint32_t* H = acts + (size_t)l * (size_t)n * 32;
            uint32_t* D = deltas + (size_t)l * (size_t)n * 32;
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                uint32_t h0 = ok0 ? H[(size_t)r0 * 32 + nt * 4 + c] : 0u;
                uint32_t h1 = ok1 ? H[(size_t)r1 * 32 + nt * 4 + c] : 0u;
                if (!(bf16_lo(h0) > 0.0f)) acc[nt][0] = 0.0f;
                if (!(bf16_hi(h0) > 0.0f)) acc[nt][1] = 0.0f;
                if (!(bf16_lo(h1) > 0.0f)) acc[nt][2] = 0.0f;
                if (!(bf16_hi(h1) > 0.0f)) acc[nt][3] = 0.0f;
            }
#pragma unroll
            for (int kt = 0; kt < 4; ++kt) {
                a[kt][0] = pack_bf16(acc[2 * kt][0], acc[2 * kt][1]);
                a[kt][1] = pack_bf16(acc[2 * kt][2], acc[2 * kt][3]);
                a[kt][2] = pack_bf16(acc[2 * kt + 1][0], acc[2 * kt + 1][1]);
                a[kt][3] = pack_bf16(acc[2 * kt + 1][2], acc[2 * kt + 1][3]);
                if (ok0) { D[(size_t)r0 * 32 + kt * 8 + c] = a[kt][0]; D[(size_t)r0 * 32 + kt * 8 + 4 + c] = a[kt][2]; }
                if (ok1) { D[(size_t)r1 * 32 + kt * 8 + c] = a[kt][1]; D[(size_t)r1 * 32 + kt * 8 + 4 + c] = a[kt][3]; }
            }
            if (l == 0) break;
            // dH_l = delta_{l+1} x W_{l+1}
            const uint2* sWl = sW + 8 * 32 + (4 - l) * 8 * 4 * 32;
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
            for (int kt = 0; kt < 4; ++kt)
#pragma unroll
                for (int nt = 0; nt < 8; ++nt) mma_bf16(acc[nt], a[kt], sWl[(nt * 4 + kt) * 32 + lane]);
        }
    }
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
    if (lane == 0 && lsum != 0.0f) atomicAdd(loss, (double)lsum);
}

// ---------------------------------------------------------------- weight gradients
// dW_{L+1} = delta_{L+1}^T x H_L over a chunk of rows (split-K). Layer L of
// blockIdx.y: 0..4 -> W1..W5 (H_0 = X), 5 -> W6 (delta = dY, 16 columns).
// Operands are staged in shared memory and fed through ldmatrix.trans.
constexpr int kWgChunk = 128;
constexpr int kWgStride = 72;  // bf16 per staged row (64 + 8 pad: conflict-free ldmatrix)

__device__ __forceinline__ void ldsm_x4_trans(uint32_t (&r)[4], const void* p) {
    uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

__global__ void __launch_bounds__(128) k_nrc_wgrad(const uint32_t* __restrict__ X, const uint32_t* __restrict__ acts,
                                                   const uint32_t* __restrict__ deltas,
                                                   const uint32_t* __restrict__ d6, int n,
                                                   float* __restrict__ partial) {
    __shared__ __align__(16) uint16_t sD[kWgChunk * kWgStride];
    __shared__ __align__(16) uint16_t sH[kWgChunk * kWgStride];
    const int L = blockIdx.y, ch = blockIdx.x;
    const int row0 = ch * kWgChunk;
    const uint32_t* Hsrc = L == 0 ? X : acts + (size_t)(L - 1) * (size_t)n * 32;
    const int dcols = L == 5 ? 16 : 64;
    const uint32_t* Dsrc = L == 5 ? d6 : deltas + (size_t)L * (size_t)n * 32;
    // Stage rows [row0, row0 + chunk): 16-byte copies, zero past n.
    for (int i = threadIdx.x; i < kWgChunk * 8; i += blockDim.x) {
        int r = i >> 3, q = i & 7, row = row0 + r;
        uint4 h = make_uint4(0, 0, 0, 0), d = make_uint4(0, 0, 0, 0);
        if (row < n) {
            h = reinterpret_cast<const uint4*>(Hsrc + (size_t)row * 32)[q];
            if (q < dcols / 8) d = reinterpret_cast<const uint4*>(Dsrc + (size_t)row * (dcols / 2))[q];
        }
        *reinterpret_cast<uint4*>(&sH[r * kWgStride + q * 8]) = h;
        *reinterpret_cast<uint4*>(&sD[r * kWgStride + q * 8]) = d;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mrows = L == 5 ? 16 : 64;
    if (warp * 16 >= mrows) return;
    const int o0 = warp * 16;
    float acc[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
    const int t8 = lane & 7, m = lane >> 3;
#pragma unroll 1
    for (int k0 = 0; k0 < kWgChunk; k0 += 16) {
        uint32_t a[4];
        // A = delta^T: matrices (k0..7, o0..7), (k0..7, o0+8..), (k0+8.., o0..), (k0+8.., o0+8..)
        ldsm_x4_trans(a, &sD[(k0 + t8 + 8 * (m >> 1)) * kWgStride + o0 + 8 * (m & 1)]);
#pragma unroll
        for (int np = 0; np < 4; ++np) {
            uint32_t b[4];
            // B = H: matrices (k0..7, n0), (k0+8.., n0), (k0..7, n0+8), (k0+8.., n0+8)
            ldsm_x4_trans(b, &sH[(k0 + t8 + 8 * (m & 1)) * kWgStride + np * 16 + 8 * (m >> 1)]);
            mma_bf16(acc[2 * np], a, make_uint2(b[0], b[1]));
            mma_bf16(acc[2 * np + 1], a, make_uint2(b[2], b[3]));
        }
    }
    float* P = partial + (size_t)ch * kNrcParams + (size_t)L * 4096;
    const int r = lane >> 2, cc = (lane & 3) * 2;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        int col = nt * 8 + cc;
        int oa = o0 + r, ob = o0 + r + 8;
        if (L < 5 || oa < kNrcOut) { P[oa * 64 + col] = acc[nt][0]; P[oa * 64 + col + 1] = acc[nt][1]; }
        if (L < 5 || ob < kNrcOut) { P[ob * 64 + col] = acc[nt][2]; P[ob * 64 + col + 1] = acc[nt][3]; }
    }
}

// ---------------------------------------------------------------- Adam
// Kingma & Ba 2015. The gradient of parameter p is the sum of the chunk
// partials in chunk order (deterministic).
// With img_w non-null the new weights also go straight into the tcgen05
// weight images (forward images of w and of the inference weights, backward
// image of w), so no packing launch follows the step.
__global__ void k_nrc_adam(const float* __restrict__ partial, int chunks, float* __restrict__ w,
                           float* __restrict__ m, float* __restrict__ v, float* __restrict__ grad, float lr,
                           float b1, float b2, float eps, float c1, float c2, float* __restrict__ ema,
                           float ema_decay, uint8_t* __restrict__ img_w, uint8_t* __restrict__ img_inf,
                           uint8_t* __restrict__ img_bwd) {
    grid_dep_wait();
    grid_dep_launch();
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kNrcParams) return;
    float g = 0.0f;
    for (int k = 0; k < chunks; ++k) g += __ldcg(partial + (size_t)k * kNrcParams + p);
    grad[p] = g;
    float mm = b1 * m[p] + (1.0f - b1) * g;
    float vv = b2 * v[p] + (1.0f - b2) * g * g;
    m[p] = mm;
    v[p] = vv;
    float wn = w[p] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    w[p] = wn;
    // Inference weights: exponential moving average of the trained ones.
    float inf = wn;
    if (ema_decay > 0.0f) {
        inf = ema_decay * ema[p] + (1.0f - ema_decay) * wn;
        ema[p] = inf;
    }
    if (img_w) {
        uint32_t fwd;
        int32_t bwd;
        nrc_tc_param_offsets(p, fwd, bwd);
        const __nv_bfloat16 b = __float2bfloat16_rn(wn);
        *reinterpret_cast<__nv_bfloat16*>(img_w + fwd) = b;
        *reinterpret_cast<__nv_bfloat16*>(img_inf + fwd) = __float2bfloat16_rn(inf);
        if (bwd >= 0) *reinterpret_cast<__nv_bfloat16*>(img_bwd + bwd) = b;
    }
}

// ---------------------------------------------------------------- encoding
// A block encodes 128 rows. Raw rows come in and encoded rows go out through
// shared memory so that both move as contiguous, coalesced words (a thread's
// own row is 64 B in and 128 B out: one row per thread would touch a line
// per lane and word). Each row's spherical coordinates are computed once and
// each position octave with one sincospif of the exactly scaled coordinate.
constexpr int kEncRows = 128;

__device__ __forceinline__ uint32_t bf16_pair(float lo, float hi) {
    return (uint32_t)bf16_bits(lo) | ((uint32_t)bf16_bits(hi) << 16);
}

__global__ void __launch_bounds__(kEncRows) k_nrc_encode(const float* __restrict__ raw, int n, float3 bmin,
                                                         float3 binv, uint16_t* __restrict__ X) {
    __shared__ float s_raw[kEncRows][kNrcRaw + 1];  // +1: conflict-free row reads
    __shared__ uint32_t s_out[kEncRows][33];
    const int t = threadIdx.x;
    grid_dep_wait();
    grid_dep_launch();
    const size_t row0 = (size_t)blockIdx.x * kEncRows;
    const int rows = min(kEncRows, n - (int)row0);
    const float* src = raw + row0 * kNrcRaw;
    for (int k = t; k < rows * kNrcRaw; k += kEncRows) s_raw[k / kNrcRaw][k % kNrcRaw] = __ldcg(src + k);
    __syncthreads();
    if (t < rows) {
        const float* r = s_raw[t];
        uint32_t* o = s_out[t];
        float pn[3] = {nrc_wrap01((r[0] - bmin.x) * binv.x), nrc_wrap01((r[1] - bmin.y) * binv.y),
                       nrc_wrap01((r[2] - bmin.z) * binv.z)};
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int f = 0; f < 8; ++f) {
                float sn, cs;
                sincospif(pn[a] * (float)(1 << f), &sn, &cs);  // the scale by 2^f is exact
                o[a * 8 + f] = bf16_pair(sn, cs);
            }
        float du, dv, nu, nv;
        sph01(r[3], r[4], r[5], du, dv);
        sph01(r[6], r[7], r[8], nu, nv);
        o[24] = bf16_pair(one_blob(du, 0, 3), one_blob(du, 1, 3));
        o[25] = bf16_pair(one_blob(du, 2, 3), one_blob(dv, 0, 3));
        o[26] = bf16_pair(one_blob(dv, 1, 3), one_blob(dv, 2, 3));
        o[27] = bf16_pair(one_blob(nu, 0, 2), one_blob(nu, 1, 2));
        o[28] = bf16_pair(one_blob(nv, 0, 2), one_blob(nv, 1, 2));
        o[29] = bf16_pair(nrc_wrap01(r[9]), r[10]);
        o[30] = bf16_pair(r[11], r[12]);
        o[31] = bf16_pair(0.2126f * r[13] + 0.7152f * r[14] + 0.0722f * r[15], 1.0f);
    }
    __syncthreads();
    uint32_t* dst = reinterpret_cast<uint32_t*>(X + row0 * kNrcIn);
    for (int k = t; k < rows * 32; k += kEncRows) dst[k] = s_out[k >> 5][k & 31];
}

// ---------------------------------------------------------------- host side
static size_t rup(size_t x, size_t a) { return (x + a - 1) / a * a; }

void nrc_alloc(aqua_ctx* ctx, NrcNet& net) {
    size_t off = 0;
    auto take = [&](size_t b) { size_t o = off; off = rup(off + b, 256); return o; };
    size_t o_w = take(4 * kNrcParams), o_m = take(4 * kNrcParams), o_v = take(4 * kNrcParams),
           o_g = take(4 * kNrcParams), o_f = take(8 * kFragFwd), o_b = take(8 * kFragBwd), o_l = take(64),
           o_e = take(4 * kNrcParams), o_fi = take(8 * kFragFwd), o_tc = take(nrc_tc_weight_bytes()),
           o_tw = take(nrc_tc_weight_bytes()), o_tb = take(nrc_tc_bwd_bytes());
    dev_alloc(ctx, net.block, off);
    char* b = (char*)net.block.ptr;
    net.w = (float*)(b + o_w);
    net.m = (float*)(b + o_m);
    net.v = (float*)(b + o_v);
    net.grad = (float*)(b + o_g);
    net.frag = (uint2*)(b + o_f);
    net.fragT = (uint2*)(b + o_b);
    net.loss = (double*)(b + o_l);
    net.ema = (float*)(b + o_e);
    net.frag_inf = (uint2*)(b + o_fi);
    net.img_tc = (uint8_t*)(b + o_tc);
    net.img_tc_w = (uint8_t*)(b + o_tw);
    net.img_tc_bwd = (uint8_t*)(b + o_tb);
    net.tc_err = (uint32_t*)(b + o_l + 8);  // next to the loss: one read-back carries both
    AQ_CUDA(cudaMemsetAsync(net.tc_err, 0, 4, ctx->stream));
}

void nrc_release(NrcNet& net) {
    dev_free(net.block);
    dev_free(net.train);
    net = NrcNet{};
}

// He-uniform initial weights from PCG32 (seed), Adam state zeroed.
void nrc_init_weights(aqua_ctx* ctx, NrcNet& net, uint64_t seed) {
    std::vector<float> w(kNrcParams);
    uint64_t inc;
    uint64_t st = pcg32_seed(seed, 0xA11CEULL, inc);
    for (int i = 0; i < kNrcParams; ++i) {
        float u = u01(pcg32_next(st, inc)) * 2.0f - 1.0f;
        float lim = i < 5 * 4096 ? sqrtf(6.0f / 64.0f) : sqrtf(3.0f / 64.0f);
        w[(size_t)i] = u * lim;
    }
    nrc_set_weights(ctx, net, w.data());
}

// mma.sync fragments of w (forward and backward) and of the inference
// weights (the EMA when enabled).
static void nrc_pack_frags(aqua_ctx* ctx, NrcNet& net) {
    int total = kFragFwd + kFragBwd;
    k_nrc_pack<<<(total + 255) / 256, 256, 0, ctx->stream>>>(net.w, net.frag, net.fragT);
    const float* inf = net.ema_decay > 0.0f ? net.ema : net.w;
    k_nrc_pack<<<(kFragFwd + 255) / 256, 256, 0, ctx->stream>>>(inf, net.frag_inf, nullptr);
    AQ_CUDA(cudaGetLastError());
}

void nrc_pack(aqua_ctx* ctx, NrcNet& net) {
    nrc_pack_frags(ctx, net);
    if (net.forward_tc)
        nrc_pack_tc(ctx, net.w, net.ema_decay > 0.0f ? net.ema : net.w, net.img_tc_w, net.img_tc, net.img_tc_bwd);
}

void nrc_set_weights(aqua_ctx* ctx, NrcNet& net, const float* host_w) {
    AQ_CUDA(cudaMemcpyAsync(net.w, host_w, 4 * kNrcParams, cudaMemcpyHostToDevice, ctx->stream));
    AQ_CUDA(cudaMemsetAsync(net.m, 0, 4 * kNrcParams, ctx->stream));
    AQ_CUDA(cudaMemsetAsync(net.v, 0, 4 * kNrcParams, ctx->stream));
    AQ_CUDA(cudaMemsetAsync(net.grad, 0, 4 * kNrcParams, ctx->stream));
    AQ_CUDA(cudaMemcpyAsync(net.ema, net.w, 4 * kNrcParams, cudaMemcpyDeviceToDevice, ctx->stream));
    net.step = 0;
    nrc_pack(ctx, net);
    AQ_CUDA(cudaStreamSynchronize(ctx->stream));
}

static int nrc_grid(aqua_ctx* ctx, int rows) {
    int tiles = (rows + 15) / 16;
    int blocks = (tiles + 3) / 4;
    return std::max(1, std::min(blocks, ctx->num_sms * 8));
}

void nrc_forward_dev(aqua_ctx* ctx, NrcNet& net, const uint16_t* X, int n, float* out) {
    if (n <= 0) return;
    if (net.forward_tc) {
        nrc_forward_tc_dev(ctx, net.img_tc, X, n, out, net.tc_err);
        return;
    }
    k_nrc_forward<false><<<nrc_grid(ctx, n), 128, 0, ctx->stream>>>(reinterpret_cast<const uint32_t*>(X), n,
                                                                     net.frag_inf, out, nullptr);
    AQ_CUDA(cudaGetLastError());
}

static void ensure_train(aqua_ctx* ctx, NrcNet& net, int n) {
    if (net.train.ptr && net.train_rows >= n) return;
    dev_free(net.train);
    int rows = std::max(n, 1024);
    int chunks = (rows + kWgChunk - 1) / kWgChunk;
    size_t off = 0;
    auto take = [&](size_t b) { size_t o = off; off = rup(off + b, 256); return o; };
    size_t o_y = take(12 * (size_t)rows), o_a = take(5 * 128 * (size_t)rows), o_d = take(5 * 128 * (size_t)rows),
           o_6 = take(32 * (size_t)rows), o_p = take(4 * (size_t)kNrcParams * chunks);
    dev_alloc(ctx, net.train, off);
    char* b = (char*)net.train.ptr;
    net.ty = (float*)(b + o_y);
    net.acts = (uint32_t*)(b + o_a);
    net.deltas = (uint32_t*)(b + o_d);
    net.d6 = (uint32_t*)(b + o_6);
    net.partial = (float*)(b + o_p);
    net.train_rows = rows;
}

void nrc_train_step_dev(aqua_ctx* ctx, NrcNet& net, const uint16_t* X, const float* target, int n) {
    if (n <= 0) return;
    ensure_train(ctx, net, n);
    cudaStream_t st = ctx->stream;
    const uint32_t* Xw = reinterpret_cast<const uint32_t*>(X);
    int g = nrc_grid(ctx, n);
    // On tcgen05 the four launches of a step (and of consecutive steps) are
    // chained (programmatic dependent launch); the forward pass zeroes the
    // loss word and Adam writes the next step's weight images.
    if (net.forward_tc) {
        nrc_forward_tc_dev(ctx, net.img_tc_w, X, n, net.ty, net.tc_err, net.acts, net.loss);
    } else {
        k_nrc_forward<true><<<g, 128, 0, st>>>(Xw, n, net.frag, net.ty, net.acts);
        AQ_CUDA(cudaMemsetAsync(net.loss, 0, 8, st));
    }
    if (net.forward_tc)
        nrc_backward_tc_dev(ctx, net.img_tc_bwd, net.ty, target, n, 1.0f / (float)(n * kNrcOut), net.acts,
                            net.deltas, net.d6, net.loss, net.tc_err);
    else
        k_nrc_backward<<<g, 128, 0, st>>>(net.ty, target, n, 1.0f / (float)(n * kNrcOut), net.fragT, net.acts,
                                          net.deltas, net.d6, net.loss);
    int chunks;
    if (net.forward_tc) {
        chunks = nrc_wgrad_tc_dev(ctx, X, net.acts, net.deltas, net.d6, n, net.partial, net.tc_err);
    } else {
        chunks = (n + kWgChunk - 1) / kWgChunk;
        k_nrc_wgrad<<<dim3(chunks, 6), 128, 0, st>>>(Xw, net.acts, net.deltas, net.d6, n, net.partial);
    }
    net.step++;
    float c1 = 1.0f - powf(net.beta1, (float)net.step), c2 = 1.0f - powf(net.beta2, (float)net.step);
    launch_chained(k_nrc_adam, dim3((kNrcParams + 255) / 256), dim3(256), 0, st, (const float*)net.partial, chunks,
                   net.w, net.m, net.v, net.grad, net.lr, net.beta1, net.beta2, net.eps, c1, c2, net.ema,
                   net.ema_decay, net.forward_tc ? net.img_tc_w : nullptr, net.img_tc, net.img_tc_bwd);
    if (!net.forward_tc) nrc_pack_frags(ctx, net);
    AQ_CUDA(cudaGetLastError());
    net.launches += net.forward_tc ? 4 : 6;
}

void nrc_check_tc(aqua_ctx* ctx, NrcNet& net) {
    if (!net.forward_tc) return;
    uint32_t e = 0;
    AQ_CUDA(cudaMemcpyAsync(&e, net.tc_err, 4, cudaMemcpyDeviceToHost, ctx->stream));
    AQ_CUDA(cudaStreamSynchronize(ctx->stream));
    if (e) {
        AQ_CUDA(cudaMemsetAsync(net.tc_err, 0, 4, ctx->stream));
        throw Error(AQUA_ERR_TIMEOUT, "tensor-core inference: an MMA completion wait expired");
    }
}

void nrc_encode_dev(aqua_ctx* ctx, NrcNet& net, const float* raw, int n, uint16_t* X) {
    if (n <= 0) return;
    float3 bmin = make_float3(net.bmin[0], net.bmin[1], net.bmin[2]);
    float3 binv = make_float3(1.0f / net.bext[0], 1.0f / net.bext[1], 1.0f / net.bext[2]);
    launch_chained(k_nrc_encode, dim3((n + kEncRows - 1) / kEncRows), dim3(kEncRows), 0, ctx->stream, raw, n, bmin,
                   binv, X);
    AQ_CUDA(cudaGetLastError());
}

}  // namespace aq
