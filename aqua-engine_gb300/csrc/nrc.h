// nrc.h — the learned radiance cache's network shape and input encoding.
//
// The reference names the integrator `"type": "nrc"` with batch_size,
// training_iters and learning_rate (scenes/integrator.json:2-7) but ships no
// implementation. This follows Mueller et al. 2021, "Real-time Neural
// Radiance Caching for Path Tracing" (SIGGRAPH): a small fully-connected
// network, trained online on radiance the path tracer produces, queried to
// end paths early.
//
// Network: 64 inputs -> 5 hidden layers of 64 (ReLU) -> 3 outputs (RGB
// radiance), no biases (input 63 is a constant 1). Weights are stored
// row-major [out][in]: W1..W5 64x64, W6 3x64 = 20,672 parameters.
//
// Input encoding (64 values) of a path vertex:
//   0..47  position: frequency encoding, 8 octaves of sin/cos per axis over
//          the scene box (finest period 1/128 of the box)
//   48..53 outgoing direction: spherical coordinates, one-blob with 3 bins
//          each (Mueller et al. 2019, "Neural Importance Sampling")
//   54..57 normal: spherical coordinates, one-blob with 2 bins each
//   58     roughness
//   59..61 diffuse albedo
//   62     luminance of the specular F0
//   63     constant 1
#pragma once

#include <math.h>
#include <stdint.h>

#include "aq_math.h"

namespace aq {

constexpr int kNrcIn = 64;
constexpr int kNrcHidden = 64;
constexpr int kNrcHiddenLayers = 5;
constexpr int kNrcOut = 3;
constexpr int kNrcParams = kNrcHiddenLayers * kNrcHidden * kNrcIn + kNrcOut * kNrcHidden;  // 20672
constexpr int kNrcRaw = 16;  // raw vertex features, floats

// Tensor-core weight images, bf16 in the no-swizzle K-major operand layout
// (element (r, k) of an R-row tile at (k / 8) R 16 + r 16 + (k % 8) 2 bytes).
// Forward image: W1..W5 as 64-row tiles (rows = outputs, K = inputs), then
// W6 padded to 16 rows. Backward image: W6^T (64 rows = inputs, K = 16
// outputs, 3 used), then W5^T..W2^T. Padding stays zero.
constexpr int kNrcTcLayerBytes = 64 * 64 * 2;  // 8 KB
constexpr int kNrcTcOutRows = 16;
constexpr int kNrcTcBwdW6Bytes = 64 * 16 * 2;  // 2 KB

AQ_HD constexpr uint32_t nrc_tc_offset(int rows, int r, int k) {
    return (uint32_t)((k >> 3) * rows * 16 + r * 16 + (k & 7) * 2);
}

// Byte offsets of parameter p (row-major [out][in] per layer) in the forward
// image and in the backward image; bwd = -1 for W1, which it leaves out.
AQ_HD void nrc_tc_param_offsets(int p, uint32_t& fwd, int32_t& bwd) {
    const int hidden = kNrcHiddenLayers * kNrcHidden * kNrcIn;
    if (p < hidden) {
        const int l = p / 4096, o = (p / 64) % 64, i = p % 64;
        fwd = (uint32_t)(l * kNrcTcLayerBytes) + nrc_tc_offset(64, o, i);
        bwd = l == 0 ? -1 : (int32_t)(kNrcTcBwdW6Bytes + (4 - l) * kNrcTcLayerBytes + nrc_tc_offset(64, i, o));
    } else {
        const int j = p - hidden, o = j / 64, i = j % 64;
        fwd = (uint32_t)(5 * kNrcTcLayerBytes) + nrc_tc_offset(kNrcTcOutRows, o, i);
        bwd = (int32_t)nrc_tc_offset(64, i, o);
    }
}

// Raw vertex features, 16 floats: position (3), outgoing direction (3),
// normal (3), roughness (1), diffuse albedo (3), specular F0 (3).
struct NrcRaw {
    float p[3], w[3], n[3], rough, kd[3], ks[3];
};

// One-blob: value of bin b (of k) for x in [0,1], Gaussian of width 1/k.
AQ_HD float one_blob(float x, int b, int k) {
    float c = ((float)b + 0.5f) / (float)k;
    float d = (x - c) * (float)k;
    return expf(-0.5f * d * d);
}

AQ_HD float nrc_wrap01(float x) { return fminf_(fmaxf_(x, 0.0f), 1.0f); }

// Spherical coordinates of a unit vector, each mapped to [0,1].
AQ_HD void sph01(float x, float y, float z, float& u, float& v) {
    u = acosf(fminf_(fmaxf_(z, -1.0f), 1.0f)) * kInvPi;
    v = (atan2f(y, x) + kPi) * (0.5f * kInvPi);
    u = nrc_wrap01(u);
    v = nrc_wrap01(v);
}

}  // namespace aq
