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
// radiance), no biases (input 62 is a constant 1). Weights are stored
// row-major [out][in]: W1..W5 64x64, W6 3x64 = 20,672 parameters.
//
// Input encoding (64 values) of a path vertex: position (frequency encoding,
// 6 octaves of sin/cos per axis over the scene box), outgoing direction and
// normal (spherical coordinates, one-blob with 4 bins each; Mueller et al.
// 2019, "Neural Importance Sampling"), roughness (one-blob, 4 bins), diffuse
// and specular albedo, a constant 1 and a 0.
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

// Encoded value c (0..63) of a vertex; pn = position normalised to [0,1]^3.
AQ_HD float nrc_encode_one(const NrcRaw& r, const float pn[3], int c) {
    if (c < 36) {
        int axis = c / 12, f = (c % 12) / 2;
        float x = pn[axis] * (float)(1 << f) * kPi;
        return (c & 1) ? cosf(x) : sinf(x);
    }
    if (c < 44) {
        float u, v;
        sph01(r.w[0], r.w[1], r.w[2], u, v);
        int k = c - 36;
        return one_blob(k < 4 ? u : v, k & 3, 4);
    }
    if (c < 52) {
        float u, v;
        sph01(r.n[0], r.n[1], r.n[2], u, v);
        int k = c - 44;
        return one_blob(k < 4 ? u : v, k & 3, 4);
    }
    if (c < 56) return one_blob(nrc_wrap01(r.rough), c - 52, 4);
    if (c < 59) return r.kd[c - 56];
    if (c < 62) return r.ks[c - 59];
    return c == 62 ? 1.0f : 0.0f;
}

}  // namespace aq
