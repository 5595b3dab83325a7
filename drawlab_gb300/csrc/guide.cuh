// Learned path-guiding proposal: a small MLP maps (position, normal) of a
// shading point to a mixture of von Mises-Fisher lobes over incident
// directions.  Device code shared by the renderer (inference inside the
// guided material kernels) and by the training kernels (guide.cu).
//
// Network (FP16 weights and activations, FP32 accumulation on the tensor
// cores with tcgen05.mma: inference in guide_tc.cuh, training in guide.cu):
//   input   6 scalars: position scaled to [0, 1]^3 by the scene bounds,
//           shading normal in [-1, 1]^3
//   encode  sin / cos (2^(k-3) pi x), k = 0..11, for each scalar: 144 features
//   layer 1 144 -> 64, ReLU
//   layer 2  64 -> 64, ReLU
//   layer 3  64 -> 40 (rows 40..47 of the padded weight are zero)
//   output  8 lobes x (mean direction m (3, normalised), log kappa, logit)
//           kappa = exp(clamp(log kappa, -3, 8)), weights = softmax(logits)
// vMF lobe: pdf(w) = kappa / (2 pi (1 - e^{-2 kappa})) exp(kappa (mu.w - 1)).
#pragma once

#include <cuda_fp16.h>

#include "device.cuh"

namespace dl {

constexpr int kGIn = 6;
constexpr int kGFreq = 12;
constexpr int kGEnc = kGIn * kGFreq * 2;  // 144
constexpr int kGHid = 64;
constexpr int kGLobes = 8;
constexpr int kGOut = 5 * kGLobes;         // 40
constexpr int kGOutPad = 48;
// parameter layout (floats / halves, one contiguous array)
constexpr int kGW1 = 0;
constexpr int kGB1 = kGW1 + kGHid * kGEnc;
constexpr int kGW2 = kGB1 + kGHid;
constexpr int kGB2 = kGW2 + kGHid * kGHid;
constexpr int kGW3 = kGB2 + kGHid;
constexpr int kGB3 = kGW3 + kGOutPad * kGHid;
constexpr int kGParams = kGB3 + kGOutPad;  // 16560
constexpr float kGLogKappaMin = -3.f, kGLogKappaMax = 8.f;

struct GuideRecord {   // one training sample, 48 bytes
    float in[6];       // position in [0, 1]^3, normal
    float w[3];        // sampled direction
    float pdf;         // its sampling pdf (solid angle)
    float L;           // radiance estimate along w (scalar)
    float pad;
};
static_assert(sizeof(GuideRecord) == 48, "record layout");

struct GuideNet {
    const void* image;   // the weight image of the tensor-core kernels (guide_tc.cuh)
    float fraction;      // probability of sampling the learned proposal
    int max_depth;       // vertices at depth >= max_depth sample the BSDF alone
    int blocks;          // grid of the guided material kernels (host side)
};

// ------------------------------------------------------------- encoding
// sin / cos of (2^(k-3) pi x) for k = 0..11 (periods from 16 scene units
// down to 1/128): sincospi at k = 0 and 6, double-angle steps in between
// (at most five; largest error 1.1e-5 over x in [-1, 1], below the fp16
// spacing the encodings are rounded to near +-1).
constexpr int kGFreqShift = 3;
constexpr int kGFreqAnchor = 6;   // frequencies per sincospi
__device__ __forceinline__ void encode_scalar_h2(float x, __half2* out) {
#pragma unroll
    for (int k0 = 0; k0 < kGFreq; k0 += kGFreqAnchor) {
        float s, c;
        sincospif(x * ((float)(1 << k0) / (float)(1 << kGFreqShift)), &s, &c);
#pragma unroll
        for (int k = 0; k < kGFreqAnchor; k++) {
            out[k0 + k] = __floats2half2_rn(s, c);  // (sin, cos): sin at the lower address
            float s2 = 2.f * s * c, c2 = 1.f - 2.f * s * s;
            s = s2;
            c = c2;
        }
    }
}

// -------------------------------------------------------------- mixture
struct VmfLobe {
    float3 mu;
    float kappa;
    float lambda;
    float inv_len;  // 1 / |m| (for gradients)
    bool clamped;   // log kappa outside [min, max]
};

// Lobes from the 40 network outputs at `o` (stride 1).
__device__ __forceinline__ void decode_lobes(const float* o, VmfLobe* L) {
    float mx = -1e30f;
#pragma unroll
    for (int j = 0; j < kGLobes; j++) mx = fmaxf(mx, o[5 * j + 4]);
    float sum = 0.f;
#pragma unroll
    for (int j = 0; j < kGLobes; j++) {
        float3 m = f3(o[5 * j], o[5 * j + 1], o[5 * j + 2]);
        float len = sqrtf(m.x * m.x + m.y * m.y + m.z * m.z);
        if (len > 1e-6f) {
            L[j].mu = f3(m.x / len, m.y / len, m.z / len);
            L[j].inv_len = 1.f / len;
        } else {
            L[j].mu = f3(0.f, 0.f, 1.f);
            L[j].inv_len = 0.f;
        }
        float lk = o[5 * j + 3];
        L[j].clamped = lk < kGLogKappaMin || lk > kGLogKappaMax;
        L[j].kappa = expf(fminf(fmaxf(lk, kGLogKappaMin), kGLogKappaMax));
        L[j].lambda = expf(o[5 * j + 4] - mx);
        sum += L[j].lambda;
    }
#pragma unroll
    for (int j = 0; j < kGLobes; j++) L[j].lambda /= sum;
}

__device__ __forceinline__ float vmf_pdf(float3 mu, float kappa, float3 w) {
    float d = mu.x * w.x + mu.y * w.y + mu.z * w.z;
    if (kappa < 1e-4f) return 0.25f * kInvPiF;
    return kappa / (2.f * kPiF * (-expm1f(-2.f * kappa))) * expf(kappa * (d - 1.f));
}

// Decoded lobes as the renderer stores them: 8 x {mu.x, mu.y, mu.z, k, c,
// lambda} floats, with k = kappa (0 for kappa < 1e-4: the uniform sphere)
// and c = lambda times the lobe's normalisation, so that
//   q(w) = sum_j c_j exp(k_j (mu_j . w - 1)).
constexpr int kGLobeFloats = 6;
constexpr int kGStoredLobes = kGLobes * kGLobeFloats;  // 48

// Decodes the 40 network outputs at `o` in place into the stored form (48
// floats from `o`; lobes in descending order, so lobe j's outputs
// [5j, 5j + 5) are read before its stored floats [6j, 6j + 6) are written).
__device__ __forceinline__ void decode_lobes_inplace(float* o) {
    float mx = -1e30f;
#pragma unroll
    for (int j = 0; j < kGLobes; j++) mx = fmaxf(mx, o[5 * j + 4]);
    float sum = 0.f;
#pragma unroll
    for (int j = kGLobes - 1; j >= 0; j--) {
        const float m0 = o[5 * j], m1 = o[5 * j + 1], m2 = o[5 * j + 2], lk = o[5 * j + 3], lg = o[5 * j + 4];
        const float len = sqrtf(m0 * m0 + m1 * m1 + m2 * m2);
        float3 mu = f3(0.f, 0.f, 1.f);
        if (len > 1e-6f) mu = f3(m0 / len, m1 / len, m2 / len);
        const float kappa = expf(fminf(fmaxf(lk, kGLogKappaMin), kGLogKappaMax));
        const float lam = expf(lg - mx);
        sum += lam;
        const bool uniform = kappa < 1e-4f;
        const float norm = uniform ? 0.25f * kInvPiF : kappa / (2.f * kPiF * (-expm1f(-2.f * kappa)));
        o[6 * j] = mu.x;
        o[6 * j + 1] = mu.y;
        o[6 * j + 2] = mu.z;
        o[6 * j + 3] = uniform ? 0.f : kappa;
        o[6 * j + 4] = lam * norm;
        o[6 * j + 5] = lam;
    }
    const float inv = 1.f / sum;
#pragma unroll
    for (int j = 0; j < kGLobes; j++) {
        o[6 * j + 4] *= inv;
        o[6 * j + 5] *= inv;
    }
}

__device__ __forceinline__ float stored_mixture_pdf(const float* lob, float3 w) {
    float p = 0.f;
#pragma unroll
    for (int j = 0; j < kGLobes; j++) {
        const float* l = lob + kGLobeFloats * j;
        const float d = l[0] * w.x + l[1] * w.y + l[2] * w.z;
        p += l[4] * __expf(l[3] * (d - 1.f));
    }
    return p;
}

// Sample a direction: lobe by its weight (u0), then the vMF lobe (Jakob's
// stable inversion of the cosine's distribution, u = (u1, u2)); k = 0 lobes
// are uniform over the sphere.
__device__ __forceinline__ float3 stored_mixture_sample(const float* lob, float u0, float2 u) {
    int j = kGLobes - 1;
    float acc = 0.f;
#pragma unroll
    for (int i = 0; i < kGLobes - 1; i++) {
        acc += lob[kGLobeFloats * i + 5];
        if (u0 < acc) {
            j = i;
            break;
        }
    }
    const float* l = lob + kGLobeFloats * j;
    const float k = l[3];
    float w;
    if (k == 0.f) {
        w = 2.f * u.x - 1.f;
    } else {
        w = 1.f + logf(u.x + (1.f - u.x) * expf(-2.f * k)) / k;
    }
    w = fminf(fmaxf(w, -1.f), 1.f);
    float v = sqrtf(fmaxf(0.f, 1.f - w * w));
    float s, c;
    sincospif(2.f * u.y, &s, &c);
    Frame f = make_onb(f3(l[0], l[1], l[2]));
    float3 loc = f3(v * c, v * s, w);
    return normalize(to_world(f, loc));
}

// Network input of a shading point: position scaled into [0, 1]^3 by the
// scene bounds, the unit shading normal.
__device__ __forceinline__ void guide_input(const DevScene& sc, float3 p, float3 n, float* in6) {
    in6[0] = fminf(fmaxf((p.x - sc.bb_lo[0]) * sc.bb_inv_ext[0], 0.f), 1.f);
    in6[1] = fminf(fmaxf((p.y - sc.bb_lo[1]) * sc.bb_inv_ext[1], 0.f), 1.f);
    in6[2] = fminf(fmaxf((p.z - sc.bb_lo[2]) * sc.bb_inv_ext[2], 0.f), 1.f);
    in6[3] = n.x;
    in6[4] = n.y;
    in6[5] = n.z;
}

}  // namespace dl
