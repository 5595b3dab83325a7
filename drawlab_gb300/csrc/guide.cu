// Training and inference of the learned path-guiding proposal (guide.cuh)
// on the fifth-generation tensor cores, and the dl_guide C ABI.
//
// One training step on a batch of n records {position, normal, sampled
// direction w, its sampling pdf p, radiance estimate L along w}:
//   loss = -(1/n) sum_i min((L_i / p_i) / mean(L / p), 20) * log q(w_i)
// (an estimate of the KL divergence from the normalised incident radiance to
// the mixture q, up to a constant), then one Adam update.  Kernels:
//   k_guide_weight_sum   mean(L / p) over the batch
//   k_guide_train_tc     forward, loss gradient, backward and the weight and
//                        bias gradients of the whole batch (tcgen05.mma)
//   k_guide_adam         Adam on the fp32 master weights; refreshes the fp16
//                        copy and the tensor cores' weight image
// Inference (k_guide_infer, and the guided material kernels in render.cu)
// runs on tcgen05 too (guide_tc.cuh).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "guide.cuh"
#include "guide_tc.cuh"
#include "internal.h"
#include "scene.h"

namespace dl {

// ------------------------------------------------------------- inference
static_assert(kGImgTrainBytes == kGuideImageBytes, "image size");

// Raw network outputs (40 per row) of n input rows, 128 rows per tile on
// the tensor cores; each of a block's two warpgroups walks its own tiles.
__global__ void __launch_bounds__(kTcThreads) k_guide_infer(const void* image, const float* in, float* out, int n,
                                                             unsigned* err) {
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    GuideTcSmem& S = *reinterpret_cast<GuideTcSmem*>(dyn_smem);
    const int ntiles = (n + kTcRows - 1) / kTcRows;
    if ((int)blockIdx.x * kTcGroups >= ntiles) return;
    const int g = tc_group(), row = tc_row();
    uint32_t phase = 0;
    bool ok = guide_tc_begin(S, image, err);
    for (int tile = blockIdx.x * kTcGroups + g; ok && tile < ntiles; tile += gridDim.x * kTcGroups) {
        const int r = tile * kTcRows + row;
        float x[kGIn] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (r < n)
            for (int i = 0; i < kGIn; i++) x[i] = in[(size_t)kGIn * r + i];
        wg_sync(g);  // the previous tile's outputs have been read
        encode_row_tc(x, S.act[g], row);
        ok = guide_tc_forward(S, g, phase, err);
        if (ok) {
            // the tile's rows are contiguous in `out`: copy them out as
            // consecutive 16-byte chunks (coalesced stores), 10 per row
            wg_sync(g);
            const int rows = min(kTcRows, n - tile * kTcRows);
            float4* dst = reinterpret_cast<float4*>(out + (size_t)tile * kTcRows * kGOut);
            const float* src = tc_out_row(S, g, 0);
            for (int c = row; c < rows * (kGOut / 4); c += kTcRows) {
                const float* q = src + (c / (kGOut / 4)) * kTcOutStride + 4 * (c % (kGOut / 4));
                dst[c] = make_float4(q[0], q[1], q[2], q[3]);
            }
        }
    }
    guide_tc_end(S, phase);
}

// -------------------------------------------------------------- training
// Record weights L/p are normalised by their batch mean and clamped at this
// multiple of it: a few records near the sun would otherwise carry the
// whole gradient of a batch.
constexpr float kGTargetClamp = 20.f;

__global__ void k_guide_weight_sum(const GuideRecord* s, int n, int stride, float* sum) {
    float acc = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const GuideRecord& r = s[(size_t)i * stride];
        acc += r.pdf > 0.f ? r.L / r.pdf : 0.f;
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(sum, acc);
}

// The loss of one record and dLoss/dOutput (40 values, scaled by `scale`).
__device__ __forceinline__ float record_grad(const float* o, const GuideRecord& s, float scale, float* d) {
    VmfLobe L[kGLobes];
    decode_lobes(o, L);
    const float3 w = f3(s.w[0], s.w[1], s.w[2]);
    float pj[kGLobes], q = 0.f;
#pragma unroll
    for (int j = 0; j < kGLobes; j++) {
        pj[j] = L[j].lambda * vmf_pdf(L[j].mu, L[j].kappa, w);
        q += pj[j];
    }
    for (int j = 0; j < kGOut; j++) d[j] = 0.f;
    if (!(q > 1e-30f) || !(scale > 0.f) || !isfinite(scale)) return 0.f;
#pragma unroll
    for (int j = 0; j < kGLobes; j++) {
        const float r = pj[j] / q, k = L[j].kappa;
        const float3 mu = L[j].mu;
        const float dot = mu.x * w.x + mu.y * w.y + mu.z * w.z;
        // d(-log q)/d(logit_j) = -(r_j - lambda_j)
        d[5 * j + 4] = -scale * (r - L[j].lambda);
        // d(-log q)/d(log kappa_j) = -r_j (1 - 2k / (e^{2k} - 1) + k (mu.w - 1))
        if (!L[j].clamped) {
            float t = k < 1e-4f ? 0.f : 1.f - 2.f * k / expm1f(2.f * k) + k * (dot - 1.f);
            d[5 * j + 3] = -scale * r * t;
        }
        // d(-log q)/dm_j = -r_j kappa_j (w - (mu.w) mu) / |m_j|
        const float f = -scale * r * k * L[j].inv_len;
        d[5 * j + 0] = f * (w.x - dot * mu.x);
        d[5 * j + 1] = f * (w.y - dot * mu.y);
        d[5 * j + 2] = f * (w.z - dot * mu.z);
    }
    return -scale * logf(q);
}

// One training batch on the tensor cores (k_guide_train_tc).  A persistent
// 128-thread block walks 128-record tiles; per tile, each thread owns one
// record and every product is a tcgen05.mma issued by thread 0 with the
// accumulator in tensor memory:
//   forward   x -> h1 -> h2 -> outputs (3 products, as in inference)
//   loss      dLoss/dOutput of the thread's record: d0 (fp16)
//   backward  d2 = (d0 W3) * [h2 > 0],  d1 = (d2 W2) * [h1 > 0]
//             (B operands W3^T, W2^T from the weight image)
//   weights   [dW1 | . | g_b1 ; . | dW2 | g_b2] += [d1 | d2]^T [x | h1 | 1]
//             [g_b3 | dW3] += d0^T [1 | h2]
// The two weight-gradient products read the activation tiles written for
// the forward and backward products as MN-major operands (M or N = the
// features, K = the tile's 128 records) and accumulate over all of the
// block's tiles in tensor memory; bias gradients come from the columns of
// ones.  At the end each warp reads its 32 accumulator lanes and adds them
// to the gradient in global memory.
//
// Loss scaling: the fp16 activation gradients leave out the loss's 1/n
// (with n ~ 3e4 records most of them would be fp16 subnormals); they
// saturate at the fp16 range, and the 1/n is applied, in fp32, when the
// accumulators are added to the gradient.
//
// Shared memory: the weight image (47,808 B), Z = [x | h1 | 1 | h2] (288
// halves per record) and D = [d0 | d1 | d2] (176 halves per record), both in
// the canonical layout.  166 KB per block: one block per SM, and no other
// tensor-core kernel of this library (70 KB each) fits beside it, so its 512
// tensor-memory columns are always free.
constexpr int kZK = 288, kDK = 176;                    // halves per record in Z and D
constexpr int kZx = 0, kZh1 = 144, kZones = 208, kZh2 = 224;
constexpr int kDd0 = 0, kDd1 = 48, kDd2 = 112;
constexpr int kTrainCols = 512;
constexpr int kAccW12 = 64, kAccW3 = kAccW12 + 224;   // accumulator columns ([0, 64): layer products)
constexpr float kHalfMax = 65504.f;

struct GuideTrainSmem {
    __half w[kGImgHalves];
    float bias[kGImgBiases];
    __half w2t[kGHid * kGHid];
    __half w3t[kGHid * kGOutPad];
    alignas(128) __half z[kTcRows * kZK];
    alignas(128) __half d[kTcRows * kDK];
    uint64_t bar_w, bar_mma, bar_g;
    uint32_t tmem;
    int fail;
};
static_assert(offsetof(GuideTrainSmem, w2t) == kGImgW2T && offsetof(GuideTrainSmem, w3t) == kGImgW3T,
              "image layout");
static_assert(sizeof(GuideTrainSmem) > 116 * 1024 + 1024, "one training block per SM");
static_assert(sizeof(GuideTrainSmem) + sizeof(GuideTcSmem) > 228 * 1024, "no inference block beside it");

__device__ __forceinline__ uint32_t pack_h2(float a, float b) {
    __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}
__device__ __forceinline__ uint32_t pack_h2_sat(float a, float b) {
    return pack_h2(fminf(fmaxf(a, -kHalfMax), kHalfMax), fminf(fmaxf(b, -kHalfMax), kHalfMax));
}

// Bias + ReLU of 64 accumulator columns into Z at feature f0 (fp16);
// returns the mask of the outputs that are > 0 after rounding.
__device__ __forceinline__ uint64_t train_hidden_epilogue(GuideTrainSmem& S, uint32_t t, const float* bias, int f0) {
    const int r = threadIdx.x;
    uint64_t mask = 0;
#pragma unroll
    for (int c0 = 0; c0 < kGHid; c0 += 16) {
        float v[16];
        tc::ld_32x32b_x16(t + c0, v);
        uint32_t p[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            __half2 h = __floats2half2_rn(fmaxf(v[2 * j] + bias[c0 + 2 * j], 0.f),
                                          fmaxf(v[2 * j + 1] + bias[c0 + 2 * j + 1], 0.f));
            if (__low2float(h) > 0.f) mask |= 1ull << (c0 + 2 * j);
            if (__high2float(h) > 0.f) mask |= 1ull << (c0 + 2 * j + 1);
            p[j] = *reinterpret_cast<const uint32_t*>(&h);
        }
        *reinterpret_cast<uint4*>(S.z + canon_index(r, f0 + c0, kZK)) = make_uint4(p[0], p[1], p[2], p[3]);
        *reinterpret_cast<uint4*>(S.z + canon_index(r, f0 + c0 + 8, kZK)) = make_uint4(p[4], p[5], p[6], p[7]);
    }
    return mask;
}

// 64 accumulator columns masked by `mask` into D at feature f0 (fp16).
__device__ __forceinline__ void train_backward_epilogue(GuideTrainSmem& S, uint32_t t, uint64_t mask, int f0) {
    const int r = threadIdx.x;
#pragma unroll
    for (int c0 = 0; c0 < kGHid; c0 += 16) {
        float v[16];
        tc::ld_32x32b_x16(t + c0, v);
        uint32_t p[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const float a = (mask >> (c0 + 2 * j)) & 1ull ? v[2 * j] : 0.f;
            const float b = (mask >> (c0 + 2 * j + 1)) & 1ull ? v[2 * j + 1] : 0.f;
            p[j] = pack_h2_sat(a, b);
        }
        *reinterpret_cast<uint4*>(S.d + canon_index(r, f0 + c0, kDK)) = make_uint4(p[0], p[1], p[2], p[3]);
        *reinterpret_cast<uint4*>(S.d + canon_index(r, f0 + c0 + 8, kDK)) = make_uint4(p[4], p[5], p[6], p[7]);
    }
}

// K-major product of one layer: acc (128 x N) = A (Z or D at feature f0,
// rows of `a_rowlen` halves) x W^T, W [N][K] at `w` (rows of K halves).
template <int K, int N>
__device__ __forceinline__ void train_issue(uint32_t acc, uint32_t a_base, int a_rowlen, int f0, uint32_t w) {
    constexpr uint32_t idesc = tc::idesc_f16_f32(kTcRows, N);
    tc::fence_after_sync();
#pragma unroll
    for (int ks = 0; ks < K / 16; ks++)
        tc::mma_f16(acc, tc::smem_desc(a_base + (f0 / 8 + 2 * ks) * 128, 128, a_rowlen * 16),
                    tc::smem_desc(w + ks * 256, 128, K * 16), idesc, ks > 0 ? 1u : 0u);
}

__global__ void __launch_bounds__(kTcRows) k_guide_train_tc(const void* image, const GuideRecord* s, int n,
                                                             int stride, const float* wsum, float* grad,
                                                             float* loss, unsigned* err) {
    extern __shared__ __align__(128) unsigned char dyn_smem[];
    GuideTrainSmem& S = *reinterpret_cast<GuideTrainSmem*>(dyn_smem);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int ntiles = (n + kTcRows - 1) / kTcRows;
    if ((int)blockIdx.x >= ntiles) return;
    if (tid == 0) {
        tc::mbar_init(&S.bar_w, 1);
        tc::mbar_init(&S.bar_mma, 1);
        tc::mbar_init(&S.bar_g, 1);
        S.fail = 0;
    }
    if (tid < 32) tc::tmem_alloc(&S.tmem, kTrainCols);
    {   // the columns of ones (features 208..223 of every record)
        const uint32_t one2 = pack_h2(1.f, 1.f);
        *reinterpret_cast<uint4*>(S.z + canon_index(tid, kZones, kZK)) = make_uint4(one2, one2, one2, one2);
        *reinterpret_cast<uint4*>(S.z + canon_index(tid, kZones + 8, kZK)) = make_uint4(one2, one2, one2, one2);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) tc::bulk_load(S.w, image, kGImgTrainBytes, &S.bar_w);
    bool failed = !tc::mbar_wait(&S.bar_w, 0, kTcWaitNs);
    if (failed) {
        S.fail = 1;
        atomicOr(err, kErrTensorWait);
    }
    uint32_t ph = 0, phg = 0;
    auto wait = [&](uint64_t* bar, uint32_t& parity) {
        if (!tc::mbar_wait(bar, parity, kTcWaitNs)) {
            failed = true;
            S.fail = 1;
            atomicOr(err, kErrTensorWait);
        } else {
            parity ^= 1u;
        }
        tc::fence_after_sync();
    };
    const uint32_t T = S.tmem;
    const uint32_t tl = T + ((uint32_t)(tid & ~31) << 16);  // this warp's lanes, column 0
    const uint32_t za = tc::smem_addr(S.z), da = tc::smem_addr(S.d), wa = tc::smem_addr(S.w);
    const float mean = *wsum / (float)n;
    const float inv_n = 1.f / (float)n;
    float lacc = 0.f;
    bool pending = false, first = true;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int r = tile * kTcRows + tid;
        GuideRecord rec = {};
        float sc = 0.f;  // the record's loss weight times n
        if (r < n) {
            rec = s[(size_t)r * stride];
            if (rec.pdf > 0.f && mean > 0.f) sc = fminf(rec.L / rec.pdf / mean, kGTargetClamp);
        }
        // the previous tile's weight-gradient products read Z and D
        if (pending) wait(&S.bar_g, phg);
        pending = false;
        encode_row_tc(rec.in, S.z, tid, kZK);
        tc::fence_smem_to_async();
        tc::fence_before_sync();
        if (__syncthreads_or(failed)) break;
        // forward
        if (tid == 0) {
            train_issue<kGEnc, kGHid>(T, za, kZK, kZx, wa + 2 * kGImgW1);
            tc::commit(&S.bar_mma);
        }
        wait(&S.bar_mma, ph);
        const uint64_t m1 = train_hidden_epilogue(S, tl, S.bias + kGImgB1, kZh1);
        tc::fence_smem_to_async();
        tc::fence_before_sync();
        if (__syncthreads_or(failed)) break;
        if (tid == 0) {
            train_issue<kGHid, kGHid>(T, za, kZK, kZh1, wa + 2 * kGImgW2);
            tc::commit(&S.bar_mma);
        }
        wait(&S.bar_mma, ph);
        const uint64_t m2 = train_hidden_epilogue(S, tl, S.bias + kGImgB2, kZh2);
        tc::fence_smem_to_async();
        tc::fence_before_sync();
        if (__syncthreads_or(failed)) break;
        if (tid == 0) {
            train_issue<kGHid, kGOutPad>(T, za, kZK, kZh2, wa + 2 * kGImgW3);
            tc::commit(&S.bar_mma);
        }
        wait(&S.bar_mma, ph);
        tc::fence_before_sync();
        if (__syncthreads_or(failed)) break;
        tc::fence_after_sync();
        {   // loss and dLoss/dOutput of this thread's record (times n)
            float o[kGOutPad];
#pragma unroll
            for (int c0 = 0; c0 < kGOutPad; c0 += 16) tc::ld_32x32b_x16(tl + c0, o + c0);
#pragma unroll
            for (int j = 0; j < kGOut; j++) o[j] += S.bias[kGImgB3 + j];
            float dd[kGOut];
            lacc += record_grad(o, rec, sc, dd);
#pragma unroll
            for (int c = 0; c < kGOutPad; c += 8) {
                uint32_t p[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int k = c + 2 * j;
                    p[j] = pack_h2_sat(k < kGOut ? dd[k] : 0.f, k + 1 < kGOut ? dd[k + 1] : 0.f);
                }
                *reinterpret_cast<uint4*>(S.d + canon_index(tid, kDd0 + c, kDK)) = make_uint4(p[0], p[1], p[2], p[3]);
            }
        }
        tc::fence_smem_to_async();
        tc::fence_before_sync();
        if (__syncthreads_or(failed)) break;
        // backward through layer 3, then layer 2
        if (tid == 0) {
            train_issue<kGOutPad, kGHid>(T, da, kDK, kDd0, wa + kGImgW3T);
            tc::commit(&S.bar_mma);
        }
        wait(&S.bar_mma, ph);
        train_backward_epilogue(S, tl, m2, kDd2);
        tc::fence_smem_to_async();
        tc::fence_before_sync();
        if (__syncthreads_or(failed)) break;
        if (tid == 0) {
            train_issue<kGHid, kGHid>(T, da, kDK, kDd2, wa + kGImgW2T);
            tc::commit(&S.bar_mma);
        }
        wait(&S.bar_mma, ph);
        train_backward_epilogue(S, tl, m1, kDd1);
        tc::fence_smem_to_async();
        tc::fence_before_sync();
        if (__syncthreads_or(failed)) break;
        // weight and bias gradients over the tile's 128 records (MN-major
        // operands, 16 records per instruction), accumulated across tiles
        if (tid == 0) {
            tc::fence_after_sync();
            constexpr uint32_t id12 = tc::idesc_f16_f32(kTcRows, 224, true, true);
            constexpr uint32_t id3 = tc::idesc_f16_f32(kTcRows, 80, true, true);
#pragma unroll
            for (int ks = 0; ks < kTcRows / 16; ks++) {
                const uint32_t acc = first && ks == 0 ? 0u : 1u;
                tc::mma_f16(T + kAccW12, tc::smem_desc(da + (kDd1 / 8) * 128 + ks * 2 * kDK * 16, kDK * 16, 128),
                            tc::smem_desc(za + ks * 2 * kZK * 16, kZK * 16, 128), id12, acc);
                tc::mma_f16(T + kAccW3, tc::smem_desc(da + ks * 2 * kDK * 16, kDK * 16, 128),
                            tc::smem_desc(za + (kZones / 8) * 128 + ks * 2 * kZK * 16, kZK * 16, 128), id3, acc);
            }
            tc::commit(&S.bar_g);
        }
        pending = true;
        first = false;
    }
    if (pending) wait(&S.bar_g, phg);
    tc::fence_before_sync();
    const bool bad = __syncthreads_or(failed) != 0;
    tc::fence_after_sync();
    if (!bad && !first) {
        // accumulator lane m: rows 0..63 = units of layer 1 (dW1, b1), 64..127
        // = units of layer 2 (dW2, b2); of the second product rows 0..39 =
        // the outputs (b3 in column 0, dW3 in columns 16..79)
        const int m = tid;
        float v[16];
        if (warp < 2) {
            for (int c0 = 0; c0 < kGEnc; c0 += 16) {
                tc::ld_32x32b_x16(tl + kAccW12 + c0, v);
#pragma unroll
                for (int j = 0; j < 16; j++) atomicAdd(grad + kGW1 + m * kGEnc + c0 + j, v[j] * inv_n);
            }
        } else {
            for (int c0 = 0; c0 < kGHid; c0 += 16) {
                tc::ld_32x32b_x16(tl + kAccW12 + kZh1 + c0, v);
#pragma unroll
                for (int j = 0; j < 16; j++) atomicAdd(grad + kGW2 + (m - kGHid) * kGHid + c0 + j, v[j] * inv_n);
            }
        }
        tc::ld_32x32b_x16(tl + kAccW12 + kZones, v);
        atomicAdd(grad + (warp < 2 ? kGB1 + m : kGB2 + m - kGHid), v[0] * inv_n);
        for (int c0 = 0; c0 < 80; c0 += 16) {
            tc::ld_32x32b_x16(tl + kAccW3 + c0, v);
            if (m < kGOut) {
                if (c0 == 0) {
                    atomicAdd(grad + kGB3 + m, v[0] * inv_n);
                } else {
#pragma unroll
                    for (int j = 0; j < 16; j++) atomicAdd(grad + kGW3 + m * kGHid + c0 - 16 + j, v[j] * inv_n);
                }
            }
        }
    }
    for (int o = 16; o; o >>= 1) lacc += __shfl_xor_sync(0xffffffffu, lacc, o);
    if ((tid & 31) == 0) atomicAdd(loss, lacc * inv_n);
    tc::fence_before_sync();
    __syncthreads();
    if (S.fail) {
        (void)tc::mbar_wait(&S.bar_w, 0, kTcWaitNs);
        (void)tc::mbar_wait(&S.bar_mma, ph, kTcWaitNs);
        (void)tc::mbar_wait(&S.bar_g, phg, kTcWaitNs);
    }
    if (tid < 32) {
        tc::fence_after_sync();
        tc::tmem_dealloc(T, kTrainCols);
    }
}

// Adam on the fp32 master copy; refreshes the fp16 copy and clears the
// gradient.  The padding rows of layer 3 stay zero.
__global__ void k_guide_adam(float* w32, __half* w16, unsigned char* image, float* grad, float* m, float* v, float lr,
                             float b1, float b2, float c1, float c2, float eps) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kGParams; i += gridDim.x * blockDim.x) {
        const bool pad = (i >= kGW3 + kGOut * kGHid && i < kGB3) || i >= kGB3 + kGOut;
        if (!pad) {
            float g = grad[i];
            float mi = b1 * m[i] + (1.f - b1) * g;
            float vi = b2 * v[i] + (1.f - b2) * g * g;
            m[i] = mi;
            v[i] = vi;
            w32[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        } else {
            w32[i] = 0.f;
        }
        w16[i] = __float2half_rn(w32[i]);
        write_image(image, i, w32[i]);
        grad[i] = 0.f;
    }
}

__global__ void k_guide_to_half(const float* w32, __half* w16, unsigned char* image) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kGParams; i += gridDim.x * blockDim.x) {
        w16[i] = __float2half_rn(w32[i]);
        write_image(image, i, w32[i]);
    }
}

// ------------------------------------------------------------------ host
namespace {

// Deterministic initial weights: uniform(-b, b) with b = sqrt(6 / fan_in)
// for the ReLU layers (He), 0.1 * sqrt(3 / fan_in) for the output layer;
// biases 0 except log kappa = 1 (broad lobes at first).
void init_params(uint64_t seed, std::vector<float>& w) {
    w.assign(kGParams, 0.f);
    uint64_t st = splitmix64(seed ^ 0x6a09e667f3bcc909ULL);
    auto uni = [&]() {
        st = splitmix64(st);
        return (float)((st >> 40) * (1.0 / 16777216.0)) * 2.f - 1.f;
    };
    const float b1 = std::sqrt(6.f / kGEnc), b2 = std::sqrt(6.f / kGHid), b3 = 0.1f * std::sqrt(3.f / kGHid);
    for (int i = 0; i < kGHid * kGEnc; i++) w[kGW1 + i] = b1 * uni();
    for (int i = 0; i < kGHid * kGHid; i++) w[kGW2 + i] = b2 * uni();
    for (int r = 0; r < kGOut; r++)
        for (int c = 0; c < kGHid; c++) w[kGW3 + r * kGHid + c] = b3 * uni();
    for (int j = 0; j < kGLobes; j++) {
        // spread the initial mean directions over the sphere
        float z = 1.f - 2.f * (j + 0.5f) / kGLobes, r = std::sqrt(std::max(0.f, 1.f - z * z));
        float ph = 2.399963f * j;
        w[kGB3 + 5 * j] = r * std::cos(ph);
        w[kGB3 + 5 * j + 1] = r * std::sin(ph);
        w[kGB3 + 5 * j + 2] = z;
        w[kGB3 + 5 * j + 3] = 1.f;
    }
}

}  // namespace

void guide_init_params(uint64_t seed, std::vector<float>& w) { init_params(seed, w); }

void guide_upload_params(dl_guide* G, const float* host) {
    cudaStream_t st = G->ctx->stream;
    DL_CUDA(cudaMemcpyAsync(G->w32.ptr, host, kGParams * 4, cudaMemcpyHostToDevice, st));
    k_guide_to_half<<<64, 256, 0, st>>>(G->w32.as<float>(), G->w16.as<__half>(), G->image.as<unsigned char>());
    DL_CUDA(cudaGetLastError());
}

// Gradient of the loss over `n` device records (every `stride`-th) added to
// G->grad; the loss sum lands in scratch[1].
void guide_gradient(dl_guide* G, const void* d_recs, int64_t n, int stride, cudaStream_t st) {
    static const bool setup = [] {
        DL_CUDA(cudaFuncSetAttribute(k_guide_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sizeof(GuideTrainSmem)));
        return true;
    }();
    (void)setup;
    float* sc = G->scratch.as<float>();
    unsigned* err = reinterpret_cast<unsigned*>(G->scratch.as<char>() + kGuideErrOffset);
    DL_CUDA(cudaMemsetAsync(sc, 0, 2 * sizeof(float), st));
    const GuideRecord* R = static_cast<const GuideRecord*>(d_recs);
    k_guide_weight_sum<<<(int)std::min<int64_t>(1024, (n + 255) / 256), 256, 0, st>>>(R, (int)n, stride, sc);
    const int64_t ntiles = (n + kTcRows - 1) / kTcRows;
    const int blocks = (int)std::min<int64_t>(ntiles, G->ctx->num_sms);
    k_guide_train_tc<<<blocks, kTcRows, sizeof(GuideTrainSmem), st>>>(G->image.ptr, R, (int)n, stride, sc,
                                                                       G->grad.as<float>(), sc + 1, err);
    DL_CUDA(cudaGetLastError());
}

void guide_adam(dl_guide* G, cudaStream_t st) {
    G->step += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)G->step), c2 = 1.f - std::pow(b2, (float)G->step);
    k_guide_adam<<<64, 256, 0, st>>>(G->w32.as<float>(), G->w16.as<__half>(), G->image.as<unsigned char>(),
                                     G->grad.as<float>(),
                                     G->m.as<float>(), G->v.as<float>(), G->cfg.learning_rate, b1, b2, c1, c2,
                                     1e-8f);
    DL_CUDA(cudaGetLastError());
}

// Train on `n` device records: `steps` Adam steps over the same batch.
float guide_train(dl_guide* G, const void* d_recs, int64_t n, int steps) {
    cudaStream_t st = G->ctx->stream;
    float loss = 0.f;
    for (int k = 0; k < steps; k++) {
        guide_gradient(G, d_recs, n, 1, st);
        guide_adam(G, st);
    }
    if (steps > 0) {
        DL_CUDA(cudaMemcpyAsync(&loss, G->scratch.as<float>() + 1, 4, cudaMemcpyDeviceToHost, st));
        DL_CUDA(cudaStreamSynchronize(st));
    }
    return loss;
}

// Blocks of k_guide_infer resident at once on one SM, from its registers and
// shared memory; the first call raises the kernel's shared-memory limit.
static int infer_blocks_per_sm() {
    DL_CUDA(cudaFuncSetAttribute(k_guide_infer, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(GuideTcSmem)));
    DL_CUDA(cudaFuncSetAttribute(k_guide_infer, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    int dev = 0;
    DL_CUDA(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    DL_CUDA(cudaGetDeviceProperties(&prop, dev));
    cudaFuncAttributes fa;
    DL_CUDA(cudaFuncGetAttributes(&fa, k_guide_infer));
    const int regs_per_warp = ((fa.numRegs + 7) / 8) * 8 * 32;
    const int by_regs = prop.regsPerMultiprocessor / std::max(1, regs_per_warp * (kTcThreads / 32));
    const size_t smem = sizeof(GuideTcSmem) + fa.sharedSizeBytes + prop.reservedSharedMemPerBlock;
    return std::max(1, std::min(by_regs, (int)(prop.sharedMemPerMultiprocessor / smem)));
}

void guide_forward(dl_guide* G, const float* d_in, float* d_out, int64_t n) {
    static const int per_sm = infer_blocks_per_sm();
    cudaStream_t st = G->ctx->stream;
    unsigned* err = reinterpret_cast<unsigned*>(G->scratch.as<char>() + kGuideErrOffset);
    DL_CUDA(cudaMemsetAsync(err, 0, sizeof(unsigned), st));
    const int64_t ntiles = (n + kTcRows - 1) / kTcRows;
    const int blocks = (int)std::min<int64_t>((ntiles + kTcGroups - 1) / kTcGroups, (int64_t)G->ctx->num_sms * per_sm);
    k_guide_infer<<<blocks, kTcThreads, sizeof(GuideTcSmem), st>>>(G->image.ptr, d_in, d_out, (int)n, err);
    DL_CUDA(cudaGetLastError());
}

}  // namespace dl
