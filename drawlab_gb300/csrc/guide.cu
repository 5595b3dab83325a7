// Training and inference of the learned path-guiding proposal (guide.cuh)
// on the fifth-generation tensor cores, and the dl_guide C ABI.
//
// One training step on a batch of n records {position, normal, sampled
// direction w, its sampling pdf p, radiance estimate L along w}:
//   loss = -(1/n) sum_i min((L_i / p_i) / mean(L / p), 20) * log q(w_i)
// (an estimate of the KL divergence from the normalised incident radiance to
// the mixture q, up to a constant), then one Adam update.  Kernels:
//   k_guide_weight_sum   mean(L / p) over the batch
//   k_guide_train        forward, loss gradient, backward and the weight
//                        and bias gradients per 128-record tile (tcgen05.mma),
//                        activations kept in shared memory, gradient sums in
//                        tensor memory; one partial gradient per block
//   k_guide_grad_reduce  the blocks' partial gradients summed
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
// the tensor cores; each of a block's five warpgroups walks its own tiles
// (one block per SM: five tiles' chains of dependent layers overlap, one
// weight copy in shared memory).
constexpr int kInferGroups = 5;
using InferSmem = GuideTcSmemT<kInferGroups>;
constexpr int kInferThreads = kTcRows * kInferGroups;
static_assert(sizeof(InferSmem) + 1024 <= 227 * 1024, "one inference block per SM");

__global__ void __launch_bounds__(kInferThreads, 1) k_guide_infer(const void* image, const float* in, float* out,
                                                                   int n, unsigned* err) {
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    InferSmem& S = *reinterpret_cast<InferSmem*>(dyn_smem);
    const int ntiles = (n + kTcRows - 1) / kTcRows;
    if ((int)blockIdx.x * kInferGroups >= ntiles) return;
    const int g = tc_group(), row = tc_row();
    uint32_t phase = 0;
    bool ok = guide_tc_begin(S, image, err);
    for (int tile = blockIdx.x * kInferGroups + g; ok && tile < ntiles; tile += gridDim.x * kInferGroups) {
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

// Per block of 256 threads, the sum of L / p over its records into
// part[blockIdx.x] (the training kernel adds the blocks' sums); block 0
// also clears the batch's loss accumulator.
constexpr int kWsumThreads = 256, kWsumMaxBlocks = 1024;
__global__ void __launch_bounds__(kWsumThreads) k_guide_weight_sum(const GuideRecord* s, int n, int stride,
                                                                    float* part, float* loss) {
    tc::pdl_launch_dependents();
    __shared__ float s_w[kWsumThreads / 32];
    float acc = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const GuideRecord& r = s[(size_t)i * stride];
        acc += r.pdf > 0.f ? r.L / r.pdf : 0.f;
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int k = 0; k < kWsumThreads / 32; k++) t += s_w[k];
        part[blockIdx.x] = t;
        if (blockIdx.x == 0) *loss = 0.f;
    }
}

// Half of the loss gradient of one record, computed by two threads: this
// one takes lobes 4h .. 4h + 3, from their 20 outputs o[0..19] (bias
// added).  The lobes are decoded as decode_lobes does and the mixture's pdf
// taken as vmf_pdf (guide.cuh), here with the hardware's fast exponential,
// logarithm and division -- this runs once per record and training step,
// latency-bound, and the gradients stay within the oracle's 1e-2 -- where
// the renderer's sampling keeps the accurate forms.  The mixture's
// normalisation needs both halves: each thread publishes, in `mine`, its
// largest logit, its sum of exp(logit - that) and the same sum weighted by
// the lobes' pdfs, and reads the other half's from `other` after a barrier
// of the whole block (every thread of the block calls this together; both
// halves then hold the same sums, added in the same order).  Writes the 20
// gradients, times `scale`, to d; returns the record's loss, -scale log q.
__device__ __forceinline__ float record_grad_half(const float* o, float3 w, float scale, float4* mine,
                                                  const float4* other, float* d) {
    constexpr int kH = kGLobes / 2;
    float mx = -1e30f;
#pragma unroll
    for (int j = 0; j < kH; j++) mx = fmaxf(mx, o[5 * j + 4]);
    float3 mu[kH];
    float kap[kH], e[kH], inv_len[kH], pdf[kH], dt[kH], e2[kH], ia[kH];
    bool clamped[kH];
    float se = 0.f, sq = 0.f;
#pragma unroll
    for (int j = 0; j < kH; j++) {
        const float3 m = f3(o[5 * j], o[5 * j + 1], o[5 * j + 2]);
        const float len2 = m.x * m.x + m.y * m.y + m.z * m.z;
        if (len2 > 1e-12f) {
            inv_len[j] = rsqrtf(len2);
            mu[j] = f3(m.x * inv_len[j], m.y * inv_len[j], m.z * inv_len[j]);
        } else {
            inv_len[j] = 0.f;
            mu[j] = f3(0.f, 0.f, 1.f);
        }
        const float lk = o[5 * j + 3];
        clamped[j] = lk < kGLogKappaMin || lk > kGLogKappaMax;
        const float k = __expf(fminf(fmaxf(lk, kGLogKappaMin), kGLogKappaMax));
        kap[j] = k;
        e[j] = __expf(o[5 * j + 4] - mx);
        dt[j] = mu[j].x * w.x + mu[j].y * w.y + mu[j].z * w.z;
        // e^{-2k} and 1 / (1 - e^{-2k}), shared by the pdf and its kappa derivative
        e2[j] = __expf(-2.f * k);
        ia[j] = __fdividef(1.f, 1.f - e2[j]);
        pdf[j] = k < 1e-4f ? 0.25f * kInvPiF : k * ia[j] * (0.5f * kInvPiF) * __expf(k * (dt[j] - 1.f));
        se += e[j];
        sq += e[j] * pdf[j];
    }
    *mine = make_float4(mx, se, sq, 0.f);
    __syncthreads();
    const float4 x = *other;
    const float M = fmaxf(mx, x.x);
    const float am = __expf(mx - M), ao = __expf(x.x - M);
    const float lsum = se * am + x.y * ao;   // sum of exp(logit - M) over the 8 lobes
    const float inv_sum = __fdividef(1.f, lsum);
    const float q = (sq * am + x.z * ao) * inv_sum;
#pragma unroll
    for (int j = 0; j < 5 * kH; j++) d[j] = 0.f;
    if (!(q > 1e-30f) || !(scale > 0.f) || !isfinite(scale)) return 0.f;
    const float inv_q = __fdividef(1.f, q);
#pragma unroll
    for (int j = 0; j < kH; j++) {
        const float lam = e[j] * am * inv_sum, k = kap[j];
        const float r = lam * pdf[j] * inv_q;
        // d(-log q)/d(logit_j) = -(r_j - lambda_j)
        d[5 * j + 4] = -scale * (r - lam);
        // d(-log q)/d(log kappa_j) = -r_j (1 - 2k / (e^{2k} - 1) + k (mu.w - 1)),
        // 2k / (e^{2k} - 1) = 2k e^{-2k} / (1 - e^{-2k})
        if (!clamped[j]) {
            const float t = k < 1e-4f ? 0.f : 1.f - 2.f * k * e2[j] * ia[j] + k * (dt[j] - 1.f);
            d[5 * j + 3] = -scale * r * t;
        }
        // d(-log q)/dm_j = -r_j kappa_j (w - (mu.w) mu) / |m_j|
        const float f = -scale * r * k * inv_len[j];
        d[5 * j + 0] = f * (w.x - dt[j] * mu[j].x);
        d[5 * j + 1] = f * (w.y - dt[j] * mu[j].y);
        d[5 * j + 2] = f * (w.z - dt[j] * mu[j].z);
    }
    return -scale * __logf(q);
}

// One training batch on the tensor cores, in three kernels:
//
//   k_guide_weight_sum  per-block sums of the records' L / pdf (the loss's
//                    target normalisation).
//   k_guide_train    one block per SM, two warpgroups (256 threads), over a
//                    range of 128-record tiles, one tile at a time.  Per tile,
//                    every product a tcgen05.mma issued by thread 0 with both
//                    operands in shared memory and the fp32 accumulator in
//                    tensor memory:
//                      forward  x -> h1 -> h2 -> outputs (3 products);
//                      the loss and dLoss/dOutput of each record (d0, fp16);
//                      backward d2 = (d0 W3) * [h2 > 0], d1 = (d2 W2) *
//                               [h1 > 0] (B operands W3^T, W2^T from the
//                               weight image);
//                      the tile's share of the weight and bias gradients,
//                               accumulated in tensor memory over the
//                               block's tiles (K = the tile's records), in
//                               two products: [d2 | d0]^T [h1 | 1 | h2]
//                               (dW2, b2, b3, dW3), issued as soon as d2
//                               exists, and [d1 | .]^T [x | 1] (dW1, b1).
//                    The activations stay in shared memory in the canonical
//                    layout, which the forward and backward products read as
//                    K-major operands and the weight-gradient products as
//                    MN-major ones (M or N = features, K = records).  The two
//                    warpgroups split each epilogue's 64 accumulator columns
//                    and each record's loss (four lobes each); while a
//                    product runs, each thread encodes one of its three
//                    inputs of the next tile into the second x buffer; the
//                    tile's weight-gradient products run while the backward
//                    epilogues and the next tile's first product go on.  At
//                    the end each block writes its gradient sums from tensor
//                    memory to global memory, feature-major (coalesced
//                    stores; layout below).
//   k_guide_grad_reduce  sums the blocks' partials in a fixed order (no
//                    atomics) into the gradient, in the parameter layout,
//                    applying the loss's 1/n.
//
// Loss scaling: the fp16 activation gradients leave out the loss's 1/n
// (with n ~ 1e5 records most of them would be fp16 subnormals); they
// saturate at the fp16 range, and the 1/n is applied, in fp32, in the
// reduction.
constexpr int kTrThreads = 2 * kTcRows;                // two warpgroups
// operand matrices in shared memory (halves per record, feature offsets)
constexpr int kXK = kGEnc + 16, kXones = kGEnc;        // X = [x | 1]
constexpr int kHK = 144, kHh1 = 0, kHones = 64, kHh2 = 80;  // H = [h1 | 1 | h2]
constexpr int kDK = 192, kDd1 = 0, kDd2 = 64, kDd0 = 128;   // D = [d1 | d2 | d0 | 0]
// tensor memory: the gradient sums (columns 0..303) and the forward /
// backward accumulator (64 columns, reused by every product)
constexpr int kTrCols = 512;
constexpr int kAccA = 0, kAccB = kXK, kAccF = 384;
static_assert(kAccB + kHK <= kAccF && kAccF + kGHid <= kTrCols, "tensor-memory columns");
constexpr float kHalfMax = 65504.f;
// A block's gradient sums in global memory, feature-major so that a warp's
// 32 units (accumulator lanes) of one feature are 32 consecutive floats:
// dW1 as [feature][unit], b1, dW2 as [feature][unit], b2, dW3 as
// [feature][output] (40 outputs), b3.
constexpr int kPW1 = 0, kPB1 = kPW1 + kGEnc * kGHid, kPW2 = kPB1 + kGHid, kPB2 = kPW2 + kGHid * kGHid;
constexpr int kPW3 = kPB2 + kGHid, kPB3 = kPW3 + kGHid * kGOut, kPSums = kPB3 + kGOut;   // 16040 floats

// The parameter (guide.cuh layout) that slot t of a block's sums holds.
__host__ __device__ constexpr int guide_sum_param(int t) {
    return t < kPB1   ? kGW1 + (t - kPW1) % kGHid * kGEnc + (t - kPW1) / kGHid
           : t < kPW2 ? kGB1 + t - kPB1
           : t < kPB2 ? kGW2 + (t - kPW2) % kGHid * kGHid + (t - kPW2) / kGHid
           : t < kPW3 ? kGB2 + t - kPB2
           : t < kPB3 ? kGW3 + (t - kPW3) % kGOut * kGHid + (t - kPW3) / kGOut
                      : kGB3 + t - kPB3;
}
static_assert(guide_sum_param(kPSums - 1) == kGB3 + kGOut - 1 && guide_sum_param(kPB3 - 1) == kGW3 + (kGOut - 1) * kGHid + kGHid - 1,
              "sum layout");

struct GuideTrSmem {
    __half w[kGImgHalves];                    // the weight image: weights, biases,
    float bias[kGImgBiases];                  // W2^T and W3^T
    __half w2t[kGHid * kGHid];
    __half w3t[kGHid * kGOutPad];
    alignas(128) __half x[2][kTcRows * kXK];  // this tile's X and the next tile's
    alignas(128) __half h[kTcRows * kHK];
    alignas(128) __half d[kTcRows * kDK];
    float4 ex[2][kTcRows];                    // the two halves' mixture sums of each record
    uint64_t bar_w, bar_mma;
    uint32_t tmem;
    float mean;
    int fail;
};
static_assert(offsetof(GuideTrSmem, w2t) == kGImgW2T && offsetof(GuideTrSmem, w3t) == kGImgW3T, "image layout");
static_assert(sizeof(GuideTrSmem) + 1024 <= 227 * 1024, "one training block per SM");
// no other tensor-memory user of this library (the guided material blocks,
// 107 KB; the inference block, 218 KB) fits beside a block: its 512 columns
// are free
static_assert(sizeof(GuideTrSmem) + 1024 + 107 * 1024 > 228 * 1024, "one tensor-memory user per SM");

__device__ __forceinline__ uint32_t pack_h2(float a, float b) {
    __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}
__device__ __forceinline__ uint32_t pack_h2_sat(float a, float b) {
    return pack_h2(fminf(fmaxf(a, -kHalfMax), kHalfMax), fminf(fmaxf(b, -kHalfMax), kHalfMax));
}

// Input i of a record, encoded into features 24 i .. 24 i + 23 of row r of X.
__device__ __forceinline__ void tr_encode(float v, __half* x, int r, int i) {
    __half2 h[kGFreq];
    encode_scalar_h2(v, h);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        uint4 q;
        q.x = *reinterpret_cast<const uint32_t*>(&h[4 * c]);
        q.y = *reinterpret_cast<const uint32_t*>(&h[4 * c + 1]);
        q.z = *reinterpret_cast<const uint32_t*>(&h[4 * c + 2]);
        q.w = *reinterpret_cast<const uint32_t*>(&h[4 * c + 3]);
        *reinterpret_cast<uint4*>(x + canon_index(r, i * 2 * kGFreq + 8 * c, kXK)) = q;
    }
}

// Bias + ReLU of the 32 accumulator columns c0 .. c0 + 31 (at t, the warp's
// lanes) into H at feature hf + c0; returns the mask of the outputs that are
// > 0 after rounding (bit j: column c0 + j).
__device__ __forceinline__ uint32_t tr_hidden_epilogue(uint32_t t, int c0, const float* bias, __half* H, int hf) {
    const int r = threadIdx.x & (kTcRows - 1);
    float v[32];
    tc::ld_32x32b_x32(t + c0, v);
    uint32_t mask = 0, p[16];
#pragma unroll
    for (int j = 0; j < 16; j++) {
        __half2 h = __floats2half2_rn(fmaxf(v[2 * j] + bias[c0 + 2 * j], 0.f),
                                      fmaxf(v[2 * j + 1] + bias[c0 + 2 * j + 1], 0.f));
        if (__low2float(h) > 0.f) mask |= 1u << (2 * j);
        if (__high2float(h) > 0.f) mask |= 1u << (2 * j + 1);
        p[j] = *reinterpret_cast<const uint32_t*>(&h);
    }
#pragma unroll
    for (int q = 0; q < 4; q++)
        *reinterpret_cast<uint4*>(H + canon_index(r, hf + c0 + 8 * q, kHK)) =
            make_uint4(p[4 * q], p[4 * q + 1], p[4 * q + 2], p[4 * q + 3]);
    return mask;
}

// The 32 accumulator columns c0 .. c0 + 31, masked by `mask`, into D at
// feature df + c0 (fp16, saturated).
__device__ __forceinline__ void tr_backward_epilogue(uint32_t t, int c0, uint32_t mask, __half* D, int df) {
    const int r = threadIdx.x & (kTcRows - 1);
    float v[32];
    tc::ld_32x32b_x32(t + c0, v);
    uint32_t p[16];
#pragma unroll
    for (int j = 0; j < 16; j++)
        p[j] = pack_h2_sat((mask >> (2 * j)) & 1u ? v[2 * j] : 0.f, (mask >> (2 * j + 1)) & 1u ? v[2 * j + 1] : 0.f);
#pragma unroll
    for (int q = 0; q < 4; q++)
        *reinterpret_cast<uint4*>(D + canon_index(r, df + c0 + 8 * q, kDK)) =
            make_uint4(p[4 * q], p[4 * q + 1], p[4 * q + 2], p[4 * q + 3]);
}

// acc (128 x N) = A x W^T: A = K features of the tile's rows, starting at
// byte address a in a matrix with rows of `arow` halves (K-major); W [N][K]
// at w (rows of K halves).  Completion on `bar`.
template <int K, int N>
__device__ __forceinline__ void tr_issue(uint32_t acc, uint32_t a, int arow, uint32_t w, uint64_t* bar) {
    constexpr uint32_t idesc = tc::idesc_f16_f32(kTcRows, N);
    tc::fence_after_sync();
#pragma unroll
    for (int ks = 0; ks < K / 16; ks++)
        tc::mma_f16(acc, tc::smem_desc(a + ks * 256, 128, arow * 16), tc::smem_desc(w + ks * 256, 128, K * 16), idesc,
                    ks > 0 ? 1u : 0u);
    tc::commit(bar);
}

// Gradient sums (acc, N columns) += A^T B over the tile's 128 records, 16
// per instruction (the block's first tile initialises them): A = 128
// features of D from feature af, B = N features of a matrix of `brow`
// halves per record at b, both MN-major.  No completion signal of its own:
// the next product's commit covers it.
template <int N>
__device__ __forceinline__ void tr_issue_grad(uint32_t acc, uint32_t da, int af, uint32_t b, int brow, bool first) {
    constexpr uint32_t idesc = tc::idesc_f16_f32(kTcRows, N, true, true);
#pragma unroll
    for (int ks = 0; ks < kTcRows / 16; ks++)
        tc::mma_f16(acc, tc::smem_desc(da + (af / 8) * 128 + ks * 2 * kDK * 16, kDK * 16, 128),
                    tc::smem_desc(b + ks * 2 * brow * 16, brow * 16, 128), idesc, first && ks == 0 ? 0u : 1u);
}

__global__ void __launch_bounds__(kTrThreads, 1) k_guide_train(const void* image, const GuideRecord* s, int n,
                                                                int stride, const float* wsum, int nwsum,
                                                                float* partial, float* loss, unsigned* err) {
    extern __shared__ __align__(128) unsigned char dyn_smem[];
    GuideTrSmem& S = *reinterpret_cast<GuideTrSmem*>(dyn_smem);
    const int tid = threadIdx.x, g = tid >> 7, r = tid & (kTcRows - 1);
    const int ntiles = (n + kTcRows - 1) / kTcRows;
    if (tid == 0) {
        tc::mbar_init(&S.bar_w, 1);
        tc::mbar_init(&S.bar_mma, 1);
        S.fail = 0;
    }
    if (tid < 32) tc::tmem_alloc(&S.tmem, kTrCols);
    tc::pdl_launch_dependents();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // the weight copy lands while the first tile's records load and encode
    if (tid == 0) tc::bulk_load(S.w, image, kGImgTrainBytes, &S.bar_w);
    {   // the constant columns, the same for every tile: ones of X (both
        // buffers) and H, zeros of D after d0's 40 outputs
        const uint32_t one2 = pack_h2(1.f, 1.f);
        const uint4 ones = make_uint4(one2, one2, one2, one2), zeros = make_uint4(0u, 0u, 0u, 0u);
        for (int c = 0; c < 16; c += 8) {
            *reinterpret_cast<uint4*>(S.x[g] + canon_index(r, kXones + c, kXK)) = ones;
            if (g == 0) *reinterpret_cast<uint4*>(S.h + canon_index(r, kHones + c, kHK)) = ones;
        }
        for (int c = kDd0 + kGOut + 8 * g; c < kDK; c += 16)
            *reinterpret_cast<uint4*>(S.d + canon_index(r, c, kDK)) = zeros;
    }
    bool failed = false;
    uint32_t ph = 0;
    auto wait = [&]() {
        if (!tc::mbar_wait(&S.bar_mma, ph, kTcWaitNs)) {
            failed = true;
            S.fail = 1;
            atomicOr(err, kErrTensorWait);
        } else {
            ph ^= 1u;
        }
        tc::fence_after_sync();
    };
    // all threads done with the step's shared and tensor memory: returns
    // true (in every thread) when a wait has failed
    auto step_sync = [&]() {
        tc::fence_smem_to_async();
        tc::fence_before_sync();
        return __syncthreads_or(failed) != 0;
    };
    const uint32_t T = S.tmem;
    const uint32_t tf = T + kAccF + ((uint32_t)(tid & 96) << 16);   // forward accumulator, this warp's lanes
    const int ch = 32 * g;                                          // this warpgroup's epilogue columns
    const uint32_t xa0 = tc::smem_addr(S.x[0]), ha = tc::smem_addr(S.h), da = tc::smem_addr(S.d);
    const uint32_t wa = tc::smem_addr(S.w);
    constexpr uint32_t kXBytes = kTcRows * kXK * 2;
    float lacc = 0.f;
    bool any = false;
    // a record as three float4: in[0..3] | in[4], in[5], w[0], w[1] | w[2], pdf, L, pad
    auto load_rec = [&](int row, float4* q) {
        if (row < n) {
            const float4* p = reinterpret_cast<const float4*>(s + (size_t)row * stride);
            q[0] = p[0];
            q[1] = p[1];
            q[2] = p[2];
        } else {
            q[0] = q[1] = q[2] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    };
    // input 3g + i of a record
    auto input = [&](const float4* q, int i) {
        const int j = 3 * g + i;
        return j == 0 ? q[0].x : j == 1 ? q[0].y : j == 2 ? q[0].z : j == 3 ? q[0].w : j == 4 ? q[1].x : q[1].y;
    };
    float4 cur[3], nxt[3];
    int k = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, k++) {
        const int row = tile * kTcRows + r;
        const int b = k & 1;
        const bool more = tile + (int)gridDim.x < ntiles;
        if (k == 0) {
            // the first tile's encoding: inputs 3g .. 3g + 2 of each record
            load_rec(row, cur);
#pragma unroll
            for (int i = 0; i < 3; i++) tr_encode(input(cur, i), S.x[0], r, 3 * g + i);
            if (!tc::mbar_wait(&S.bar_w, 0, kTcWaitNs)) {
                failed = true;
                S.fail = 1;
                atomicOr(err, kErrTensorWait);
            }
            if (step_sync()) break;
        }
        // (later tiles: their X was complete at the previous tile's last barrier)
        // the next tile's records arrive while this tile's first products run
        if (more) load_rec((tile + (int)gridDim.x) * kTcRows + r, nxt);
        const uint32_t xa = xa0 + b * kXBytes;
        // layer 1: x -> h1 (after the previous tile's gradient products,
        // which read H and D: the commit covers them)
        if (tid == 0) tr_issue<kGEnc, kGHid>(T + kAccF, xa, kXK, wa + 2 * kGImgW1, &S.bar_mma);
        if (k == 0) {
            tc::pdl_wait();   // k_guide_weight_sum has finished
            if (tid < 32) {   // the batch's mean weight, summed the same way in every block
                float sum = 0.f;
                for (int j = tid; j < nwsum; j += 32) sum += wsum[j];
                for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
                if (tid == 0) S.mean = sum / (float)n;
            }
        }
        wait();
        const uint32_t m1 = tr_hidden_epilogue(tf, ch, S.bias + kGImgB1, S.h, kHh1);
        if (step_sync()) break;
        // the record's loss weight times n (the mean is visible after the barrier)
        const float mean = S.mean;
        const float pdf = cur[2].y, Lr = cur[2].z;
        const float sc = row < n && pdf > 0.f && mean > 0.f ? fminf(Lr / pdf / mean, kGTargetClamp) : 0.f;
        // layer 2: h1 -> h2.  While a product runs, each thread encodes one
        // of its three inputs of the next tile into the other X buffer (its
        // last reader, the previous tile's gradient product, has completed)
        if (tid == 0) tr_issue<kGHid, kGHid>(T + kAccF, ha + (kHh1 / 8) * 128, kHK, wa + 2 * kGImgW2, &S.bar_mma);
        if (more) tr_encode(input(nxt, 0), S.x[b ^ 1], r, 3 * g);
        wait();
        const uint32_t m2 = tr_hidden_epilogue(tf, ch, S.bias + kGImgB2, S.h, kHh2);
        if (step_sync()) break;
        // layer 3: h2 -> outputs
        if (tid == 0) tr_issue<kGHid, kGOutPad>(T + kAccF, ha + (kHh2 / 8) * 128, kHK, wa + 2 * kGImgW3, &S.bar_mma);
        if (more) tr_encode(input(nxt, 1), S.x[b ^ 1], r, 3 * g + 1);
        wait();
        {   // loss and dLoss/dOutput (times n) of the record, lobes 4g .. 4g + 3, into D (d0 features 20g ..)
            float o[20];
            float v[32];
            tc::ld_32x32b_x32(tf + 16 * g, v);   // columns 16g .. 16g + 31 hold outputs 20g .. 20g + 19
#pragma unroll
            for (int j = 0; j < 20; j++) o[j] = (g ? v[4 + j] : v[j]) + S.bias[kGImgB3 + 20 * g + j];
            float dd[20];
            const float lr = record_grad_half(o, f3(cur[1].z, cur[1].w, cur[2].x), sc, &S.ex[g][r], &S.ex[g ^ 1][r],
                                              dd);
            if (g == 0) lacc += lr;
#pragma unroll
            for (int c = 0; c < 20; c += 4)
                *reinterpret_cast<uint2*>(S.d + canon_index(r, kDd0 + 20 * g + c, kDK)) =
                    make_uint2(pack_h2_sat(dd[c], dd[c + 1]), pack_h2_sat(dd[c + 2], dd[c + 3]));
        }
        if (step_sync()) break;
        // backward through layer 3: d0 W3 -> d2
        if (tid == 0) tr_issue<kGOutPad, kGHid>(T + kAccF, da + (kDd0 / 8) * 128, kDK, wa + kGImgW3T, &S.bar_mma);
        if (more) tr_encode(input(nxt, 2), S.x[b ^ 1], r, 3 * g + 2);
        wait();
        tr_backward_epilogue(tf, ch, m2, S.d, kDd2);
        if (step_sync()) break;
        // backward through layer 2: d2 W2 -> d1; then, behind it on the
        // tensor cores, [d2 | d0]^T [h1 | 1 | h2] (its inputs are complete
        // and nothing writes them before the next tile's first product)
        if (tid == 0) {
            tr_issue<kGHid, kGHid>(T + kAccF, da + (kDd2 / 8) * 128, kDK, wa + kGImgW2T, &S.bar_mma);
            tr_issue_grad<kHK>(T + kAccB, da, kDd2, ha, kHK, k == 0);
        }
        wait();
        tr_backward_epilogue(tf, ch, m1, S.d, kDd1);
        if (step_sync()) break;
        // [d1 | d2]^T [x | 1]; it completes before the next tile's first
        // product does (one issuing thread, products in order), which every
        // thread waits for before it writes H, D or this X buffer again
        if (tid == 0) tr_issue_grad<kXK>(T + kAccA, da, kDd1, xa, kXK, k == 0);
        any = true;
#pragma unroll
        for (int i = 0; i < 3; i++) cur[i] = nxt[i];
    }
    // every product of the block complete (after a failed wait: skipped)
    tc::fence_before_sync();
    if (__syncthreads_or(failed) == 0 && any) {
        if (tid == 0) tc::commit(&S.bar_mma);
        wait();
    }
    for (int o = 16; o; o >>= 1) lacc += __shfl_xor_sync(0xffffffffu, lacc, o);
    if (g == 0 && (tid & 31) == 0 && any) atomicAdd(loss, lacc / (float)n);
    tc::fence_before_sync();
    const bool bad = __syncthreads_or(failed) != 0;
    tc::fence_after_sync();
    // the block's gradient sums (feature-major: each store of a warp writes
    // one feature of its 32 units, 128 contiguous bytes); warps w and w + 4
    // read the same accumulator lanes and split the columns
    float* out = partial + (size_t)blockIdx.x * kPSums;
    const uint32_t tl = T + ((uint32_t)(tid & 96) << 16);
    const bool live = any && !bad;
    // ncols (16 or 32) columns from col: column j to out[dst + j * stride];
    // stride 0: a bias (its 16 columns of ones hold the same sum), column 0 only
    auto run = [&](uint32_t col, int ncols, int dst, int stride, bool keep) {
        float v[32];
        if (!live) {
#pragma unroll
            for (int j = 0; j < 32; j++) v[j] = 0.f;
        } else if (ncols == 32) {
            tc::ld_32x32b_x32(tl + col, v);
        } else {
            tc::ld_32x32b_x16(tl + col, v);
        }
        if (keep && stride == 0) out[dst] = v[0];
        if (keep && stride > 0)
            for (int j = 0; j < ncols; j++) out[dst + j * stride] = v[j];
    };
    if (r < kGHid) {   // accumulator lanes 0..63: unit r of layer 1 (first sums), of layer 2 (second sums)
        if (g == 0) {
            for (int c0 = 0; c0 < 128; c0 += 32) run(kAccA + c0, 32, kPW1 + c0 * kGHid + r, kGHid, true);
            run(kAccA + 128, 16, kPW1 + 128 * kGHid + r, kGHid, true);
            run(kAccA + kXones, 16, kPB1 + r, 0, true);
        } else {
            for (int c0 = 0; c0 < kGHid; c0 += 32) run(kAccB + kHh1 + c0, 32, kPW2 + c0 * kGHid + r, kGHid, true);
            run(kAccB + kHones, 16, kPB2 + r, 0, true);
        }
    } else {           // lanes 64..103 of the second sums: output r - 64 (b3, dW3 half by half)
        const int o = min(r - kGHid, kGOut - 1);
        const bool keep = r - kGHid < kGOut;
        if (g == 0) run(kAccB + kHones, 16, kPB3 + o, 0, keep);
        run(kAccB + kHh2 + ch, 32, kPW3 + ch * kGOut + o, kGOut, keep);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (S.fail) {
        (void)tc::mbar_wait(&S.bar_w, 0, kTcWaitNs);
        (void)tc::mbar_wait(&S.bar_mma, ph, kTcWaitNs);
    }
    if (tid < 32) {
        tc::fence_after_sync();
        tc::tmem_dealloc(T, kTrCols);
    }
}

// grad[p] = (1/n) sum over the training blocks of their gradient sums (the
// slot t that holds parameter p = guide_sum_param(t)).  A block takes 32
// consecutive slots; its 8 warps split the blocks' sums and add theirs in
// shared memory.  The padding outputs of layer 3 (rows 40..47) have no
// slots and stay as they are.
constexpr int kRedWarps = 8;
__global__ void __launch_bounds__(32 * kRedWarps) k_guide_grad_reduce(const float* partial, int nblocks, float inv_n,
                                                                        float* grad) {
    __shared__ float s_sum[kRedWarps][32];
    tc::pdl_wait();   // k_guide_train has written every block's partials
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int t = blockIdx.x * 32 + lane;
    float acc = 0.f;
    if (t < kPSums) {
#pragma unroll 4
        for (int b = w; b < nblocks; b += kRedWarps) acc += partial[(size_t)b * kPSums + t];
    }
    s_sum[w][lane] = acc;
    __syncthreads();
    if (w == 0 && t < kPSums) {
        float sum = 0.f;
#pragma unroll
        for (int k = 0; k < kRedWarps; k++) sum += s_sum[k][lane];
        grad[guide_sum_param(t)] = sum * inv_n;
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

// A launch on `st` that may begin while the previous kernel of the stream is
// still running (programmatic stream serialization); the kernel waits for
// that kernel (griddepcontrol.wait) before it reads what it wrote.
template <typename... KArgs, typename... Args>
static cudaError_t launch_dependent(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                    Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Training blocks for a batch of n records: one per SM, at most one per tile.
static int64_t train_blocks(const dl_guide* G, int64_t n) {
    const int64_t ntiles = (n + kTcRows - 1) / kTcRows;
    return std::max<int64_t>(1, std::min<int64_t>(ntiles, std::max(1, G->ctx->num_sms)));
}

// Device buffers of a training batch of up to n records: the blocks' partial
// gradients and the weight sums.  Called before any training launch,
// outside graph captures and render loops.
void guide_reserve(dl_guide* G, int64_t n) {
    G->partial.ensure((size_t)train_blocks(G, n) * kPSums * 4);
    G->wsum.ensure(kWsumMaxBlocks * sizeof(float));
}

// Gradient of the loss over `n` device records (every `stride`-th) written
// to G->grad (entries outside the network's parameters untouched); the
// loss sum lands in scratch[1].  guide_reserve(G, n) must have run.
void guide_gradient(dl_guide* G, const void* d_recs, int64_t n, int stride, cudaStream_t st) {
    static const bool setup = [] {
        DL_CUDA(cudaFuncSetAttribute(k_guide_train, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sizeof(GuideTrSmem)));
        DL_CUDA(cudaFuncSetAttribute(k_guide_train, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        return true;
    }();
    (void)setup;
    const int nb = (int)train_blocks(G, n);
    if (n < 1 || G->partial.bytes < (size_t)nb * kPSums * 4 || G->wsum.bytes < kWsumMaxBlocks * sizeof(float))
        throw Error(DL_ERR_INVALID_ARG, "guide training buffers not reserved for this batch");
    float* sc = G->scratch.as<float>();   // [1]: the loss
    unsigned* err = reinterpret_cast<unsigned*>(G->scratch.as<char>() + kGuideErrOffset);
    const GuideRecord* R = static_cast<const GuideRecord*>(d_recs);
    const int nws = (int)std::min<int64_t>(kWsumMaxBlocks, (n + kWsumThreads - 1) / kWsumThreads);
    float* wsum = G->wsum.as<float>();
    k_guide_weight_sum<<<nws, kWsumThreads, 0, st>>>(R, (int)n, stride, wsum, sc + 1);
    // the next two kernels start their prologues while their predecessor
    // runs (programmatic dependent launch); each waits for it before using
    // what it wrote
    float* part = G->partial.as<float>();
    float* grad = G->grad.as<float>();
    const void* img = G->image.ptr;
    const int ni = (int)n;
    const float inv_n = 1.f / (float)n;
    DL_CUDA(launch_dependent(k_guide_train, dim3(nb), dim3(kTrThreads), sizeof(GuideTrSmem), st, img, R, ni, stride,
                             (const float*)wsum, nws, part, sc + 1, err));
    DL_CUDA(launch_dependent(k_guide_grad_reduce, dim3((kPSums + 31) / 32), dim3(32 * kRedWarps), 0, st,
                             (const float*)part, nb, inv_n, grad));
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
    guide_reserve(G, n);
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
                                 (int)sizeof(InferSmem)));
    DL_CUDA(cudaFuncSetAttribute(k_guide_infer, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    int dev = 0;
    DL_CUDA(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    DL_CUDA(cudaGetDeviceProperties(&prop, dev));
    cudaFuncAttributes fa;
    DL_CUDA(cudaFuncGetAttributes(&fa, k_guide_infer));
    const int regs_per_warp = ((fa.numRegs + 7) / 8) * 8 * 32;
    const int by_regs = prop.regsPerMultiprocessor / std::max(1, regs_per_warp * (kInferThreads / 32));
    const size_t smem = sizeof(InferSmem) + fa.sharedSizeBytes + prop.reservedSharedMemPerBlock;
    return std::max(1, std::min(by_regs, (int)(prop.sharedMemPerMultiprocessor / smem)));
}

void guide_forward(dl_guide* G, const float* d_in, float* d_out, int64_t n) {
    static const int per_sm = infer_blocks_per_sm();
    cudaStream_t st = G->ctx->stream;
    unsigned* err = reinterpret_cast<unsigned*>(G->scratch.as<char>() + kGuideErrOffset);
    DL_CUDA(cudaMemsetAsync(err, 0, sizeof(unsigned), st));
    const int64_t ntiles = (n + kTcRows - 1) / kTcRows;
    const int blocks =
        (int)std::min<int64_t>((ntiles + kInferGroups - 1) / kInferGroups, (int64_t)G->ctx->num_sms * per_sm);
    k_guide_infer<<<blocks, kInferThreads, sizeof(InferSmem), st>>>(G->image.ptr, d_in, d_out, (int)n, err);
    DL_CUDA(cudaGetLastError());
}

}  // namespace dl
