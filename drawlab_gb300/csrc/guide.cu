// Training and inference of the learned path-guiding proposal (guide.cuh)
// on the fifth-generation tensor cores, and the dl_guide C ABI.
//
// One training step on a batch of n records {position, normal, sampled
// direction w, its sampling pdf p, radiance estimate L along w}:
//   loss = -(1/n) sum_i min((L_i / p_i) / mean(L / p), 20) * log q(w_i)
// (an estimate of the KL divergence from the normalised incident radiance to
// the mixture q, up to a constant), then one Adam update.  Kernels:
//   k_guide_weight_sum   mean(L / p) over the batch
//   k_guide_fwdbwd       forward, loss gradient and backward per 128-record
//                        tile (tcgen05.mma), activations staged in global memory
//   k_guide_wgrad        the weight and bias gradients of the whole batch as
//                        one split-K tensor-core product over the staged tiles
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

// The loss of one record and dLoss/dOutput (40 values, scaled by `scale`):
// the lobes decoded as decode_lobes does and the mixture's pdf as vmf_pdf
// (guide.cuh), here with the hardware's fast exponential, logarithm and
// division -- this runs once per record and training step, latency-bound,
// and the gradients stay within the oracle's 1e-2 -- where the renderer's
// sampling keeps the accurate forms.
__device__ __forceinline__ float record_grad(const float* o, const GuideRecord& s, float scale, float* d) {
    const float3 w = f3(s.w[0], s.w[1], s.w[2]);
    float mx = -1e30f;
#pragma unroll
    for (int j = 0; j < kGLobes; j++) mx = fmaxf(mx, o[5 * j + 4]);
    float3 mu[kGLobes];
    float kap[kGLobes], lam[kGLobes], inv_len[kGLobes], pj[kGLobes];
    bool clamped[kGLobes];
    float lsum = 0.f;
#pragma unroll
    for (int j = 0; j < kGLobes; j++) {
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
        kap[j] = __expf(fminf(fmaxf(lk, kGLogKappaMin), kGLogKappaMax));
        lam[j] = __expf(o[5 * j + 4] - mx);
        lsum += lam[j];
    }
    const float inv_sum = __fdividef(1.f, lsum);
    float q = 0.f;
#pragma unroll
    for (int j = 0; j < kGLobes; j++) {
        lam[j] *= inv_sum;
        const float k = kap[j];
        const float dot = mu[j].x * w.x + mu[j].y * w.y + mu[j].z * w.z;
        const float pdf = k < 1e-4f ? 0.25f * kInvPiF
                                    : k * __fdividef(1.f, 2.f * kPiF * (1.f - __expf(-2.f * k))) * __expf(k * (dot - 1.f));
        pj[j] = lam[j] * pdf;
        q += pj[j];
    }
    for (int j = 0; j < kGOut; j++) d[j] = 0.f;
    if (!(q > 1e-30f) || !(scale > 0.f) || !isfinite(scale)) return 0.f;
    const float inv_q = __fdividef(1.f, q);
#pragma unroll
    for (int j = 0; j < kGLobes; j++) {
        const float r = pj[j] * inv_q, k = kap[j];
        const float dot = mu[j].x * w.x + mu[j].y * w.y + mu[j].z * w.z;
        // d(-log q)/d(logit_j) = -(r_j - lambda_j)
        d[5 * j + 4] = -scale * (r - lam[j]);
        // d(-log q)/d(log kappa_j) = -r_j (1 - 2k / (e^{2k} - 1) + k (mu.w - 1))
        if (!clamped[j]) {
            const float t = k < 1e-4f ? 0.f : 1.f - __fdividef(2.f * k, __expf(2.f * k) - 1.f) + k * (dot - 1.f);
            d[5 * j + 3] = -scale * r * t;
        }
        // d(-log q)/dm_j = -r_j kappa_j (w - (mu.w) mu) / |m_j|
        const float f = -scale * r * k * inv_len[j];
        d[5 * j + 0] = f * (w.x - dot * mu[j].x);
        d[5 * j + 1] = f * (w.y - dot * mu[j].y);
        d[5 * j + 2] = f * (w.z - dot * mu[j].z);
    }
    return -scale * __logf(q);
}

// One training batch on the tensor cores, in three kernels:
//
//   k_guide_fwdbwd   per 128-record tile (one per block, two blocks per SM,
//                    so two tiles' chains of dependent products overlap):
//                    forward x -> h1 -> h2 -> outputs (3 products), the loss
//                    and dLoss/dOutput of each thread's record (d0, fp16),
//                    backward d2 = (d0 W3) * [h2 > 0] and d1 = (d2 W2) *
//                    [h1 > 0] (B operands W3^T, W2^T from the weight image).
//                    Every product is a tcgen05.mma issued by thread 0, the
//                    accumulator in tensor memory.  The activations the
//                    weight gradients need are written to global staging in
//                    the tensor cores' canonical layout, one 128-record tile
//                    after another: Z = [x | h1 | 1 | h2] (288 halves per
//                    record) and D = [d0 | d1 | d2] (176 halves).
//   k_guide_wgrad    the weight and bias gradients as one split-K product
//                    over the records: [dW1 | . | g_b1 ; . | dW2 | g_b2] =
//                    [d1 | d2]^T [x | h1 | 1] and [g_b3 | dW3] = d0^T [1 | h2],
//                    Z and D read as MN-major operands (M or N = features, K =
//                    records).  Each block streams its range of 64-record
//                    slices through a three-stage pipeline (bulk copies into
//                    shared memory, completion on mbarriers; the products of
//                    one slice run while the next slices load) and writes its
//                    partial sums from tensor memory to global memory, in the
//                    parameter layout.
//   k_guide_grad_reduce  sums the blocks' partials into the gradient (no
//                    atomics), applying the loss's 1/n.
//
// Loss scaling: the fp16 activation gradients leave out the loss's 1/n
// (with n ~ 3e4 records most of them would be fp16 subnormals); they
// saturate at the fp16 range, and the 1/n is applied, in fp32, in the
// reduction.
constexpr int kZK = 288, kDK = 176;                    // halves per record in Z and D
constexpr int kZx = 0, kZh1 = 144, kZones = 208, kZh2 = 224;
constexpr int kDd0 = 0, kDd1 = 48, kDd2 = 112;
constexpr int kFbCols = 64;                            // tensor-memory columns of a forward/backward block
constexpr float kHalfMax = 65504.f;

struct GuideFbSmem {
    __half w[kGImgHalves];
    float bias[kGImgBiases];
    __half w2t[kGHid * kGHid];
    __half w3t[kGHid * kGOutPad];
    alignas(128) __half p[kTcRows * kGEnc];   // x (K = 144), then h2 (K = 64), then d2 (K = 64)
    alignas(128) __half q[kTcRows * kGHid];   // h1 (K = 64), then d0 (K = 48)
    uint64_t bar_w, bar_mma;
    uint32_t tmem;
    int fail;
};
static_assert(offsetof(GuideFbSmem, w2t) == kGImgW2T && offsetof(GuideFbSmem, w3t) == kGImgW3T, "image layout");
static_assert(2 * (sizeof(GuideFbSmem) + 1024) <= 228 * 1024, "two forward/backward blocks per SM");

__device__ __forceinline__ uint32_t pack_h2(float a, float b) {
    __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}
__device__ __forceinline__ uint32_t pack_h2_sat(float a, float b) {
    return pack_h2(fminf(fmaxf(a, -kHalfMax), kHalfMax), fminf(fmaxf(b, -kHalfMax), kHalfMax));
}

// One 16-byte chunk (features fs..fs+7 of row r in a shared operand with
// rows of K halves, none when smem is null; features fg..fg+7 of row r in
// the global staging tile with rows of G halves).
__device__ __forceinline__ void put_chunk(__half* smem, int K, __half* glob, int G, int r, int fs, int fg,
                                          uint4 v) {
    if (smem) *reinterpret_cast<uint4*>(smem + canon_index(r, fs, K)) = v;
    *reinterpret_cast<uint4*>(glob + canon_index(r, fg, G)) = v;
}

// Bias + ReLU of 64 accumulator columns: into shared memory (K = 64 rows,
// feature 0) and the Z staging tile at feature zf; returns the mask of the
// outputs that are > 0 after rounding.
__device__ __forceinline__ uint64_t fb_hidden_epilogue(uint32_t t, const float* bias, __half* smem, __half* zt,
                                                       int zf) {
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
        put_chunk(smem, kGHid, zt, kZK, r, c0, zf + c0, make_uint4(p[0], p[1], p[2], p[3]));
        put_chunk(smem, kGHid, zt, kZK, r, c0 + 8, zf + c0 + 8, make_uint4(p[4], p[5], p[6], p[7]));
    }
    return mask;
}

// 64 accumulator columns masked by `mask`: into shared memory (K = 64,
// feature 0; none when smem is null) and the D staging tile at feature df.
__device__ __forceinline__ void fb_backward_epilogue(uint32_t t, uint64_t mask, __half* smem, __half* dt, int df) {
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
        put_chunk(smem, kGHid, dt, kDK, r, c0, df + c0, make_uint4(p[0], p[1], p[2], p[3]));
        put_chunk(smem, kGHid, dt, kDK, r, c0 + 8, df + c0 + 8, make_uint4(p[4], p[5], p[6], p[7]));
    }
}

// K-major product of one layer: acc (128 x N) = A (rows of K halves at
// a_base) x W^T, W [N][K] at `w` (rows of K halves); completion on `bar`.
template <int K, int N>
__device__ __forceinline__ void fb_issue(uint32_t acc, uint32_t a_base, uint32_t w, uint64_t* bar) {
    constexpr uint32_t idesc = tc::idesc_f16_f32(kTcRows, N);
    tc::fence_after_sync();
#pragma unroll
    for (int ks = 0; ks < K / 16; ks++)
        tc::mma_f16(acc, tc::smem_desc(a_base + ks * 256, 128, K * 16), tc::smem_desc(w + ks * 256, 128, K * 16),
                    idesc, ks > 0 ? 1u : 0u);
    tc::commit(bar);
}

__global__ void __launch_bounds__(kTcRows) k_guide_fwdbwd(const void* image, const GuideRecord* s, int n, int stride,
                                                           const float* wsum, int nwsum, __half* zg, __half* dg,
                                                           float* loss, unsigned* err) {
    extern __shared__ __align__(128) unsigned char dyn_smem[];
    GuideFbSmem& S = *reinterpret_cast<GuideFbSmem*>(dyn_smem);
    const int tid = threadIdx.x;
    const int ntiles = (n + kTcRows - 1) / kTcRows;
    if ((int)blockIdx.x >= ntiles) return;
    if (tid == 0) {
        tc::mbar_init(&S.bar_w, 1);
        tc::mbar_init(&S.bar_mma, 1);
        S.fail = 0;
    }
    if (tid < 32) tc::tmem_alloc(&S.tmem, kFbCols);
    tc::pdl_launch_dependents();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // the weight copy lands while the first records load and encode; every
    // thread waits for it before the first product
    if (tid == 0) tc::bulk_load(S.w, image, kGImgTrainBytes, &S.bar_w);
    bool failed = false, weights = false;
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
    const uint32_t tl = T + ((uint32_t)(tid & ~31) << 16);  // this warp's lanes, column 0
    const uint32_t pa = tc::smem_addr(S.p), qa = tc::smem_addr(S.q), wa = tc::smem_addr(S.w);
    float mean = 0.f;   // read once the batch's weight sum is complete
    float lacc = 0.f;
    const uint32_t one2 = pack_h2(1.f, 1.f);
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int r = tile * kTcRows + tid;
        __half* zt = zg + (size_t)tile * kTcRows * kZK;
        __half* dt = dg + (size_t)tile * kTcRows * kDK;
        GuideRecord rec = {};
        if (r < n) rec = s[(size_t)r * stride];
        // x: the encoding, into P (K = 144) and Z; the columns of ones into Z
#pragma unroll
        for (int i = 0; i < kGIn; i++) {
            __half2 h[kGFreq];
            encode_scalar_h2(rec.in[i], h);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                uint4 v;
                v.x = *reinterpret_cast<const uint32_t*>(&h[4 * c]);
                v.y = *reinterpret_cast<const uint32_t*>(&h[4 * c + 1]);
                v.z = *reinterpret_cast<const uint32_t*>(&h[4 * c + 2]);
                v.w = *reinterpret_cast<const uint32_t*>(&h[4 * c + 3]);
                const int f = i * 2 * kGFreq + 8 * c;
                put_chunk(S.p, kGEnc, zt, kZK, tid, f, kZx + f, v);
            }
        }
        put_chunk(nullptr, 0, zt, kZK, tid, 0, kZones, make_uint4(one2, one2, one2, one2));
        put_chunk(nullptr, 0, zt, kZK, tid, 0, kZones + 8, make_uint4(one2, one2, one2, one2));
        if (!weights) {
            weights = true;
            if (!tc::mbar_wait(&S.bar_w, 0, kTcWaitNs)) {
                failed = true;
                S.fail = 1;
                atomicOr(err, kErrTensorWait);
            }
            tc::pdl_wait();   // k_guide_weight_sum has finished
            float sum = 0.f;
            for (int k = 0; k < nwsum; k++) sum += wsum[k];   // the same order in every block
            mean = sum / (float)n;
        }
        // the record's loss weight times n
        const float sc = r < n && rec.pdf > 0.f && mean > 0.f ? fminf(rec.L / rec.pdf / mean, kGTargetClamp) : 0.f;
        if (step_sync()) break;
        // layer 1: P (x) -> h1 into Q and Z
        if (tid == 0) fb_issue<kGEnc, kGHid>(T, pa, wa + 2 * kGImgW1, &S.bar_mma);
        wait();
        const uint64_t m1 = fb_hidden_epilogue(tl, S.bias + kGImgB1, S.q, zt, kZh1);
        if (step_sync()) break;
        // layer 2: Q (h1) -> h2 into P and Z
        if (tid == 0) fb_issue<kGHid, kGHid>(T, qa, wa + 2 * kGImgW2, &S.bar_mma);
        wait();
        const uint64_t m2 = fb_hidden_epilogue(tl, S.bias + kGImgB2, S.p, zt, kZh2);
        if (step_sync()) break;
        // layer 3: P (h2) -> outputs
        if (tid == 0) fb_issue<kGHid, kGOutPad>(T, pa, wa + 2 * kGImgW3, &S.bar_mma);
        wait();
        {   // loss and dLoss/dOutput of this thread's record (times n) into Q (K = 48) and D
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
                put_chunk(S.q, kGOutPad, dt, kDK, tid, c, kDd0 + c, make_uint4(p[0], p[1], p[2], p[3]));
            }
        }
        if (step_sync()) break;
        // backward through layer 3: Q (d0) x W3 -> d2 into P and D
        if (tid == 0) fb_issue<kGOutPad, kGHid>(T, qa, wa + kGImgW3T, &S.bar_mma);
        wait();
        fb_backward_epilogue(tl, m2, S.p, dt, kDd2);
        if (step_sync()) break;
        // backward through layer 2: P (d2) x W2 -> d1 into D
        if (tid == 0) fb_issue<kGHid, kGHid>(T, pa, wa + kGImgW2T, &S.bar_mma);
        wait();
        fb_backward_epilogue(tl, m1, nullptr, dt, kDd1);
        if (step_sync()) break;
    }
    for (int o = 16; o; o >>= 1) lacc += __shfl_xor_sync(0xffffffffu, lacc, o);
    if ((tid & 31) == 0) atomicAdd(loss, lacc / (float)n);
    tc::fence_before_sync();
    __syncthreads();
    if (S.fail) {
        (void)tc::mbar_wait(&S.bar_w, 0, kTcWaitNs);
        (void)tc::mbar_wait(&S.bar_mma, ph, kTcWaitNs);
    }
    if (tid < 32) {
        tc::fence_after_sync();
        tc::tmem_dealloc(T, kFbCols);
    }
}

// Weight gradients: split-K over 64-record slices of the staged Z and D.
constexpr int kWgRecs = 64;                            // records per pipeline stage
constexpr int kWgStages = 3;
constexpr uint32_t kWgZBytes = kWgRecs * kZK * 2;      // 36,864
constexpr uint32_t kWgDBytes = kWgRecs * kDK * 2;      // 22,528
constexpr int kWgCols = 512;                           // tensor memory: 224 + 80 accumulator columns
constexpr int kAcc12 = 0, kAcc3 = 224;

struct GuideWgSmem {
    alignas(128) __half z[kWgStages][kWgRecs * kZK];
    alignas(128) __half d[kWgStages][kWgRecs * kDK];
    uint64_t full[kWgStages], empty[kWgStages], done;
    uint32_t tmem;
    int fail;
};
// no other tensor-memory user of this library (the guided material and
// inference blocks, 107 KB) fits beside a block: its 512 columns are free
static_assert(sizeof(GuideWgSmem) + 1024 + 107 * 1024 > 228 * 1024, "one tensor-memory user per SM");

__global__ void __launch_bounds__(kTcRows) k_guide_wgrad(const __half* zg, const __half* dg, int nslices,
                                                          float* partial, unsigned* err) {
    extern __shared__ __align__(128) unsigned char dyn_smem[];
    GuideWgSmem& S = *reinterpret_cast<GuideWgSmem*>(dyn_smem);
    const int tid = threadIdx.x;
    // this block's slices [s0, s1)
    const int per = nslices / (int)gridDim.x, extra = nslices % (int)gridDim.x;
    const int b = blockIdx.x;
    const int s0 = b * per + min(b, extra), s1 = s0 + per + (b < extra ? 1 : 0);
    const int steps = s1 - s0;
    if (tid == 0) {
        for (int k = 0; k < kWgStages; k++) {
            tc::mbar_init(&S.full[k], 1);
            tc::mbar_init(&S.empty[k], 1);
        }
        tc::mbar_init(&S.done, 1);
        S.fail = 0;
    }
    if (tid < 32) tc::tmem_alloc(&S.tmem, kWgCols);
    tc::pdl_launch_dependents();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t T = S.tmem;
    tc::pdl_wait();   // k_guide_fwdbwd has staged every tile (and the previous reduction read the partials)
    if (tid == 0 && steps > 0) {
        bool failed = false;
        // per stage: the parity of its copy in flight, -1 for none (a stage
        // is refilled only after its previous copy was waited for)
        int inflight[kWgStages];
        for (int k = 0; k < kWgStages; k++) inflight[k] = -1;
        auto load = [&](int i) {  // slice s0 + i into stage i % kWgStages
            const int st = i % kWgStages;
            const size_t sl = (size_t)(s0 + i);
            inflight[st] = (i / kWgStages) & 1;
            tc::mbar_expect_tx(&S.full[st], kWgZBytes + kWgDBytes);
            tc::bulk_copy(S.z[st], zg + sl * kWgRecs * kZK, kWgZBytes, &S.full[st]);
            tc::bulk_copy(S.d[st], dg + sl * kWgRecs * kDK, kWgDBytes, &S.full[st]);
        };
        auto fail_now = [&]() {
            failed = true;
            S.fail = 1;
            atomicOr(err, kErrTensorWait);
        };
        for (int i = 0; i < min(kWgStages, steps); i++) load(i);
        constexpr uint32_t id12 = tc::idesc_f16_f32(kTcRows, 224, true, true);
        constexpr uint32_t id3 = tc::idesc_f16_f32(kTcRows, 80, true, true);
        for (int i = 0; i < steps && !failed; i++) {
            const int st = i % kWgStages;
            if (!tc::mbar_wait(&S.full[st], (uint32_t)(i / kWgStages) & 1u, kTcWaitNs)) {
                fail_now();
                break;
            }
            inflight[st] = -1;
            tc::fence_after_sync();
            const uint32_t za = tc::smem_addr(S.z[st]), da = tc::smem_addr(S.d[st]);
#pragma unroll
            for (int ks = 0; ks < kWgRecs / 16; ks++) {
                const uint32_t acc = i == 0 && ks == 0 ? 0u : 1u;
                tc::mma_f16(T + kAcc12, tc::smem_desc(da + (kDd1 / 8) * 128 + ks * 2 * kDK * 16, kDK * 16, 128),
                            tc::smem_desc(za + ks * 2 * kZK * 16, kZK * 16, 128), id12, acc);
                tc::mma_f16(T + kAcc3, tc::smem_desc(da + ks * 2 * kDK * 16, kDK * 16, 128),
                            tc::smem_desc(za + (kZones / 8) * 128 + ks * 2 * kZK * 16, kZK * 16, 128), id3, acc);
            }
            tc::commit(&S.empty[st]);
            // refill the stage the previous slice used, once its products are
            // done (this slice's products queue behind them meanwhile)
            const int j = i - 1;
            if (j >= 0 && j + kWgStages < steps) {
                const int sj = j % kWgStages;
                if (!tc::mbar_wait(&S.empty[sj], (uint32_t)(j / kWgStages) & 1u, kTcWaitNs)) {
                    fail_now();
                    break;
                }
                load(j + kWgStages);
            }
        }
        tc::commit(&S.done);
        if (!tc::mbar_wait(&S.done, 0, kTcWaitNs)) fail_now();
        if (failed) {
            // let every copy in flight land before the block frees its
            // shared memory (bounded waits)
            for (int k = 0; k < kWgStages; k++)
                if (inflight[k] >= 0) (void)tc::mbar_wait(&S.full[k], (uint32_t)inflight[k], kTcWaitNs);
        }
    }
    tc::fence_before_sync();
    const bool bad = __syncthreads_or(tid == 0 ? S.fail : 0) != 0;
    tc::fence_after_sync();
    // the block's partial sums, in the parameter layout (each thread writes
    // its accumulator lane's entries as contiguous runs); which columns a
    // warp reads depends on its lanes' units, the same for all its lanes
    float* out = partial + (size_t)b * kGParams;
    const uint32_t tl = T + ((uint32_t)(tid & ~31) << 16);
    const bool live = steps > 0 && !bad;
    const int m = tid, warp = tid >> 5;
    auto run = [&](uint32_t col, int ncols, int dst, bool keep) {  // ncols (16 or 32) columns -> out[dst ..)
        float v[32];
        if (!live) {
#pragma unroll
            for (int j = 0; j < 32; j++) v[j] = 0.f;
        } else if (ncols == 32) {
            tc::ld_32x32b_x32(tl + col, v);
        } else {
            tc::ld_32x32b_x16(tl + col, v);
        }
        if (keep)
            for (int j = 0; j < ncols; j += 4)
                *reinterpret_cast<float4*>(out + dst + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
        return v[0];
    };
    if (warp < 2) {
        // lanes 0..63: units of layer 1 (dW1 rows from the x columns, b1)
        for (int c0 = 0; c0 < 128; c0 += 32) (void)run(kAcc12 + c0, 32, kGW1 + m * kGEnc + c0, true);
        (void)run(kAcc12 + 128, 16, kGW1 + m * kGEnc + 128, true);
        out[kGB1 + m] = run(kAcc12 + kZones, 16, 0, false);
        // lanes 0..39 of the second product: the outputs (b3 in column 0, dW3 in 16..79)
        const bool o = m < kGOut;
        const float g3 = run(kAcc3, 16, 0, false);
        if (o) out[kGB3 + m] = g3;
        for (int c0 = 16; c0 < 80; c0 += 32) (void)run(kAcc3 + c0, 32, kGW3 + m * kGHid + (c0 - 16), o);
    } else {
        // lanes 64..127: units of layer 2 (dW2 rows from the h1 columns, b2)
        for (int c0 = 0; c0 < kGHid; c0 += 32)
            (void)run(kAcc12 + kZh1 + c0, 32, kGW2 + (m - kGHid) * kGHid + c0, true);
        out[kGB2 + m - kGHid] = run(kAcc12 + kZones, 16, 0, false);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (tid < 32) {
        tc::fence_after_sync();
        tc::tmem_dealloc(T, kWgCols);
    }
}

// grad[i] = (1/n) sum over the weight-gradient blocks of their partial
// sums (parameter layout).  A block takes 32 consecutive parameters; its 8
// warps split the partials and add their sums in shared memory.  The padding
// outputs of layer 3 (rows 40..47) have no entries and stay as they are.
constexpr int kRedWarps = 8;
__global__ void __launch_bounds__(32 * kRedWarps) k_guide_grad_reduce(const float* partial, int nblocks, float inv_n,
                                                                        float* grad) {
    __shared__ float s_sum[kRedWarps][32];
    tc::pdl_wait();   // k_guide_wgrad has written every block's partials
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int i = blockIdx.x * 32 + lane;
    const bool pad = (i >= kGW3 + kGOut * kGHid && i < kGB3) || i >= kGB3 + kGOut;
    float acc = 0.f;
    if (i < kGParams && !pad) {
#pragma unroll 4
        for (int b = w; b < nblocks; b += kRedWarps) acc += partial[(size_t)b * kGParams + i];
    }
    s_sum[w][lane] = acc;
    __syncthreads();
    if (w == 0 && i < kGParams && !pad) {
        float t = 0.f;
#pragma unroll
        for (int k = 0; k < kRedWarps; k++) t += s_sum[k][lane];
        grad[i] = t * inv_n;
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

// Device buffers of a training batch of up to n records: the staged
// activations (Z, D) and the weight-gradient partial sums.  Called before
// any training launch, outside graph captures and render loops.
void guide_reserve(dl_guide* G, int64_t n) {
    const int64_t ntiles = (n + kTcRows - 1) / kTcRows;
    G->stage_z.ensure((size_t)ntiles * kTcRows * kZK * 2);
    G->stage_d.ensure((size_t)ntiles * kTcRows * kDK * 2);
    const int64_t nslices = ntiles * (kTcRows / kWgRecs);
    const int64_t nb = std::min<int64_t>(nslices, std::max(1, G->ctx->num_sms));
    G->partial.ensure((size_t)nb * kGParams * 4);
    G->wsum.ensure(kWsumMaxBlocks * sizeof(float));
}

// Gradient of the loss over `n` device records (every `stride`-th) written
// to G->grad (entries outside the network's parameters untouched); the
// loss sum lands in scratch[1].  guide_reserve(G, n) must have run.
void guide_gradient(dl_guide* G, const void* d_recs, int64_t n, int stride, cudaStream_t st) {
    static const bool setup = [] {
        DL_CUDA(cudaFuncSetAttribute(k_guide_fwdbwd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sizeof(GuideFbSmem)));
        DL_CUDA(cudaFuncSetAttribute(k_guide_fwdbwd, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        DL_CUDA(cudaFuncSetAttribute(k_guide_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sizeof(GuideWgSmem)));
        return true;
    }();
    (void)setup;
    const int64_t ntiles = (n + kTcRows - 1) / kTcRows;
    const int64_t nslices = ntiles * (kTcRows / kWgRecs);
    const int sms = std::max(1, G->ctx->num_sms);
    const int nb = (int)std::min<int64_t>(nslices, sms);
    if (G->stage_z.bytes < (size_t)ntiles * kTcRows * kZK * 2 || G->stage_d.bytes < (size_t)ntiles * kTcRows * kDK * 2 ||
        G->partial.bytes < (size_t)nb * kGParams * 4 || G->wsum.bytes < kWsumMaxBlocks * sizeof(float))
        throw Error(DL_ERR_INVALID_ARG, "guide training buffers not reserved for this batch");
    float* sc = G->scratch.as<float>();   // [1]: the loss
    unsigned* err = reinterpret_cast<unsigned*>(G->scratch.as<char>() + kGuideErrOffset);
    const GuideRecord* R = static_cast<const GuideRecord*>(d_recs);
    const int nws = (int)std::min<int64_t>(kWsumMaxBlocks, (n + kWsumThreads - 1) / kWsumThreads);
    float* wsum = G->wsum.as<float>();
    k_guide_weight_sum<<<nws, kWsumThreads, 0, st>>>(R, (int)n, stride, wsum, sc + 1);
    // the next three kernels start their prologues while their predecessor
    // runs (programmatic dependent launch); each waits for it before using
    // what it wrote
    const int fb_blocks = (int)std::min<int64_t>(ntiles, 2 * (int64_t)sms);
    __half* zg = G->stage_z.as<__half>();
    __half* dg = G->stage_d.as<__half>();
    float* part = G->partial.as<float>();
    float* grad = G->grad.as<float>();
    const void* img = G->image.ptr;
    const int ni = (int)n, ns = (int)nslices;
    const float inv_n = 1.f / (float)n;
    DL_CUDA(launch_dependent(k_guide_fwdbwd, dim3(fb_blocks), dim3(kTcRows), sizeof(GuideFbSmem), st, img, R, ni,
                             stride, (const float*)wsum, nws, zg, dg, sc + 1, err));
    DL_CUDA(launch_dependent(k_guide_wgrad, dim3(nb), dim3(kTcRows), sizeof(GuideWgSmem), st, (const __half*)zg,
                             (const __half*)dg, ns, part, err));
    DL_CUDA(launch_dependent(k_guide_grad_reduce, dim3((kGParams + 31) / 32), dim3(32 * kRedWarps), 0, st,
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
