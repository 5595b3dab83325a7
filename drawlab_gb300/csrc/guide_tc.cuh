// The guiding network (guide.cuh) on the fifth-generation tensor cores.
//
// A block holds G warpgroups (two in the guided material kernels, five in
// the standalone inference kernel) that share one copy of the weights; each
// warpgroup evaluates its own 128 rows at a time, one row per thread,
// independently of the others (G tiles in flight per block, synchronised by
// per-warpgroup named barriers).  Each thread writes
// its row's input encoding into its warpgroup's operand tile; the
// warpgroup's first thread issues each layer as tcgen05.mma instructions
// (M = 128 rows, N = 64 or 48 outputs, K = 16 per instruction) with both
// operands in shared memory and the fp32 accumulator in the warpgroup's 64
// tensor-memory columns; completion arrives on the warpgroup's mbarrier.
// Each warp then reads its 32 rows back with tcgen05.ld, adds the bias,
// applies ReLU, and writes the fp16 activations as the next layer's
// operand.  The outputs land, fp32, in a per-row slot of shared memory.
//
// The weights reach shared memory in one bulk copy (cp.async.bulk) of the
// weight image: the fp16 matrices already in the tensor core's canonical
// K-major layout, followed by the fp32 biases (and, for the training
// kernel, transposed copies of W2 and W3).  The Adam kernel keeps the image
// current (guide.cu).
//
// Every wait is bounded (one second): a wait that runs out sets bit 2 of the
// error word, the block stops using the network (its paths sample the BSDF
// alone, which stays unbiased) and waits once more, again bounded, for its
// outstanding copies before it frees its tensor memory.
#pragma once

#include <cuda_fp16.h>

#include <cstddef>

#include "guide.cuh"
#include "tcgen05.cuh"

namespace dl {

constexpr int kTcRows = 128;                     // rows per tile = threads per warpgroup
constexpr int kTcGroups = 2;                     // warpgroups (tiles in flight) per guided block
constexpr int kTcThreads = kTcRows * kTcGroups;  // threads per guided block
constexpr uint64_t kTcWaitNs = 1000000000ull;
constexpr unsigned kErrTensorWait = 2u;  // error-word bit: a tensor-core wait ran out

// Weight image: W1 [64][144], W2 [64][64], W3 [48][64] (halves, canonical
// layout), then the biases b1 [64], b2 [64], b3 [48] (floats).
constexpr int kGImgW1 = 0;
constexpr int kGImgW2 = kGImgW1 + kGHid * kGEnc;
constexpr int kGImgW3 = kGImgW2 + kGHid * kGHid;
constexpr int kGImgHalves = kGImgW3 + kGOutPad * kGHid;  // 16384
constexpr int kGImgB1 = 0, kGImgB2 = kGHid, kGImgB3 = 2 * kGHid;
constexpr int kGImgBiases = 2 * kGHid + kGOutPad;            // 176
constexpr int kGImgBytes = kGImgHalves * 2 + kGImgBiases * 4;  // 33472: what inference loads
// The training kernel also loads the transposed matrices of layers 2 and 3
// (the backward pass multiplies by W, not W^T): W2^T [64][64] and W3^T [64][48].
constexpr int kGImgW2T = kGImgBytes;                                  // byte offsets
constexpr int kGImgW3T = kGImgW2T + kGHid * kGHid * 2;
constexpr int kGImgTrainBytes = kGImgW3T + kGHid * kGOutPad * 2;      // 47808
static_assert(kGImgBytes % 16 == 0 && kGImgTrainBytes % 16 == 0, "bulk copies move multiples of 16 bytes");

// Canonical layout without swizzle of an R x K fp16 matrix (R rows of K
// halves): core matrices of 8 rows x 8 halves stored as 128 contiguous
// bytes; core matrices adjacent along K are 128 bytes apart, 8-row groups
// K * 16 bytes apart.  Read as a K-major operand (rows = M or N), the
// descriptor's leading byte offset is 128 and its stride byte offset K * 16.
// The same bytes read as an MN-major operand (rows = the K dimension of the
// product, the K halves = M or N) take leading byte offset K * 16 (along the
// product's K) and stride byte offset 128 (along M or N): the no-swizzle
// descriptor keeps the leading offset on the product's K axis either way.
__host__ __device__ constexpr int canon_index(int r, int k, int K) {
    return (r >> 3) * (K * 8) + (k >> 3) * 64 + (r & 7) * 8 + (k & 7);
}

__host__ __device__ constexpr bool guide_param_is_weight(int i) {
    return i < kGB1 || (i >= kGW2 && i < kGB2) || (i >= kGW3 && i < kGB3);
}

// Byte offset in the weight image of parameter i (parameter layout of guide.cuh).
__host__ __device__ constexpr int guide_image_offset(int i) {
    return i < kGB1   ? 2 * (kGImgW1 + canon_index((i - kGW1) / kGEnc, (i - kGW1) % kGEnc, kGEnc))
           : i < kGW2 ? kGImgHalves * 2 + 4 * (kGImgB1 + i - kGB1)
           : i < kGB2 ? 2 * (kGImgW2 + canon_index((i - kGW2) / kGHid, (i - kGW2) % kGHid, kGHid))
           : i < kGW3 ? kGImgHalves * 2 + 4 * (kGImgB2 + i - kGB2)
           : i < kGB3 ? 2 * (kGImgW3 + canon_index((i - kGW3) / kGHid, (i - kGW3) % kGHid, kGHid))
                      : kGImgHalves * 2 + 4 * (kGImgB3 + i - kGB3);
}

// Byte offset of parameter i in the transposed copies, -1 outside W2 and W3.
__host__ __device__ constexpr int guide_image_offset_t(int i) {
    return (i >= kGW2 && i < kGB2)
               ? kGImgW2T + 2 * canon_index((i - kGW2) % kGHid, (i - kGW2) / kGHid, kGHid)
           : (i >= kGW3 && i < kGB3)
               ? kGImgW3T + 2 * canon_index((i - kGW3) % kGHid, (i - kGW3) / kGHid, kGOutPad)
               : -1;
}

__device__ __forceinline__ void write_image(unsigned char* img, int i, float v) {
    if (guide_param_is_weight(i)) {
        const __half h = __float2half_rn(v);
        *reinterpret_cast<__half*>(img + guide_image_offset(i)) = h;
        const int t = guide_image_offset_t(i);
        if (t >= 0) *reinterpret_cast<__half*>(img + t) = h;
    } else {
        *reinterpret_cast<float*>(img + guide_image_offset(i)) = v;
    }
}

// floats per output row: the 40 outputs, decoded in place into 48 lobe
// floats; odd, so the rows of a warp fall in distinct banks
constexpr int kTcOutStride = kGStoredLobes + 1;

// Shared memory of a block of G warpgroups (tiles in flight) sharing one
// weight copy; 64 tensor-memory columns per warpgroup (the allocation is
// rounded up to a power of two).
template <int G>
struct GuideTcSmemT {
    static constexpr int kGroups = G;
    static constexpr uint32_t kCols = G <= 2 ? 128u : G <= 4 ? 256u : 512u;
    static_assert(G >= 1 && G <= 8, "one to eight warpgroups");
    __half w[kGImgHalves];    // the image: weights ...
    float bias[kGImgBiases];  // ... and biases, contiguous
    // per warpgroup: encodings; then the hidden activations (K = 64 layout);
    // then the fp32 outputs (kTcOutStride floats per row), decoded in place
    alignas(16) __half act[G][kTcRows * kGEnc];
    uint64_t bar_w, bar_mma[G];
    uint32_t tmem;
    int fail;
};
using GuideTcSmem = GuideTcSmemT<kTcGroups>;
static_assert(offsetof(GuideTcSmem, bias) == kGImgHalves * 2, "image layout");
static_assert(offsetof(GuideTcSmem, act) % 16 == 0 && (kTcRows * kGEnc * 2) % 16 == 0, "operand alignment");
static_assert(kTcRows * kTcOutStride * 4 <= kTcRows * kGEnc * 2, "outputs fit the operand tile");

__device__ __forceinline__ int tc_group() { return (int)threadIdx.x >> 7; }  // the thread's warpgroup
__device__ __forceinline__ int tc_row() { return (int)threadIdx.x & (kTcRows - 1); }  // its row in the tile

// Named barrier 1 + g over warpgroup g's 128 threads (0 is __syncthreads).
__device__ __forceinline__ void wg_sync(int g) {
    asm volatile("bar.sync %0, 128;\n" :: "r"(1 + g) : "memory");
}
// The same barrier, returning whether `pred` holds in any of its threads.
__device__ __forceinline__ bool wg_or(int g, bool pred) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, %2, 128, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r) : "r"((uint32_t)pred), "r"(1 + g) : "memory");
    return r != 0;
}

template <class Sm>
__device__ __forceinline__ float* tc_out_row(Sm& S, int g, int r) {
    return reinterpret_cast<float*>(S.act[g]) + r * kTcOutStride;
}

template <class Sm>
__device__ __forceinline__ void tc_record_failure(Sm& S, unsigned* err) {
    S.fail = 1;
    if (err) atomicOr(err, kErrTensorWait);
}

// Block start (all threads): barriers, tensor memory, the weight image.
// Returns false (in every thread) when the weights did not arrive in time.
template <class Sm>
__device__ __forceinline__ bool guide_tc_begin(Sm& S, const void* image, unsigned* err) {
    if (threadIdx.x == 0) {
        tc::mbar_init(&S.bar_w, 1);
        for (int g = 0; g < Sm::kGroups; g++) tc::mbar_init(&S.bar_mma[g], 1);
        S.fail = 0;
    }
    if (threadIdx.x < 32) tc::tmem_alloc(&S.tmem, Sm::kCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (threadIdx.x == 0) tc::bulk_load(S.w, image, kGImgBytes, &S.bar_w);
    const bool ok = tc::mbar_wait(&S.bar_w, 0, kTcWaitNs);
    if (!ok) tc_record_failure(S, err);
    return __syncthreads_and(ok) != 0;
}

// Block end (all threads): after a failed wait, wait (bounded) for the
// outstanding weight copy and the thread's warpgroup's outstanding layer
// (`mma_phase`: that warpgroup's next parity), then free the tensor memory.
template <class Sm>
__device__ __forceinline__ void guide_tc_end(Sm& S, uint32_t mma_phase) {
    tc::fence_before_sync();
    __syncthreads();
    if (S.fail) {
        (void)tc::mbar_wait(&S.bar_w, 0, kTcWaitNs);
        (void)tc::mbar_wait(&S.bar_mma[tc_group()], mma_phase, kTcWaitNs);
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        tc::fence_after_sync();
        tc::tmem_dealloc(S.tmem, Sm::kCols);
    }
}

// The encoding of one input row, written as 16-byte chunks of the canonical
// layout of a matrix with rows of K halves (features 0..143 of row r).
__device__ __forceinline__ void encode_row_tc(const float* in6, __half* act, int r, int K = kGEnc) {
#pragma unroll
    for (int i = 0; i < kGIn; i++) {
        __half2 h[kGFreq];
        encode_scalar_h2(in6[i], h);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            uint4 v;
            v.x = *reinterpret_cast<const uint32_t*>(&h[4 * c]);
            v.y = *reinterpret_cast<const uint32_t*>(&h[4 * c + 1]);
            v.z = *reinterpret_cast<const uint32_t*>(&h[4 * c + 2]);
            v.w = *reinterpret_cast<const uint32_t*>(&h[4 * c + 3]);
            *reinterpret_cast<uint4*>(act + canon_index(r, i * 2 * kGFreq + 8 * c, K)) = v;
        }
    }
}

// One layer of warpgroup g: D (its tensor-memory columns) = act (128 x K)
// W^T, W [N][K] in the image.
template <int K, int N, class Sm>
__device__ __forceinline__ void tc_issue_layer(Sm& S, int g, int w_off) {
    constexpr uint32_t idesc = tc::idesc_f16_f32(kTcRows, N);
    const uint32_t a = tc::smem_addr(S.act[g]), b = tc::smem_addr(S.w + w_off);
    tc::fence_after_sync();
#pragma unroll
    for (int ks = 0; ks < K / 16; ks++)
        tc::mma_f16(S.tmem + 64u * g, tc::smem_desc(a + ks * 256, 128, K * 16), tc::smem_desc(b + ks * 256, 128, K * 16),
                    idesc, ks > 0 ? 1u : 0u);
    tc::commit(&S.bar_mma[g]);
}

// The warp's 32 accumulator lanes in its warpgroup's columns.
template <class Sm>
__device__ __forceinline__ uint32_t tc_warp_tmem(const Sm& S, int g) {
    return S.tmem + 64u * g + ((uint32_t)(tc_row() & ~31) << 16);
}

// Bias + ReLU of the warp's 32 rows (64 columns of tensor memory), written
// as the next layer's operand (K = 64 layout).
template <class Sm>
__device__ __forceinline__ void tc_hidden_epilogue(Sm& S, int g, const float* bias) {
    const int r = tc_row();
    const uint32_t t = tc_warp_tmem(S, g);
    __half* act = S.act[g];
#pragma unroll
    for (int c0 = 0; c0 < kGHid; c0 += 16) {
        float v[16];
        tc::ld_32x32b_x16(t + c0, v);
        uint32_t p[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            __half2 h = __floats2half2_rn(fmaxf(v[2 * j] + bias[c0 + 2 * j], 0.f),
                                          fmaxf(v[2 * j + 1] + bias[c0 + 2 * j + 1], 0.f));
            p[j] = *reinterpret_cast<const uint32_t*>(&h);
        }
        *reinterpret_cast<uint4*>(act + canon_index(r, c0, kGHid)) = make_uint4(p[0], p[1], p[2], p[3]);
        *reinterpret_cast<uint4*>(act + canon_index(r, c0 + 8, kGHid)) = make_uint4(p[4], p[5], p[6], p[7]);
    }
    tc::fence_smem_to_async();
}

// Runs the network on the 128 rows whose encodings the threads of
// warpgroup g wrote to S.act[g].  All threads of the warpgroup call it
// together.  On return (true) each thread's 40 outputs are at
// tc_out_row(S, g, tc_row()).  `phase` is the parity of the next completion
// of S.bar_mma[g], kept by every thread of the warpgroup.  Returns false
// (the same in every thread of the warpgroup) after a wait ran out.
template <class Sm>
__device__ __forceinline__ bool guide_tc_forward(Sm& S, int g, uint32_t& phase, unsigned* err) {
    bool failed = false;
    const bool issuer = tc_row() == 0;
    auto wait = [&]() {
        if (!tc::mbar_wait(&S.bar_mma[g], phase, kTcWaitNs)) {
            failed = true;
            tc_record_failure(S, err);
        } else {
            phase ^= 1u;
        }
        tc::fence_after_sync();
    };
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    wg_sync(g);
    if (issuer) tc_issue_layer<kGEnc, kGHid>(S, g, kGImgW1);
    wait();
    tc_hidden_epilogue(S, g, S.bias + kGImgB1);
    tc::fence_before_sync();
    if (wg_or(g, failed)) return false;
    if (issuer) tc_issue_layer<kGHid, kGHid>(S, g, kGImgW2);
    wait();
    tc_hidden_epilogue(S, g, S.bias + kGImgB2);
    tc::fence_before_sync();
    if (wg_or(g, failed)) return false;
    if (issuer) tc_issue_layer<kGHid, kGOutPad>(S, g, kGImgW3);
    wait();
    tc::fence_before_sync();
    if (wg_or(g, failed)) return false;
    tc::fence_after_sync();
    float* out = tc_out_row(S, g, tc_row());
    const uint32_t t = tc_warp_tmem(S, g);
#pragma unroll
    for (int c0 = 0; c0 < kGOutPad; c0 += 16) {
        float v[16];
        tc::ld_32x32b_x16(t + c0, v);
#pragma unroll
        for (int j = 0; j < 16; j++)
            if (c0 + j < kGOut) out[c0 + j] = v[j] + S.bias[kGImgB3 + c0 + j];
    }
    return true;
}

}  // namespace dl
