// Training and inference of the learned path-guiding proposal (guide.cuh)
// on the tensor cores, and the dl_guide C ABI.
//
// One training step on a batch of n records {position, normal, sampled
// direction w, its sampling pdf p, radiance estimate L along w}:
//   loss = -(1/n) sum_i min((L_i / p_i) / mean(L / p), 20) * log q(w_i)
// (an estimate of the KL divergence from the normalised incident radiance to
// the mixture q, up to a constant), then one Adam update.  Kernels:
//   k_guide_weight_sum   mean(L / p) over the batch
//   k_guide_fwd_bwd      per 16-row tile: encoding, forward (mma.sync),
//                        dLoss/dOutput, backward through layers 3 and 2
//                        (mma.sync); stores the fp16 activations and output
//                        gradients of every row, bias gradients by column
//                        sums
//   k_guide_wgrad        weight gradients dW = dY^T Z over the batch
//                        (mma.sync, K = batch rows)
//   k_guide_adam         Adam on the fp32 master weights; refreshes the fp16
//                        copy and the tensor cores' weight image
// Inference (k_guide_infer, and the guided material kernels in render.cu)
// runs on tcgen05 (guide_tc.cuh).
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
static_assert(kGImgBytes == kGuideImageBytes, "image size");

// Raw network outputs (40 per row) of n input rows, 128 rows per tile on
// the tensor cores.
__global__ void __launch_bounds__(kTcRows) k_guide_infer(const void* image, const float* in, float* out, int n,
                                                          unsigned* err) {
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    GuideTcSmem& S = *reinterpret_cast<GuideTcSmem*>(dyn_smem);
    const int ntiles = (n + kTcRows - 1) / kTcRows;
    if ((int)blockIdx.x >= ntiles) return;
    uint32_t phase = 0;
    bool ok = guide_tc_begin(S, image, err);
    for (int tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x) {
        const int r = tile * kTcRows + threadIdx.x;
        float x[kGIn] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (r < n)
            for (int i = 0; i < kGIn; i++) x[i] = in[(size_t)kGIn * r + i];
        __syncthreads();  // the previous tile's outputs have been read
        encode_row_tc(x, S.act, threadIdx.x);
        ok = guide_tc_forward(S, phase, err);
        if (ok && r < n) {
            const float* o = tc_out_row(S, threadIdx.x);
            for (int j = 0; j < kGOut; j++) out[(size_t)r * kGOut + j] = o[j];
        }
    }
    guide_tc_end(S, phase);
}

// -------------------------------------------------------------- training
constexpr int kTrainWarps = 2;
// Record weights L/p are normalised by their batch mean and clamped at this
// multiple of it: a few records near the sun would otherwise carry the
// whole gradient of a batch.
constexpr float kGTargetClamp = 20.f;
struct TrainTile {
    GuideTile f;                 // x: encoding, then layer-2 output; h: layer-1 output; o: output
    __half d0[16 * kGHs];        // dLoss / dOutput (48 used)
    __half d2[16 * kGHs];        // dLoss / d(layer-2 output)
};

// Activations of the batch kept for the weight gradients (halves, row-major).
struct TrainActs {
    __half* x;    // [n][144] encoding
    __half* h1;   // [n][64]
    __half* h2;   // [n][64]
    __half* d0;   // [n][48]
    __half* d2;   // [n][64]
    __half* d1;   // [n][64]
};

__global__ void k_guide_weight_sum(const GuideRecord* s, int n, int stride, float* sum) {
    float acc = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const GuideRecord& r = s[(size_t)i * stride];
        acc += r.pdf > 0.f ? r.L / r.pdf : 0.f;
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(sum, acc);
}

// Column sums over the 16 rows of a C fragment pair, added to g[col], g[col+1].
__device__ __forceinline__ void add_colsums(float* g, int col, float a0, float a1, int lane) {
    for (int o = 4; o < 32; o <<= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
    }
    if ((lane >> 2) == 0) {
        atomicAdd(g + col, a0);
        atomicAdd(g + col + 1, a1);
    }
}

// dY (16 x N) = (dIn (16 x K) W) masked by act > 0; W row-major [K][N] halves.
// Writes dY as halves to `out` (smem, stride lds) and `gout` (global, stride N),
// column sums of the fp32 values into gbias.
template <int K, int N>
__device__ __forceinline__ void backward16(const __half* din, int ldi, const __half* W, const __half* act, int lda,
                                           __half* out, int lds, __half* gout, float* gbias, int lane) {
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < N / 8; nt++) {
        float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int ks = 0; ks < K / 16; ks++) {
            uint32_t a[4], b[2];
            frag_a(a, din + ks * 16, ldi, lane);
            frag_b_w(b, W + (ks * 16) * N + nt * 8, N, lane);
            mma16816(c, a, b);
        }
        const int col = nt * 8 + 2 * t;
        if (!(__half2float(act[g * lda + col]) > 0.f)) c[0] = 0.f;
        if (!(__half2float(act[g * lda + col + 1]) > 0.f)) c[1] = 0.f;
        if (!(__half2float(act[(g + 8) * lda + col]) > 0.f)) c[2] = 0.f;
        if (!(__half2float(act[(g + 8) * lda + col + 1]) > 0.f)) c[3] = 0.f;
        __half h0 = __float2half_rn(c[0]), h1 = __float2half_rn(c[1]);
        __half h2 = __float2half_rn(c[2]), h3 = __float2half_rn(c[3]);
        out[g * lds + col] = h0;
        out[g * lds + col + 1] = h1;
        out[(g + 8) * lds + col] = h2;
        out[(g + 8) * lds + col + 1] = h3;
        gout[g * N + col] = h0;
        gout[g * N + col + 1] = h1;
        gout[(g + 8) * N + col] = h2;
        gout[(g + 8) * N + col + 1] = h3;
        add_colsums(gbias, col, c[0] + c[2], c[1] + c[3], lane);
    }
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

__global__ void __launch_bounds__(32 * kTrainWarps) k_guide_fwd_bwd(const __half* w16, const float* w32,
                                                                    const GuideRecord* s, int n, int stride,
                                                                    const float* wsum, float* grad,
                                                                    TrainActs A, float* loss) {
    __shared__ TrainTile tiles[kTrainWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    TrainTile& T = tiles[warp];
    const int ntiles = (n + 15) / 16;
    const float mean = *wsum / (float)n;
    float lacc = 0.f;
    for (int tile = blockIdx.x * kTrainWarps + warp; tile < ntiles; tile += gridDim.x * kTrainWarps) {
        const int r0 = tile * 16;
        const int r = r0 + (lane & 15);
        // rows past the batch are zero inputs with zero loss weight
        if (lane < 16) {
            float x[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (r < n)
                for (int i = 0; i < 6; i++) x[i] = s[(size_t)r * stride].in[i];
            encode_input(x, T.f.x + lane * kGXs);
            for (int k = 0; k < kGEnc; k++) A.x[(size_t)r * kGEnc + k] = T.f.x[lane * kGXs + k];
        }
        __syncwarp();
        // forward, keeping layer-1 (h) and layer-2 (x) activations
        layer16<kGEnc, kGHid, true>(T.f.x, kGXs, w16 + kGW1, w32 + kGB1, T.f.h, kGHs, nullptr, 0, lane);
        __syncwarp();
        layer16<kGHid, kGHid, true>(T.f.h, kGHs, w16 + kGW2, w32 + kGB2, T.f.x, kGXs, nullptr, 0, lane);
        __syncwarp();
        layer16<kGHid, kGOutPad, false>(T.f.x, kGXs, w16 + kGW3, w32 + kGB3, nullptr, 0, T.f.o, kGOs, lane);
        __syncwarp();
        if (lane < 16) {
            float d[kGOut];
            float sc = 0.f;
            GuideRecord rec = {};
            if (r < n) rec = s[(size_t)r * stride];
            if (r < n && rec.pdf > 0.f && mean > 0.f) sc = fminf(rec.L / rec.pdf / mean, kGTargetClamp) / (float)n;
            lacc += record_grad(T.f.o + lane * kGOs, rec, sc, d);
            for (int j = 0; j < kGOutPad; j++) {
                float v = j < kGOut ? d[j] : 0.f;
                T.d0[lane * kGHs + j] = __float2half_rn(v);
                A.d0[(size_t)r * kGOutPad + j] = __float2half_rn(v);
                if (j < kGOut && v != 0.f) atomicAdd(grad + kGB3 + j, v);
            }
            for (int k = 0; k < kGHid; k++) {
                A.h1[(size_t)r * kGHid + k] = T.f.h[lane * kGHs + k];
                A.h2[(size_t)r * kGHid + k] = T.f.x[lane * kGXs + k];
            }
        }
        __syncwarp();
        // backward through layers 3 and 2 (activation buffers hold whole
        // tiles: rows past the batch carry zero gradients)
        backward16<kGOutPad, kGHid>(T.d0, kGHs, w16 + kGW3, T.f.x, kGXs, T.d2, kGHs, A.d2 + (size_t)r0 * kGHid,
                                    grad + kGB2, lane);
        __syncwarp();
        backward16<kGHid, kGHid>(T.d2, kGHs, w16 + kGW2, T.f.h, kGHs, T.d0, kGHs, A.d1 + (size_t)r0 * kGHid,
                                 grad + kGB1, lane);
        __syncwarp();
    }
    for (int o = 16; o; o >>= 1) lacc += __shfl_xor_sync(0xffffffffu, lacc, o);
    if (lane == 0) atomicAdd(loss, lacc);
}

// G[m][n] += sum_r dY[r][m] Z[r][n] for m < M, n < N over rows [0, rows):
// one warp per (m16 x n8 tile, chunk of kWgradRows rows).
constexpr int kWgradRows = 512;

__global__ void k_guide_wgrad(const __half* dY, int ldy, const __half* Z, int ldz, int M, int N, int rows,
                              float* G) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int tiles_n = N / 8, tiles = (M / 16) * tiles_n;
    const int chunks = (rows + kWgradRows - 1) / kWgradRows;
    if (warp >= tiles * chunks) return;
    const int tile = warp % tiles, chunk = warp / tiles;
    const int m0 = (tile / tiles_n) * 16, n0 = (tile % tiles_n) * 8;
    const int g = lane >> 2, t = lane & 3;
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    const int rbeg = chunk * kWgradRows, rend = min(rows, rbeg + kWgradRows);
    const __half zero = __float2half_rn(0.f);
    auto ldy_at = [&](int r, int m) { return r < rend ? dY[(size_t)r * ldy + m] : zero; };
    auto ldz_at = [&](int r, int nn) { return r < rend ? Z[(size_t)r * ldz + nn] : zero; };
    for (int k0 = rbeg; k0 < rend; k0 += 16) {
        uint32_t a[4], b[2];
        // A[m][k] = dY[k][m]
        a[0] = pack2(ldy_at(k0 + 2 * t, m0 + g), ldy_at(k0 + 2 * t + 1, m0 + g));
        a[1] = pack2(ldy_at(k0 + 2 * t, m0 + g + 8), ldy_at(k0 + 2 * t + 1, m0 + g + 8));
        a[2] = pack2(ldy_at(k0 + 2 * t + 8, m0 + g), ldy_at(k0 + 2 * t + 9, m0 + g));
        a[3] = pack2(ldy_at(k0 + 2 * t + 8, m0 + g + 8), ldy_at(k0 + 2 * t + 9, m0 + g + 8));
        // B[k][n] = Z[k][n]
        b[0] = pack2(ldz_at(k0 + 2 * t, n0 + g), ldz_at(k0 + 2 * t + 1, n0 + g));
        b[1] = pack2(ldz_at(k0 + 2 * t + 8, n0 + g), ldz_at(k0 + 2 * t + 9, n0 + g));
        mma16816(c, a, b);
    }
    atomicAdd(G + (size_t)(m0 + g) * N + n0 + 2 * t, c[0]);
    atomicAdd(G + (size_t)(m0 + g) * N + n0 + 2 * t + 1, c[1]);
    atomicAdd(G + (size_t)(m0 + g + 8) * N + n0 + 2 * t, c[2]);
    atomicAdd(G + (size_t)(m0 + g + 8) * N + n0 + 2 * t + 1, c[3]);
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

size_t guide_act_bytes(int64_t rows) {
    return (size_t)rows * (kGEnc + 4 * kGHid + kGOutPad) * sizeof(__half);
}

void guide_init_params(uint64_t seed, std::vector<float>& w) { init_params(seed, w); }

void guide_upload_params(dl_guide* G, const float* host) {
    cudaStream_t st = G->ctx->stream;
    DL_CUDA(cudaMemcpyAsync(G->w32.ptr, host, kGParams * 4, cudaMemcpyHostToDevice, st));
    k_guide_to_half<<<64, 256, 0, st>>>(G->w32.as<float>(), G->w16.as<__half>(), G->image.as<unsigned char>());
    DL_CUDA(cudaGetLastError());
}

// Gradient of the loss over `n` device records into G->grad (added to it);
// returns nothing, the loss sum lands in scratch[1].
void guide_gradient(dl_guide* G, const void* d_recs, int64_t n, int stride, cudaStream_t st) {
    const int64_t ntiles = (n + 15) / 16, npad = ntiles * 16;
    G->acts.ensure(guide_act_bytes(npad));
    __half* a = G->acts.as<__half>();
    TrainActs A;
    A.x = a;
    A.h1 = A.x + npad * kGEnc;
    A.h2 = A.h1 + npad * kGHid;
    A.d0 = A.h2 + npad * kGHid;
    A.d2 = A.d0 + npad * kGOutPad;
    A.d1 = A.d2 + npad * kGHid;
    float* sc = G->scratch.as<float>();
    DL_CUDA(cudaMemsetAsync(sc, 0, 2 * sizeof(float), st));
    const GuideRecord* R = static_cast<const GuideRecord*>(d_recs);
    k_guide_weight_sum<<<(int)std::min<int64_t>(1024, (n + 255) / 256), 256, 0, st>>>(R, (int)n, stride, sc);
    const int blocks = (int)std::min<int64_t>((ntiles + kTrainWarps - 1) / kTrainWarps, 152 * 16);
    k_guide_fwd_bwd<<<blocks, 32 * kTrainWarps, 0, st>>>(G->w16.as<__half>(), G->w32.as<float>(), R, (int)n, stride,
                                                         sc,
                                                         G->grad.as<float>(), A, sc + 1);
    auto wgrad = [&](const __half* dy, int ldy, const __half* z, int ldz, int M, int N, float* out) {
        const int tiles = (M / 16) * (N / 8);
        const int chunks = (int)((npad + kWgradRows - 1) / kWgradRows);
        const int warps = tiles * chunks;
        k_guide_wgrad<<<(warps + 3) / 4, 128, 0, st>>>(dy, ldy, z, ldz, M, N, (int)npad, out);
    };
    float* g = G->grad.as<float>();
    wgrad(A.d1, kGHid, A.x, kGEnc, kGHid, kGEnc, g + kGW1);
    wgrad(A.d2, kGHid, A.h1, kGHid, kGHid, kGHid, g + kGW2);
    wgrad(A.d0, kGOutPad, A.h2, kGHid, kGOutPad, kGHid, g + kGW3);
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
    const int by_regs = prop.regsPerMultiprocessor / std::max(1, regs_per_warp * (kTcRows / 32));
    const size_t smem = sizeof(GuideTcSmem) + fa.sharedSizeBytes + prop.reservedSharedMemPerBlock;
    return std::max(1, std::min(by_regs, (int)(prop.sharedMemPerMultiprocessor / smem)));
}

void guide_forward(dl_guide* G, const float* d_in, float* d_out, int64_t n) {
    static const int per_sm = infer_blocks_per_sm();
    cudaStream_t st = G->ctx->stream;
    unsigned* err = reinterpret_cast<unsigned*>(G->scratch.as<char>() + kGuideErrOffset);
    DL_CUDA(cudaMemsetAsync(err, 0, sizeof(unsigned), st));
    const int64_t ntiles = (n + kTcRows - 1) / kTcRows;
    const int blocks = (int)std::min<int64_t>(ntiles, (int64_t)G->ctx->num_sms * per_sm);
    k_guide_infer<<<blocks, kTcRows, sizeof(GuideTcSmem), st>>>(G->image.ptr, d_in, d_out, (int)n, err);
    DL_CUDA(cudaGetLastError());
}

}  // namespace dl
