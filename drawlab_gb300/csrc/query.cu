// Device queries of single plugin functions, behind dl_bsdf_query and
// dl_scene_env_query: the reference's BSDF::eval / pdf / sample
// (include/tracer/bsdf.h:62-104, and the OptiX material callables of
// src/optix/cuda/material/*.cu) and its Envmap::sampleDirection /
// pdfDirection / eval (include/optix/light/envmap.h:25-94), evaluated by the
// same device functions the material and miss kernels inline, on batches of
// given directions and uniform numbers.  They let the per-function golden
// vectors recorded from the reference's own code check the device code
// directly, not only through whole paths.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "device.cuh"
#include "internal.h"
#include "scene.h"

namespace dl {

struct BsdfQueryOut {
    float* eval;   // n x 3
    float* pdf;    // n
    float* s_wo;   // n x 3
    float* s_w;    // n x 3
    float* s_eta;  // n
    int* s_measure;
};

template <int T>
__global__ void __launch_bounds__(128) k_bsdf_query(DevMaterial m, int64_t n, const float* __restrict__ wi,
                                                     const float* __restrict__ wo, const float* __restrict__ smp,
                                                     BsdfQueryOut out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        BRec q;
        q.wi = f3(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
        q.wo = f3(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
        q.measure = M_SOLID;
        q.eta = 1.f;
        const float3 e = bsdf_eval<T>(m, q);
        out.eval[3 * i] = e.x;
        out.eval[3 * i + 1] = e.y;
        out.eval[3 * i + 2] = e.z;
        out.pdf[i] = bsdf_pdf<T>(m, q);
        BRec s;
        s.wi = q.wi;
        s.wo = f3(0.f, 0.f, 0.f);
        s.measure = M_UNKNOWN;
        s.eta = 1.f;
        const float3 w = bsdf_sample<T>(m, s, make_float2(smp[3 * i], smp[3 * i + 1]), smp[3 * i + 2]);
        out.s_wo[3 * i] = s.wo.x;
        out.s_wo[3 * i + 1] = s.wo.y;
        out.s_wo[3 * i + 2] = s.wo.z;
        out.s_w[3 * i] = w.x;
        out.s_w[3 * i + 1] = w.y;
        out.s_w[3 * i + 2] = w.z;
        out.s_eta[i] = s.eta;
        out.s_measure[i] = s.measure;
    }
}

// Envmap queries of a scene: samples from (xi, shading normal) and the
// density and radiance of given directions.
__global__ void __launch_bounds__(128) k_env_query(DevScene sc, int64_t n, const float* __restrict__ xi,
                                                    const float* __restrict__ nrm, const float* __restrict__ dirs,
                                                    float* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float3 d;
        float spdf = 0.f;
        const float3 r = env_sample(sc, f3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]),
                                    f3(xi[3 * i], xi[3 * i + 1], xi[3 * i + 2]), d, spdf);
        const float3 q = f3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]);
        const float3 v = env_lookup_dir(sc, q);
        float* o = out + 11 * i;
        o[0] = d.x;
        o[1] = d.y;
        o[2] = d.z;
        o[3] = spdf;
        o[4] = r.x;
        o[5] = r.y;
        o[6] = r.z;
        o[7] = env_pdf(sc, q);
        o[8] = v.x;
        o[9] = v.y;
        o[10] = v.z;
    }
}

namespace {
int query_grid(const dl_context* ctx, int64_t n) {
    const int sms = ctx->num_sms > 0 ? ctx->num_sms : 152;
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + 127) / 128, (int64_t)sms * 8));
}

// One device allocation per call, freed on every exit path.
struct Scratch {
    void* p = nullptr;
    explicit Scratch(size_t bytes) {
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            throw Error(e == cudaErrorMemoryAllocation ? DL_ERR_OOM : DL_ERR_CUDA,
                        std::string("cudaMalloc: ") + cudaGetErrorString(e));
        }
    }
    ~Scratch() {
        if (p) cudaFree(p);
    }
    template <typename T>
    T* at(size_t byte_offset) const { return reinterpret_cast<T*>(static_cast<char*>(p) + byte_offset); }
};
}  // namespace

void bsdf_query(dl_context* ctx, const dl_material_desc& md, int64_t n, const float* wi, const float* wo,
                const float* smp, float* eval, float* pdf, float* s_wo, float* s_w, float* s_eta, int32_t* s_measure) {
    if (n == 0) return;
    cudaStream_t st = ctx->stream;
    DevMaterial m;
    std::memset(&m, 0, sizeof(m));
    m.type = md.type;
    for (int k = 0; k < 3; k++) {
        m.albedo[k] = md.albedo[k];
        m.specular[k] = md.specular[k];
    }
    m.ax = md.alpha[0];
    m.ay = md.alpha[1];
    m.int_ior = md.int_ior;
    m.ext_ior = md.ext_ior;
    m.ks = 1 - std::max(std::max(md.albedo[0], md.albedo[1]), md.albedo[2]);
    for (int k = 0; k < kTexSlots; k++) m.tex[k] = -1;
    m.has_tex = 0;
    // inputs wi, wo, smp (3n words each); outputs eval 3n, pdf n, s_wo 3n,
    // s_w 3n, s_eta n, s_measure n
    const size_t f = sizeof(float) * (size_t)n;
    Scratch buf(f * 21);
    float* d_wi = buf.at<float>(0);
    float* d_wo = buf.at<float>(3 * f);
    float* d_smp = buf.at<float>(6 * f);
    BsdfQueryOut out;
    out.eval = buf.at<float>(9 * f);
    out.pdf = buf.at<float>(12 * f);
    out.s_wo = buf.at<float>(13 * f);
    out.s_w = buf.at<float>(16 * f);
    out.s_eta = buf.at<float>(19 * f);
    out.s_measure = buf.at<int>(20 * f);
    DL_CUDA(cudaMemcpyAsync(d_wi, wi, 3 * f, cudaMemcpyHostToDevice, st));
    DL_CUDA(cudaMemcpyAsync(d_wo, wo, 3 * f, cudaMemcpyHostToDevice, st));
    DL_CUDA(cudaMemcpyAsync(d_smp, smp, 3 * f, cudaMemcpyHostToDevice, st));
    const int g = query_grid(ctx, n);
    switch (m.type) {
        case MAT_DIFFUSE: k_bsdf_query<MAT_DIFFUSE><<<g, 128, 0, st>>>(m, n, d_wi, d_wo, d_smp, out); break;
        case MAT_MIRROR: k_bsdf_query<MAT_MIRROR><<<g, 128, 0, st>>>(m, n, d_wi, d_wo, d_smp, out); break;
        case MAT_DIELECTRIC: k_bsdf_query<MAT_DIELECTRIC><<<g, 128, 0, st>>>(m, n, d_wi, d_wo, d_smp, out); break;
        case MAT_MICROFACET: k_bsdf_query<MAT_MICROFACET><<<g, 128, 0, st>>>(m, n, d_wi, d_wo, d_smp, out); break;
        case MAT_ANISO_GGX: k_bsdf_query<MAT_ANISO_GGX><<<g, 128, 0, st>>>(m, n, d_wi, d_wo, d_smp, out); break;
        default: throw Error(DL_ERR_INVALID_ARG, "dl_bsdf_query: unknown material type");
    }
    DL_CUDA(cudaGetLastError());
    DL_CUDA(cudaMemcpyAsync(eval, out.eval, 3 * f, cudaMemcpyDeviceToHost, st));
    DL_CUDA(cudaMemcpyAsync(pdf, out.pdf, f, cudaMemcpyDeviceToHost, st));
    DL_CUDA(cudaMemcpyAsync(s_wo, out.s_wo, 3 * f, cudaMemcpyDeviceToHost, st));
    DL_CUDA(cudaMemcpyAsync(s_w, out.s_w, 3 * f, cudaMemcpyDeviceToHost, st));
    DL_CUDA(cudaMemcpyAsync(s_eta, out.s_eta, f, cudaMemcpyDeviceToHost, st));
    DL_CUDA(cudaMemcpyAsync(s_measure, out.s_measure, f, cudaMemcpyDeviceToHost, st));
    DL_CUDA(cudaStreamSynchronize(st));
}

void env_query(dl_scene* S, int64_t n, const float* xi, const float* nrm, const float* dirs, float* s_dir,
               float* s_pdf, float* s_val, float* pdf, float* val) {
    if (S->dev.env_light < 0) throw Error(DL_ERR_INVALID_ARG, "dl_scene_env_query: the scene has no envmap");
    if (n == 0) return;
    dl_context* ctx = S->ctx;
    cudaStream_t st = ctx->stream;
    const size_t f = sizeof(float) * (size_t)n;
    Scratch buf(f * (9 + 11));
    float* d_xi = buf.at<float>(0);
    float* d_nrm = buf.at<float>(3 * f);
    float* d_dirs = buf.at<float>(6 * f);
    float* d_out = buf.at<float>(9 * f);
    DL_CUDA(cudaMemcpyAsync(d_xi, xi, 3 * f, cudaMemcpyHostToDevice, st));
    DL_CUDA(cudaMemcpyAsync(d_nrm, nrm, 3 * f, cudaMemcpyHostToDevice, st));
    DL_CUDA(cudaMemcpyAsync(d_dirs, dirs, 3 * f, cudaMemcpyHostToDevice, st));
    k_env_query<<<query_grid(ctx, n), 128, 0, st>>>(S->dev, n, d_xi, d_nrm, d_dirs, d_out);
    DL_CUDA(cudaGetLastError());
    std::vector<float> h((size_t)n * 11);
    DL_CUDA(cudaMemcpyAsync(h.data(), d_out, 11 * f, cudaMemcpyDeviceToHost, st));
    DL_CUDA(cudaStreamSynchronize(st));
    for (int64_t i = 0; i < n; i++) {
        const float* o = &h[11 * (size_t)i];
        for (int k = 0; k < 3; k++) {
            s_dir[3 * i + k] = o[k];
            s_val[3 * i + k] = o[4 + k];
            val[3 * i + k] = o[8 + k];
        }
        s_pdf[i] = o[3];
        pdf[i] = o[7];
    }
}

}  // namespace dl

namespace dl {

// ------------------------------------------------------ L2 read bandwidth
// Streams a buffer that fits in L2 with L2-only loads (ld.global.cg: no L1
// allocation), `passes` times over, after one warm-up pass: the L2 -> SM
// read bandwidth that bounds the traversal kernels' node and triangle
// fetches when the BVH is L2-resident.  One pass reads the buffer once in
// total over all threads; the xor of what a thread read is stored only if
// it equals `sentinel` (never, in practice), which keeps the loads live.
__global__ void __launch_bounds__(256) k_l2_read(const float4* __restrict__ buf, int64_t n4, int passes,
                                                  unsigned sentinel, unsigned* __restrict__ out) {
    unsigned acc = 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int p = 0; p < passes; p++) {
        // start each pass at a different offset so a thread reads other lines
        const int64_t start = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x + (int64_t)p * 4099 * 32) % stride;
        for (int64_t i = start; i < n4; i += stride) {
            float4 v;
            asm volatile("ld.global.cg.v4.f32 {%0, %1, %2, %3}, [%4];"
                         : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                         : "l"(buf + i));
            acc ^= __float_as_uint(v.x) ^ __float_as_uint(v.y) ^ __float_as_uint(v.z) ^ __float_as_uint(v.w);
        }
    }
    if (acc == sentinel) out[0] = acc;
}

double measure_l2_read(dl_context* ctx, int64_t bytes, int passes) {
    cudaStream_t st = ctx->stream;
    const int64_t n4 = bytes / 16;
    Scratch buf((size_t)n4 * 16 + 256);
    float4* d = buf.at<float4>(0);
    unsigned* out = buf.at<unsigned>((size_t)n4 * 16);
    DL_CUDA(cudaMemsetAsync(d, 0x3c, (size_t)n4 * 16, st));
    const int sms = ctx->num_sms > 0 ? ctx->num_sms : 152;
    const int grid = sms * 8;
    k_l2_read<<<grid, 256, 0, st>>>(d, n4, 1, 0x9e3779b9u, out);  // warm-up: the buffer into L2
    DL_CUDA(cudaEventRecord(ctx->ev0, st));
    k_l2_read<<<grid, 256, 0, st>>>(d, n4, passes, 0x9e3779b9u, out);
    DL_CUDA(cudaEventRecord(ctx->ev1, st));
    DL_CUDA(cudaGetLastError());
    DL_CUDA(cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    DL_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    return (double)n4 * 16.0 * passes / (ms * 1e-3) / 1e9;
}

}  // namespace dl
