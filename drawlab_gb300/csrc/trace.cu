// Ray-batch traversal kernels behind dl_trace_closest / dl_trace_any
// (the reference's Accel::rayIntersect, include/tracer/accel.h:52, over the
// OCTree of src/tracer/accel/octree.cpp:53-133).
#include <cuda_runtime.h>

#include "device.cuh"
#include "internal.h"

namespace dl {

// rays: n x 8 floats (ox, oy, oz, tmin, dx, dy, dz, tmax) as 2 float4.
// hits: n x float4 (t, u, v, original triangle id bits; -1 = miss).
template <bool kCount>
__global__ void __launch_bounds__(128) k_trace_closest(DevScene sc, const float4* __restrict__ rays, int64_t n,
                                                       float4* __restrict__ hits, unsigned int* err_out,
                                                       unsigned long long* counts) {
    uint32_t err = 0, nn = 0, nt = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float4 o = __ldg(rays + 2 * i), d = __ldg(rays + 2 * i + 1);
        float t = 0.f, u = 0.f, v = 0.f;
        int tri = trace_closest<kCount>(sc, xyz(o), xyz(d), o.w, d.w, t, u, v, err, nn, nt);
        int prim = tri >= 0 ? __float_as_int(__ldg(sc.tris + 3 * tri).w) : -1;
        hits[i] = make_float4(tri >= 0 ? t : 0.f, tri >= 0 ? u : 0.f, tri >= 0 ? v : 0.f, __int_as_float(prim));
    }
    if (err) atomicOr(err_out, err);
    if (kCount) {
        atomicAdd(counts, (unsigned long long)nn);
        atomicAdd(counts + 1, (unsigned long long)nt);
    }
}

template <bool kCount>
__global__ void __launch_bounds__(128) k_trace_any(DevScene sc, const float4* __restrict__ rays, int64_t n,
                                                   uint8_t* __restrict__ occ, unsigned int* err_out,
                                                   unsigned long long* counts) {
    uint32_t err = 0, nn = 0, nt = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float4 o = __ldg(rays + 2 * i), d = __ldg(rays + 2 * i + 1);
        occ[i] = trace_any<kCount>(sc, xyz(o), xyz(d), o.w, d.w, err, nn, nt) ? 1 : 0;
    }
    if (err) atomicOr(err_out, err);
    if (kCount) {
        atomicAdd(counts, (unsigned long long)nn);
        atomicAdd(counts + 1, (unsigned long long)nt);
    }
}

static int trace_grid(int sms, int64_t n) {
    int64_t want = (n + 127) / 128;
    int64_t cap = (int64_t)sms * 64;
    return (int)std::max<int64_t>(1, std::min(want, cap));
}

// Launch on the context stream; `scratch` holds the error word and the two
// traversal counters (24 bytes, zeroed here).
void trace_closest_launch(dl_scene* S, const float* d_rays, int64_t n, float* d_hits, void* scratch, bool count) {
    cudaStream_t st = S->ctx->stream;
    DL_CUDA(cudaMemsetAsync(scratch, 0, 24, st));
    unsigned int* err = static_cast<unsigned int*>(scratch);
    unsigned long long* counts = reinterpret_cast<unsigned long long*>(static_cast<char*>(scratch) + 8);
    int g = trace_grid(S->ctx->num_sms, n);
    if (n == 0) return;
    if (count)
        k_trace_closest<true><<<g, 128, 0, st>>>(S->dev, reinterpret_cast<const float4*>(d_rays), n,
                                                 reinterpret_cast<float4*>(d_hits), err, counts);
    else
        k_trace_closest<false><<<g, 128, 0, st>>>(S->dev, reinterpret_cast<const float4*>(d_rays), n,
                                                  reinterpret_cast<float4*>(d_hits), err, counts);
    DL_CUDA(cudaGetLastError());
}

void trace_any_launch(dl_scene* S, const float* d_rays, int64_t n, uint8_t* d_occ, void* scratch, bool count) {
    cudaStream_t st = S->ctx->stream;
    DL_CUDA(cudaMemsetAsync(scratch, 0, 24, st));
    unsigned int* err = static_cast<unsigned int*>(scratch);
    unsigned long long* counts = reinterpret_cast<unsigned long long*>(static_cast<char*>(scratch) + 8);
    int g = trace_grid(S->ctx->num_sms, n);
    if (n == 0) return;
    if (count)
        k_trace_any<true><<<g, 128, 0, st>>>(S->dev, reinterpret_cast<const float4*>(d_rays), n, d_occ, err, counts);
    else
        k_trace_any<false><<<g, 128, 0, st>>>(S->dev, reinterpret_cast<const float4*>(d_rays), n, d_occ, err, counts);
    DL_CUDA(cudaGetLastError());
}

}  // namespace dl
