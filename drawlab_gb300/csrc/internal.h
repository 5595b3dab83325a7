// Host-side internals of libdlgpu: context, scene, device buffers, errors.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/drawlab.h"
#include "layout.h"

namespace dl {

// Status-carrying exception used inside the library; converted to a status
// code and dl_last_error() message at the C ABI.
struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define DL_CUDA(call)                                                                      \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                             \
            throw ::dl::Error(DL_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Owning device allocation that only grows.
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    void ensure(size_t n) {
        if (n <= bytes) return;
        release();
        cudaError_t e = cudaMalloc(&ptr, n);
        if (e != cudaSuccess) {
            cudaGetLastError();
            ptr = nullptr;
            throw Error(e == cudaErrorMemoryAllocation ? DL_ERR_OOM : DL_ERR_CUDA,
                        std::string("cudaMalloc(") + std::to_string(n) + "): " + cudaGetErrorString(e));
        }
        bytes = n;
    }
    template <typename T>
    T* as() const { return static_cast<T*>(ptr); }
    template <typename T>
    void upload(const std::vector<T>& v, cudaStream_t s) {
        ensure(std::max<size_t>(v.size() * sizeof(T), 16));
        if (!v.empty()) {
            DL_CUDA(cudaMemcpyAsync(ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
        }
    }
};

// Pinned host staging buffer that only grows.
struct HostBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    ~HostBuf() {
        if (ptr) cudaFreeHost(ptr);
    }
    void ensure(size_t n) {
        if (n <= bytes) return;
        if (ptr) cudaFreeHost(ptr);
        ptr = nullptr;
        bytes = 0;
        DL_CUDA(cudaMallocHost(&ptr, n));
        bytes = n;
    }
    template <typename T>
    T* as() const { return static_cast<T*>(ptr); }
};

constexpr int kNumMaterialTypes = 5;

// Launch shape of the wavefront, chosen by dl_autotune (these defaults
// otherwise): path slots in flight, resident CTAs per SM of the traversal
// kernels and of the shading kernels, iterations per captured graph (even).
struct TuneParams {
    // 32M slots (6.9 GB of path state; a render uses at most one slot per
    // path): fewer, fuller wavefront iterations per frame
    int64_t paths_in_flight = (int64_t)1 << 25;
    int trav_ctas_per_sm = 8;
    int shade_ctas_per_sm = 16;
    int shade_threads = 128;   // threads per CTA of the miss and material kernels
    int iters_per_graph = 8;
};

// A queue length that kernels bump with atomics, alone in its 128-byte line:
// atomics on one line serialise in one L2 slice, so the hot counters are
// spread over separate lines (and so over slices).
struct alignas(128) QueueCount {
    int n;
};

// Device counters of one wavefront render (see render.cu).
struct RenderCounters {
    alignas(128) int ext[2];     // extension-ray queue lengths (ping-pong)
    alignas(128) int shadow[2];  // shadow-ray queue lengths
    QueueCount mat[2][kNumMaterialTypes + 1];  // material-sorted hit queues + miss queue (ping-pong)
    alignas(128) unsigned int work_ext;        // chunk cursors of the traversal kernels
    alignas(128) unsigned int work_sh;
    alignas(128) unsigned long long next_path;
    alignas(128) unsigned int guide_next;      // training records claimed (guided renders)
    // Values of the current pass, written by the host after the counters are
    // reset, so the captured graph stays valid across passes and frames.
    alignas(128) unsigned long long pass_total;  // paths of the pass
    int pass_spp_offset;                         // single render: sample index of the pass's first sample
    unsigned int pass_keep;                      // guided: training-record keep threshold (24-bit hash)
    void* pass_recs;                             // guided: where the pass writes its training records
    alignas(128) unsigned long long stat_ext;
    unsigned long long stat_shadow;
    unsigned long long stat_camera;   // filled on the host: paths started = min(next_path, paths)
    unsigned long long stat_invalid;
    unsigned long long stat_nodes_ext;
    unsigned long long stat_tris_ext;
    unsigned long long stat_nodes_sh;
    unsigned long long stat_tris_sh;
    unsigned int err;
    unsigned int pad2;
};

// Wavefront path-state buffers, sized for the pool and reused across renders.
struct RenderBuffers {
    int64_t capacity = 0;
    DevBuf rec, pos;   // 128-byte path record per slot (pos: Li mode)
    DevBuf ext_q[2], mat_q[kNumMaterialTypes + 1];
    DevBuf sh_o, sh_d, sh_c;
    DevBuf counters, invalid;
    DevBuf samples;   // per-path radiance of the current sample chunk (film gather input)
    DevBuf grec;      // guided renders: per-slot training-record links (32 B)
    DevBuf requests;  // batch: the pass's request table
    HostBuf host_requests;
    DevBuf batch_films;  // batch: films of requests without a caller film
    DevBuf film;      // internal film when the caller gives no device film
    DevBuf rgb;       // resolved image
    DevBuf li_xys, li_out, li_pos;
    HostBuf host_counters;
    HostBuf host_stage;
    HostBuf host_pass;   // staging of the pass values
    void ensure(int64_t cap);
    size_t device_bytes() const;
};

struct TraceBuffers {
    DevBuf rays, hits, occ;
    DevBuf wavefront;   // path slots, queues and counters of wavefront ray batches
    HostBuf stage;
};

}  // namespace dl

struct dl_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::string error;
    dl_stats stats{};
    dl::RenderBuffers render;
    dl::TraceBuffers trace;
    int num_sms = 0;
    dl::TuneParams tune;
    bool kernel_timing = false;
    std::vector<cudaEvent_t> timing_events;  // created on first timed render
    // CUDA graph of one batch of wavefront iterations, reused while the
    // kernel parameters stay byte-identical.
    cudaGraphExec_t graph_exec = nullptr;
    std::vector<unsigned char> graph_key;
    // Side streams and fork/join events: the miss kernel and the material
    // kernels of an iteration run as parallel graph branches.
    static constexpr int kAux = 5;
    cudaStream_t aux[kAux] = {nullptr};
    cudaEvent_t fork_ev = nullptr;
    cudaEvent_t join_ev[kAux] = {nullptr};
    ~dl_context() {
        for (cudaEvent_t e : timing_events) cudaEventDestroy(e);
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        for (int i = 0; i < kAux; i++) {
            if (aux[i]) cudaStreamDestroy(aux[i]);
            if (join_ev[i]) cudaEventDestroy(join_ev[i]);
        }
        if (fork_ev) cudaEventDestroy(fork_ev);
    }
};

// Learned guiding proposal: parameters (fp32 master, fp16 copy), Adam state
// and training buffers (guide.cu).
struct dl_guide {
    dl_context* ctx = nullptr;
    dl_guide_config cfg{};
    dl::DevBuf w32, w16, grad, m, v, scratch, recs, io_in, io_out;
    dl::DevBuf image;       // the weights as the tensor-core kernels load them (guide_tc.cuh)
    dl::DevBuf pass_recs;   // training records of guided render passes (two halves, alternating)
    dl::DevBuf partial;                    // a training batch's per-block gradient sums
    dl::DevBuf wsum;                       // per-block sums of L / p of a training batch
    int64_t step = 0;
    // training runs on its own stream, overlapping the next pass
    cudaStream_t train_stream = nullptr;
    cudaEvent_t pass_done[2] = {nullptr, nullptr}, train_done[2] = {nullptr, nullptr};
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    ~dl_guide() {
        for (int k = 0; k < 2; k++) {
            if (pass_done[k]) cudaEventDestroy(pass_done[k]);
            if (train_done[k]) cudaEventDestroy(train_done[k]);
        }
        if (t0) cudaEventDestroy(t0);
        if (t1) cudaEventDestroy(t1);
        if (train_stream) cudaStreamDestroy(train_stream);
    }
};

struct dl_scene {
    dl_context* ctx = nullptr;
    dl::DevScene dev{};
    dl::DevBuf nodes, tris, tri_vidx, normals, meshes, materials, lights, emit_tris, emit_cdf;
    dl::DevBuf env_tex, env_accel, light_pick;
    dl::DevBuf texels, textures, texcoords;   // bitmap textures, their table, per-vertex texcoords
    std::vector<int32_t> tri_order;   // leaf-order triangle -> original id
    dl_scene_info info{};
    dl_render_opts defaults{};
    float filter_radius[2] = {2.0f, 0.5f};
};
