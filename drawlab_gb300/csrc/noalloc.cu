// dl_li_static: per-path radiance with no allocation at call time.
//
// Who needs it: callers that must not allocate device memory while they
// render -- an engine that hands all device memory to its own pool at
// start-up and forbids allocation afterwards, a real-time loop with a fixed
// memory budget, or a host thread that may not block on the driver's
// allocator.  dl_li grows its path pool on demand; this entry point instead
// runs the same wavefront kernels out of one fixed, file-scope device array.
// It is a synchronous call: it returns after the paths have finished.
//
// Limits and sharing:
//  * the array holds kStaticPathSlots = 16384 path slots (240 bytes each,
//    3.75 MiB in all) and lives on every GPU that loads the library until the
//    process exits;
//  * requests with max_paths_in_flight above 16384 are rejected with
//    DL_ERR_INVALID_ARG (0 means "use the whole pool"); the number of paths n
//    itself is not limited, slots are reused as paths finish;
//  * every call uses the same array and leaves its contents behind; the
//    counters that must start at zero are cleared at the start of each call;
//  * two calls whose work overlaps on the GPU (different streams or
//    contexts on one device) race on the array and corrupt each other, so
//    calls from all contexts on one device must be serialised by the caller.
#include <cuda_runtime.h>

#include <exception>
#include <mutex>
#include <string>

#include "internal.h"
#include "scene.h"

namespace dl {

size_t fixed_pool_bytes(int64_t slots);
void render_li_fixed(dl_scene* S, const dl_render_opts& o, void* pool, int64_t slots, int64_t li_n,
                     const int* d_xys, float* d_L, float* d_pos);

constexpr int64_t kStaticPathSlots = 16384;
constexpr size_t kStaticPoolBytes = 240 * (size_t)kStaticPathSlots + 256;

// The pool.  Host code must not use this name as an address: it is a host
// stand-in for the device symbol.  Its device address comes from
// cudaGetSymbolAddress, per device, below.
static __device__ __align__(256) unsigned char g_static_pool[kStaticPoolBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void* g_pool_addr[kMaxDevices] = {nullptr};

// Once per device, with that device current: resolve the pool's device
// address.  The first dl_li_static call on a device does this, so that
// first call belongs before any stream capture.
cudaError_t pool_address(int device, void** out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_pool_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_pool);
        if (e != cudaSuccess) return e;
        g_pool_addr[device] = p;
    }
    *out = g_pool_addr[device];
    return cudaSuccess;
}
}  // namespace

}  // namespace dl

extern "C" int dl_li_static(dl_scene* scene, const dl_render_opts* opts, int64_t n, const int32_t* d_xys,
                            float* d_L, float* d_pos) {
    static_assert(dl::kStaticPoolBytes >= 256, "pool size");
    if (!scene) return DL_ERR_INVALID_ARG;
    dl_context* ctx = scene->ctx;
    ctx->error.clear();
    if (!opts || n < 0 || n >= ((int64_t)1 << 31) || (n > 0 && (!d_xys || !d_L || !d_pos))) {
        ctx->error = "dl_li_static: bad arguments";
        return DL_ERR_INVALID_ARG;
    }
    if (opts->max_paths_in_flight < 0 || opts->max_paths_in_flight > dl::kStaticPathSlots) {
        ctx->error = "dl_li_static: max_paths_in_flight exceeds the static pool of 16384 paths";
        return DL_ERR_INVALID_ARG;
    }
    if (opts->rr_depth < 0 || (opts->flags & ~(uint32_t)(DL_RENDER_FIX_POINT_LIGHT | DL_RENDER_POWER_LIGHT_PICK)) ||
        (opts->filter != DL_FILTER_GAUSSIAN && opts->filter != DL_FILTER_BOX)) {
        ctx->error = "dl_li_static: unsupported render options";
        return DL_ERR_INVALID_ARG;
    }
    if (n == 0) return DL_OK;
    if (dl::fixed_pool_bytes(dl::kStaticPathSlots) > dl::kStaticPoolBytes) return DL_ERR_INVALID_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    void* pool = nullptr;
    if (e == cudaSuccess) e = dl::pool_address(ctx->device, &pool);
    if (e != cudaSuccess) {
        ctx->error = std::string("dl_li_static: static pool address: ") + cudaGetErrorString(e);
        return DL_ERR_CUDA;
    }
    int64_t slots = opts->max_paths_in_flight > 0 ? opts->max_paths_in_flight : dl::kStaticPathSlots;
    slots = (slots / 32) * 32;
    if (slots < 32) slots = 32;
    try {
        dl::render_li_fixed(scene, *opts, pool, slots, n, d_xys, d_L, d_pos);
    } catch (const dl::Error& err) {
        ctx->error = err.what();
        return err.status;
    } catch (const std::exception& err) {
        ctx->error = err.what();
        return DL_ERR_CUDA;
    }
    return DL_OK;
}
